"""Seeded synthetic circuits of the benchmark workloads.

All draws use ``numpy.random.default_rng(seed)``.

* `power_grid(n)`: n x n resistive mesh; segment conductance
  ``exp(N(0, 0.3))`` S (median 1 S), a sink ``U(0, 1 mA)`` at every node,
  1.0 V pads at the 4 corners and at every 25th node of a clockwise walk of
  the border starting at the top-left corner (100 x 100: 19 pads, 10,019
  unknowns). Structure follows voltax/benchmarks/benchmark_power_grid.py:30-66.
* `power_grid_batch(sides)`: an uneven batch of such grids as one circuit
  of independent segments (`Circuit.with_segments`).
* `ring_oscillator(stages)`: CMOS ring of EKV inverters (NMOS w=1u, PMOS
  w=2u, l=0.13u), VDD 1.2 V, 5 fF per stage; `ring_initial_state` gives the
  alternating rail pattern with a 0.1 V kick on node 0.
* `ring_oscillator_level1(stages)`: the reference's own ring benchmark
  circuit (exact Level-1 devices) with its alternating initial state.
* `mirror_adder_mc(instances)`: 4-bit ripple-carry adder of 28-transistor
  mirror full adders, per-device ``dvth ~ N(0, 30 mV)`` and
  ``log W += N(0, 0.05)``; A and B step 0000 -> 1111 with 20 ps edges.
"""

from __future__ import annotations

import functools
import itertools

import numpy as np
import torch

from .builder import CircuitBuilder
from .elements import Level1MOSFET, MOSProcess
from .library import cmos
from .signals import Step

VDD = 1.2


def grid_pads(n: int, every: int = 25) -> list[tuple[int, int]]:
    """Pad sites: corners plus every `every`-th node of the border walk."""
    walk = ([(0, j) for j in range(n)] + [(i, n - 1) for i in range(1, n)]
            + [(n - 1, j) for j in range(n - 2, -1, -1)]
            + [(i, 0) for i in range(n - 2, 0, -1)])
    sites = {walk[p] for p in range(0, len(walk), every)}
    sites |= {(0, 0), (0, n - 1), (n - 1, 0), (n - 1, n - 1)}
    return sorted(sites)


def _grid_arrays(n: int, rng, sigma: float, sink_max: float):
    """One grid in the order a per-device `CircuitBuilder` walk visits it:
    segments (i, j)-(i, j+1) then (i, j)-(i+1, j) for i, j row-major, a sink
    at every node, then the pads. Returns the nodes as row-major ids in
    first-seen order, the segment ends and pads as indices into that order,
    and the conductances and sinks."""
    ids = np.arange(n * n).reshape(n, n)
    right = np.stack([ids[:, :-1], ids[:, 1:]], -1)                # (n, n-1, 2)
    down = np.stack([ids[:-1, :], ids[1:, :]], -1)                 # (n-1, n, 2)
    ends = np.full((n, n, 2, 2), -1, np.int64)  # per site: [right, down] x (a, c)
    ends[:, :-1, 0] = right
    ends[:-1, :, 1] = down
    ends = ends.reshape(-1, 2)
    ends = ends[ends[:, 0] >= 0]
    pads = np.array([i * n + j for i, j in grid_pads(n)], np.int64)
    walk = np.concatenate([ends.ravel(), ids.ravel(), pads])
    first = np.unique(walk, return_index=True)[1]
    order = np.argsort(first, kind="stable")          # row-major ids, first seen first
    rank = np.empty(n * n, np.int64)
    rank[order] = np.arange(n * n)
    g = np.exp(rng.normal(0.0, sigma, len(ends)))
    sinks = rng.uniform(0.0, sink_max, n * n)
    return order, rank[ends], rank[ids.ravel()], rank[pads], g, sinks


class _Names:
    """Name strings shared by the grids of one batch (freed with it): the
    ``n{i}_{j}`` site names of each side, and ``R0, R1, ...`` style counters."""

    def __init__(self):
        self._sites: dict[int, tuple[str, ...]] = {}
        self._numbered: dict[str, list[str]] = {}

    def sites(self, n: int) -> tuple[str, ...]:
        got = self._sites.get(n)
        if got is None:
            got = self._sites[n] = tuple(f"n{q // n}_{q % n}" for q in range(n * n))
        return got

    def numbered(self, letter: str, count: int) -> list[str]:
        have = self._numbered.setdefault(letter, [])
        if len(have) < count:
            have.extend(f"{letter}{q}" for q in range(len(have), count))
        return have[:count]


def _grids(sides, seeds, sigma: float, sink_max: float, vpad: float, prefixes):
    """Grids as one circuit, built from arrays: the node numbering, device
    names, groups and parameters of adding every segment, sink and pad to a
    `CircuitBuilder` one by one (grid by grid), without the per-device
    objects."""
    from .circuit import Circuit
    from .elements import CurrentSource, Resistor, VoltageSource

    names, seg = [], []
    r_nodes, i_nodes, v_nodes = [], [], []
    r_val, i_val = [], []
    r_names, i_names, v_names = [], [], []
    off = 0
    known = _Names()
    for k, (n, seed, pre) in enumerate(zip(sides, seeds, prefixes)):
        n = int(n)
        order, ends, sink_at, pad_at, g, sinks = _grid_arrays(
            n, np.random.default_rng(seed), sigma, sink_max)
        site = known.sites(n)
        names += map(pre.__add__, (site[q] for q in order.tolist()))
        seg += [k] * len(order)
        r_nodes.append(ends + off)
        r_val.append(1.0 / g)
        i_nodes.append(sink_at + off)
        i_val.append(sinks)
        v_nodes.append(pad_at + off)
        r_names += map(pre.__add__, known.numbered("R", len(ends)))
        i_names += map(pre.__add__, known.numbered("I", len(sinks)))
        v_names += map(pre.__add__, known.numbered("Vpad", len(pad_at)))
        off += len(order)
    cat = np.concatenate
    gnd = lambda a: np.stack([a, np.full_like(a, -1)], 1)  # noqa: E731
    tables = {"Resistor": cat(r_nodes), "CurrentSource": gnd(cat(i_nodes)),
              "VoltageSource": gnd(cat(v_nodes))}
    groups, devices = {}, []
    rows = lambda t: tuple(zip(*t.T.tolist()))  # noqa: E731  (node tuples, made by zip)
    for gname, make, members in (
            ("Resistor", lambda t: Resistor(rows(t), cat(r_val)), r_names),
            ("CurrentSource", lambda t: CurrentSource(rows(t), cat(i_val)), i_names),
            ("VoltageSource", lambda t: VoltageSource(rows(t), np.full(len(t), float(vpad))),
             v_names)):
        if members:
            table = tables[gname]
            el = make(table)
            table.setflags(write=False)
            el.__dict__["_node_table"] = (el.nodes, table)  # the array node_array() returns
            groups[gname] = el
            # the (device, group, index) triples a builder's name map lays out
            devices.append(tuple(zip(members, itertools.repeat(gname), range(len(members)))))
    return Circuit(groups, tuple(names), tuple(itertools.chain.from_iterable(devices))), seg


def power_grid(n: int = 100, seed: int = 0, sigma: float = 0.3,
               sink_max: float = 1e-3, vpad: float = 1.0):
    return _grids([n], [seed], sigma, sink_max, vpad, [""])[0]


def power_grid_batch(sides, seed: int = 0, sigma: float = 0.3, sink_max: float = 1e-3,
                     vpad: float = 1.0):
    """An uneven batch of grids as one circuit of independent segments:
    grid k (nodes ``g{k}_n{i}_{j}``) is `power_grid` ``(sides[k],
    seed + k)``, and segment k is its nodes and pad currents."""
    sides = [int(n) for n in sides]
    c, seg = _grids(sides, [seed + k for k in range(len(sides))], sigma, sink_max, vpad,
                    [f"g{k}_" for k in range(len(sides))])
    return c.with_segments(seg)


def grid_sides(count: int, lo: int, hi: int, seed: int = 0) -> list[int]:
    """Mesh sides drawn uniformly from {lo, ..., hi}."""
    return [int(x) for x in np.random.default_rng(seed).integers(lo, hi + 1, count)]


def ring_oscillator(stages: int = 101, cload: float = 5e-15):
    b = CircuitBuilder()
    b.vsource("vdd", "0", VDD, name="Vdd")
    nodes = [f"n{k}" for k in range(stages)]
    cmos.ring_oscillator(b, nodes, "vdd", wn=1e-6, wp=2e-6)
    for nd in nodes:
        b.capacitor(nd, "0", cload)
    return b.build(), nodes


def ring_initial_state(circuit, nodes, kick: float = 0.1) -> torch.Tensor:
    """Alternating rails (node k at VDD for odd k) with node 0 at `kick`."""
    v = {"vdd": VDD, **{nd: VDD * (k % 2) for k, nd in enumerate(nodes)}}
    v[nodes[0]] = kick
    return circuit.state(v=v)


def ring_oscillator_level1(stages: int = 101, smooth: float = 0.0, gamma: float = 0.0,
                           cload: float = 5e-15):
    """The ring of voltax/benchmarks/benchmark_ring_oscillator.py:52-64:
    exact Level-1 inverters (``smooth=0``; NMOS kp 400 uA/V^2, PMOS
    200 uA/V^2, vth 0.4 V, lam 0.04/V, overlap 0.3 nF/m; W 0.4 / 0.8 um,
    L 0.13 um), 5 fF per stage, VDD 1.2 V; nodes ``n1 .. n<stages>``."""
    extra = dict(vth=0.4, lam=0.04, cov=0.3e-9, gamma=gamma)
    b = CircuitBuilder(nmos=MOSProcess.nmos(kp=400e-6, **extra),
                       pmos=MOSProcess.pmos(kp=200e-6, **extra),
                       mos_model=functools.partial(Level1MOSFET, smooth=smooth))
    b.vsource("vdd", "0", VDD, name="Vdd")
    nodes = [f"n{k}" for k in range(1, stages + 1)]
    cmos.ring_oscillator(b, nodes, "vdd", wn=0.4e-6, wp=0.8e-6)
    for nd in nodes:
        b.capacitor(nd, "0", cload)
    return b.build(), nodes


def ring_level1_initial_state(circuit, nodes) -> torch.Tensor:
    """Alternating 0.9 / 0.1 VDD (voltax/benchmarks/benchmark_ring_oscillator.py:44-49)."""
    v = {"vdd": VDD, **{nd: (0.9 if k % 2 == 0 else 0.1) * VDD for k, nd in enumerate(nodes)}}
    return circuit.state(v=v)


def mirror_adder(bits: int = 4, edge: float = 20e-12, delay: float = 50e-12,
                 cload: float = 1e-15):
    """One nominal adder; inputs A, B step 0 -> VDD at `delay`, cin = 0."""
    b = CircuitBuilder()
    b.vsource("vdd", "0", VDD, name="Vdd")
    a = [f"a{i}" for i in range(bits)]
    c = [f"b{i}" for i in range(bits)]
    for nd in a + c:
        b.vsource(nd, "0", Step(0.0, VDD, delay, edge), name=f"V{nd}")
    s = [f"s{i}" for i in range(bits)]
    cmos.mirror_ripple_adder(b, a, c, "0", s, "co", "vdd")
    for nd in s + ["co"]:
        b.capacitor(nd, "0", cload)
    return b.build()


def mirror_adder_mc(instances: int = 4096, seed: int = 0, bits: int = 4,
                    sigma_vth: float = 0.03, sigma_logw: float = 0.05):
    """`mirror_adder` with a leading instance axis on the MOSFET parameters."""
    c = mirror_adder(bits)
    rng = np.random.default_rng(seed)
    for name in sorted(c.elements):
        el = c.elements[name]
        if not hasattr(el, "dvth"):
            continue
        n = el.size
        new = el.with_nodes(el.nodes)
        new.dvth = torch.as_tensor(rng.normal(0.0, sigma_vth, (instances, n)))
        new.log_w = el.log_w + torch.as_tensor(rng.normal(0.0, sigma_logw,
                                                          (instances, n)))
        new.log_l = el.log_l.expand(instances, n).clone()
        c = c.replace(name, new)
    return c


# ----------------------------------------------------------------- OTA chain
OTA_GROUPS = 21
"""OTAs of the chain share their parameter shifts by position modulo this."""


def ota_chain(stages: int = 66, vbias: float = 0.6, vin: float = 0.6):
    """A chain of 5-transistor OTAs, each wired as a unity-gain follower of the
    previous output (the 5T OTA of voltax/benchmarks/benchmark_ota.py:51-68,
    with EKV devices): per stage the nodes d1 (mirror), out and tail, plus
    the shared vdd, bias and input -> 3 * stages + 3 nodes (66 stages: 201).

    Parameters enter through `ota_params`; the nominal circuit has VDD 1.2 V.
    """
    b = CircuitBuilder()
    b.vsource("vdd", "0", VDD, name="Vdd")
    b.vsource("bias", "0", vbias, name="Vbias")
    b.vsource("in", "0", vin, name="Vin")
    prev = "in"
    for k in range(stages):
        d1, out, tail = f"d1_{k}", f"out{k}", f"tail{k}"
        b.nmos(d1, prev, tail, "0", w=2e-6, name=f"M1_{k}")
        b.nmos(out, out, tail, "0", w=2e-6, name=f"M2_{k}")
        b.pmos(d1, d1, "vdd", "vdd", w=4e-6, name=f"M3_{k}")
        b.pmos(out, d1, "vdd", "vdd", w=4e-6, name=f"M4_{k}")
        b.nmos(tail, "bias", "0", "0", w=2e-6, name=f"M5_{k}")
        prev = out
    return b.build()


def ota_params(n: int, seed: int = 0) -> np.ndarray:
    """``(n, 64)`` parameter vectors: VDD ~ U(0.9, 1.3) V, then per position
    group g < 21: the input-pair Vth shift ~ N(0, 30 mV), the mirror log-W
    shift ~ N(0, 0.05) and the tail Vth shift ~ N(0, 30 mV)."""
    rng = np.random.default_rng(seed)
    p = np.empty((n, 1 + 3 * OTA_GROUPS))
    p[:, 0] = rng.uniform(0.9, 1.3, n)
    shifts = rng.normal(0.0, 1.0, (n, OTA_GROUPS, 3)) * np.array([0.03, 0.05, 0.03])
    p[:, 1:] = shifts.reshape(n, -1)
    return p


def apply_ota_params(circuit, params: np.ndarray):
    """Batched copy of `ota_chain` with the parameter vectors applied."""
    params = torch.as_tensor(params, dtype=torch.float64)
    B = params.shape[0]
    c = circuit
    vdd = c.elements["VoltageSource"]
    idx = c.layout.device("Vdd")[1]
    val = vdd.value.value.expand(B, vdd.size).clone()
    val[:, idx] = params[:, 0]
    c = c.replace("VoltageSource", vdd.with_dc(val))
    shifts = params[:, 1:].reshape(B, OTA_GROUPS, 3)
    for gname in ("EKVMOSFET_n", "EKVMOSFET_p"):
        el = c.elements[gname]
        names = c.devices(gname)
        dv = torch.zeros(B, el.size, dtype=torch.float64)
        lw = el.log_w.expand(B, el.size).clone()
        for i, name in enumerate(names):
            role, k = name.split("_")
            grp = int(k) % OTA_GROUPS
            if role in ("M1", "M2"):
                dv[:, i] = shifts[:, grp, 0]
            elif role == "M5":
                dv[:, i] = shifts[:, grp, 2]
            else:  # M3, M4: the mirror
                lw[:, i] = lw[:, i] + shifts[:, grp, 1]
        new = el.with_nodes(el.nodes)
        new.dvth = dv
        new.log_w = lw
        new.log_l = el.log_l.expand(B, el.size).clone()
        c = c.replace(gname, new)
    return c
