"""Benchmark: batched Newton solves/s on the Monte Carlo mirror-adder workload.

Workload (one "step"): 4096 instances of a 4-bit ripple-carry adder of
28-transistor mirror full adders (EKV MOSFETs, per-device Vth and log W
mismatch), A and B stepping 0000 -> 1111 with 20 ps edges; a DC operating
point and a 501-point backward-Euler transient over 1 ns, i.e. 4096 x 501
Newton solves (stamp + refactor + solve until converged) per step. Inputs
are synthetic (seeded), parameters resident in HBM before the timed region
for ``value``; ``e2e`` goes through the public API from pinned host buffers.

``value`` is the chosen form (FP32 supernodal factors + FP64 refinement);
``plain_fp64`` is the same workload with FP64 factors, and ``match`` is the
largest node-voltage difference between the two (relative to 1 V).

``--impl reference`` times the compiled CPU restatement of the reference
algorithm (oracle/cvx.c) on all host cores (one thread per core, whole
instances per step); ``cpu_baseline`` is the same code on one thread.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Newton solves/sec batched (stamp+LU+solve) vs plain FP64 GPU at 1e-9 match"
UNIT = "solves/s"
INSTANCES = 4096
T_STOP, N_T = 1e-9, 501


class Workload:
    """One benchmark configuration: how to build it and what one solve is."""

    def __init__(self, name, analysis, method, t_stop, n_t, outputs, default_instances):
        self.name, self.analysis, self.method = name, analysis, method
        self.t_stop, self.n_t, self.outputs = t_stop, n_t, outputs
        self.default_instances = default_instances

    def circuit(self, instances, seed=0):
        from voltax_gb300 import workloads as wl
        if self.name == "adder_mc":
            return wl.mirror_adder_mc(instances, seed=seed)
        if self.name == "ring101":
            return wl.ring_oscillator(101)[0]
        if self.name == "ring101_l1":
            return wl.ring_oscillator_level1(101)[0]
        if self.name == "grid100":
            return wl.power_grid(100, seed=seed)
        if self.name == "ota_warm":
            return wl.apply_ota_params(wl.ota_chain(OTA_STAGES),
                                       wl.ota_params(instances, seed=OTA_TEST_SEED + seed))
        if self.name == "grids":
            return wl.power_grid_batch(wl.grid_sides(instances, *GRID_SIDES, seed=seed),
                                       seed=seed)
        raise ValueError(self.name)

    def cpu_circuit(self, instances, seed=0):
        """The circuit a CPU leg times: for the grid batch at most its first
        CPU_GRIDS grids (grid k of a batch is the same circuit at any batch
        size), so that the leg stays a bounded sample; else the workload."""
        if self.name != "grids" or instances <= CPU_GRIDS:
            return self.circuit(instances, seed)
        from voltax_gb300 import workloads as wl
        sides = wl.grid_sides(instances, *GRID_SIDES, seed=seed)[:CPU_GRIDS]
        return wl.power_grid_batch(sides, seed=seed)

    def ic(self, circuit):
        """Initial condition: "dc" or a state vector."""
        if self.name == "ring101":
            from voltax_gb300 import workloads as wl
            return wl.ring_initial_state(circuit, [f"n{k}" for k in range(101)])
        if self.name == "ring101_l1":
            from voltax_gb300 import workloads as wl
            return wl.ring_level1_initial_state(circuit, [f"n{k}" for k in range(1, 102)])
        return "dc"

    def times(self, n_t=None):
        n = self.n_t if n_t is None else n_t
        return np.linspace(0.0, self.t_stop, n) if self.analysis == "transient" else \
            np.zeros(1)

    def label(self, instances, n_t):
        if self.name == "adder_mc":
            return f"mirror_adder_mc{instances}"
        if self.name == "ring101":
            return f"ring_oscillator101_trap{n_t}"
        if self.name == "ring101_l1":
            return f"ring_oscillator101_level1_be{n_t}"
        if self.name == "ota_warm":
            return f"ota_chain{OTA_STAGES}_dc_warm_start{instances}"
        if self.name == "grids":
            return f"power_grid_batch{instances}_sides{GRID_SIDES[0]}-{GRID_SIDES[1]}_dc_adjoint"
        return "power_grid100_dc"


WORKLOADS = {
    "adder_mc": Workload("adder_mc", "transient", "be", T_STOP, N_T,
                         ["s0", "s1", "s2", "s3", "co"], INSTANCES),
    "ring101": Workload("ring101", "transient", "trap", 2e-9, 2001, ["n0", "n50", "n100"], 1),
    "grid100": Workload("grid100", "dc", None, 0.0, 1, None, 1),
    # voltax's own ring benchmark (benchmarks/benchmark_sparse.py:143-176): exact
    # Level 1, backward Euler, 3445 steps over 0.3 ns (uniform here; the
    # reference steps on ngspice's accepted points)
    "ring101_l1": Workload("ring101_l1", "transient", "be", 0.3e-9, 3446,
                           ["n1", "n51", "n101"], 1),
    "ota_warm": Workload("ota_warm", "dc", None, 0.0, 1, None, 10000),
    "grids": Workload("grids", "dc", None, 0.0, 1, None, 32),
}
# uneven batch: `instances` grids of side U{50..120} in one segmented circuit
GRID_SIDES = (50, 120)
CPU_GRIDS = 32  # grids in the CPU legs' sample of a larger batch
# learned warm start: 66-stage OTA chain (201 nodes), 200k training
# operating points (parameter seed 1), 10k held-out instances (seed 2)
OTA_STAGES, OTA_TRAIN, OTA_TRAIN_SEED, OTA_TEST_SEED = 66, 200_000, 1, 2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="adder_mc", choices=sorted(WORKLOADS))
    ap.add_argument("--instances", type=int, default=None)
    ap.add_argument("--time-points", type=int, default=None)
    ap.add_argument("--engine", default="auto", choices=["auto", "generic", "fused"])
    ap.add_argument("--block", type=int, default=0, choices=[0, 32, 64, 128, 256, 512],
                    help="fused kernel threads per instance (32: one warp per instance; "
                         "0: the library's or the autotuner's choice)")
    ap.add_argument("--refine", type=int, default=None,
                    help="FP64 refinement sweeps per solve of the FP32-factor form "
                         "(default: the library's choice per engine)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extra", action="store_true",
                    help="adder_mc: skip the bounded runs of the other configurations")
    ap.add_argument("--train", type=int, default=None, help="ota_warm: training instances")
    ap.add_argument("--epochs", type=int, default=40, help="ota_warm: training epochs")
    ap.add_argument("--grid-sides", type=int, nargs=2, default=None, metavar=("LO", "HI"),
                    help="grids: mesh sides drawn from U{LO..HI} (default 50 120; the "
                         "full uneven-grid configuration is --instances 512 --grid-sides 50 300)")
    a = ap.parse_args()
    if a.grid_sides is not None:
        global GRID_SIDES
        lo, hi = a.grid_sides
        if not 2 <= lo <= hi:
            ap.error("--grid-sides needs 2 <= LO <= HI")
        GRID_SIDES = (lo, hi)
    w = WORKLOADS[a.workload]
    if a.instances is None:
        a.instances = w.default_instances
    if a.time_points is None:
        a.time_points = w.n_t
    return a


# ----------------------------------------------------------------- clocks
class Clocks:
    """nvidia-smi samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 5 + i and r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


# ----------------------------------------------------------------- CPU legs
def _cpu_systems(w, instances, count, seed=0):
    """Compiled-oracle systems for the CPU legs. Their plan comes from the
    oracle's numpy planner, so the CPU legs load no library of the product
    (only oracle/_build/libcvx.so)."""
    from oracle import cbase
    from oracle import plan as oplan
    from voltax_gb300 import symbolic
    c = w.cpu_circuit(instances, seed=seed)
    st = symbolic.structure(c)
    plan = oplan.make_plan_numpy(st)
    ic = w.ic(c)
    z0 = None if isinstance(ic, str) else ic.numpy()
    return [cbase.CSystem(c, st, plan, b % c.batch) for b in range(count)], z0


def _cpu_run(w, sysm, z0, ts):
    if w.analysis == "dc":
        return sysm.run(ts[:1], dc_first=True)
    return sysm.run(ts, z0=z0, method=w.method, dc_first=z0 is None)


def cpu_superlu(w, instances, min_seconds=5.0):
    """A conventional CPU sparse baseline for the DC workloads: SuperLU
    (scipy.sparse.linalg.splu) factor + solve of the Newton matrix at the
    zero state, one thread, repeated for `min_seconds` (a DC solve of these
    linear circuits is one such factor + solve plus a convergence check)."""
    if w.analysis != "dc" or w.name == "ota_warm":
        return None
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    from oracle import stamp as ost
    from voltax_gb300 import symbolic
    try:
        from threadpoolctl import threadpool_limits
    except ImportError:  # not installed on every box; SuperLU itself is serial
        threadpool_limits = None
    c = w.cpu_circuit(instances, seed=0)
    st = symbolic.structure(c)
    z = np.zeros(c.size)
    A = sp.csr_matrix((ost.jacobian(c, st, z, 0.0, 1.0, 0.0), st.indices, st.indptr),
                      shape=(c.size, c.size)).tocsc()
    rhs = -ost.f(c, z, 0.0)
    per = min(instances, CPU_GRIDS) if w.name == "grids" else 1
    ctx = threadpool_limits(1) if threadpool_limits else None
    try:
        if ctx:
            ctx.__enter__()
        spla.splu(A).solve(rhs)
        n, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < min_seconds:
            spla.splu(A).solve(rhs)
            n += 1
        secs = time.perf_counter() - t0
    finally:
        if ctx:
            ctx.__exit__(None, None, None)
    return {"value": n * per / secs, "unit": UNIT, "cores": 1, "kind": "superlu",
            "sample": f"{n} SuperLU factor + solve of the {c.size}-unknown Newton matrix, "
                      f"{secs:.1f} s (scipy.sparse.linalg.splu)"}


def cpu_baseline(w, n_t, instances, min_seconds=10.0):
    """The compiled CPU restatement (oracle/cvx.c), one thread, whole
    instances until `min_seconds` have passed."""
    # the grid batch is one circuit holding `instances` grids (segments)
    per_run = min(instances, CPU_GRIDS) if w.name == "grids" else 1
    systems, z0 = _cpu_systems(w, instances, 1 if per_run > 1 else min(instances, 64))
    ts = w.times(n_t)
    _cpu_run(w, systems[0], z0, ts[:3])
    solves, t0, i = 0, time.perf_counter(), 0
    while time.perf_counter() - t0 < min_seconds and i < 10000:
        _cpu_run(w, systems[i % len(systems)], z0, ts)
        solves += len(ts) * per_run
        i += 1
    secs = time.perf_counter() - t0
    what = "DC solve" if w.analysis == "dc" else f"DC + {len(ts) - 1} {w.method.upper()} steps"
    if per_run > 1:
        what = (f"DC solve of all {per_run} grids" if per_run == instances else
                f"DC solve of the first {per_run} of the {instances} grids")
    return {"value": solves / secs, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{i} whole instances ({what} each) on 1 thread, {secs:.1f} s; "
                      "compiled C restatement oracle/cvx.c"}


def run_reference(a):
    from concurrent.futures import ThreadPoolExecutor
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    w = WORKLOADS[a.workload]
    cores = os.cpu_count() or 1
    per_thread = 4 if w.analysis == "transient" and w.name == "adder_mc" else 1
    if w.name == "grid100":
        per_thread = 8
    if w.name == "grids":
        cores = min(cores, 2)  # each system is the whole batch
    ts = w.times(a.time_points)
    systems, z0 = _cpu_systems(w, a.instances, cores * per_thread)
    # a grid-batch system solves each of its grids (one Newton solve per grid)
    per_system = min(a.instances, CPU_GRIDS) if w.name == "grids" else 1

    def work(i):  # ctypes releases the GIL inside cvx_run
        for j in range(per_thread):
            _cpu_run(w, systems[i * per_thread + j], z0, ts)
        return per_thread * len(ts) * per_system

    with ThreadPoolExecutor(cores) as ex:
        for _ in range(a.warmup):
            list(ex.map(work, range(cores)))
        times, solves = [], 0
        for _ in range(a.steps):
            t0 = time.perf_counter()
            solves += sum(ex.map(work, range(cores)))
            times.append(time.perf_counter() - t0)
    total = sum(times)
    value = solves / total
    sample = (f"{cores} threads x {per_thread} whole instances "
              f"({len(ts) * per_system} solves each) per step; compiled C restatement "
              "oracle/cvx.c")
    if w.name == "grids" and per_system < a.instances:
        sample += f"; each instance is the first {per_system} of the {a.instances} grids"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * total / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w.label(a.instances, len(ts)), "instances": a.instances,
                       "time_points": len(ts), "method": w.method or "dc",
                       "t_stop_s": w.t_stop, "solves_per_step": a.instances * len(ts),
                       "sample": sample},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def to_device(c, device, pin=False):
    """The circuit with every parameter tensor on `device` (or pinned host)."""
    out = c
    for name in sorted(c.elements):
        el = c.elements[name]
        new = el.with_nodes(el.nodes)
        for f in el.fields:
            t = getattr(el, f)
            setattr(new, f, t.pin_memory() if pin else t.to(device))
        if hasattr(el, "value"):
            new.value = el.value.map(lambda t: t.pin_memory() if pin else t.to(device))
        if hasattr(el, "process"):
            new.process = el.process
        out = out.replace(name, new)
    return out


def h2d_bytes(c):
    return sum(t.numel() * 8 for el in c.elements.values()
               for t in ([getattr(el, f) for f in el.fields] +
                         (el.value.params() if hasattr(el, "value") else [])))


def oracle_check(w, circuit, z, ts, ic, count=16):
    """Acceptance of the GPU's chosen-form results on a sample of instances
    against the compiled FP64 oracle (oracle/cvx.c): the oracle solves each
    sampled instance itself (largest node-voltage difference, relative with a
    1 mV floor), and evaluates the FP64 residual r(z*) at the GPU's solution
    (largest KCL residual) and one more Newton step from it (largest
    |dz| / (atol + rtol |z*|); <= 1 passes voltax's convergence test).
    `z`: (B, n_t, S) or (B, S) numpy trajectories of the GPU run."""
    from oracle import cbase
    from voltax_gb300 import symbolic
    st = symbolic.structure(circuit)
    B = circuit.batch
    pick = sorted(set(np.linspace(0, B - 1, min(count, B)).round().astype(int).tolist()))
    z0 = None if isinstance(ic, str) else ic.numpy()
    method = w.method or "dc"
    nv = circuit.n_nodes
    worst = {"rel": 0.0, "kcl": 0.0, "ratio": 0.0}
    t0 = time.perf_counter()
    for b in pick:
        cs = cbase.CSystem(circuit, st, st.plan, b)
        zb = z[b].reshape(len(ts), circuit.size)
        if w.analysis == "dc":
            zr, okr, _ = cs.run(ts[:1], dc_first=True)
        else:
            zr, okr, _ = cs.run(ts, z0=z0, method=method, dc_first=z0 is None)
        a, r = zb[:, :nv], zr[:, :nv]
        worst["rel"] = max(worst["rel"], float(np.max(np.abs(a - r) / np.maximum(np.abs(r),
                                                                                 1e-3))))
        kcl, ratio = cs.check(ts[: len(zb)], zb, method=method if w.analysis != "dc" else "dc",
                              dc_first=z0 is None)
        worst["kcl"] = max(worst["kcl"], float(np.max(kcl)))
        worst["ratio"] = max(worst["ratio"], float(np.max(ratio)))
    return {"instances": len(pick), "time_points": len(ts),
            "max_rel_node_v": worst["rel"], "max_kcl_residual_a": worst["kcl"],
            "max_newton_step_ratio": worst["ratio"],
            "pass": bool(worst["rel"] <= 1e-9 and worst["ratio"] <= 1.0),
            "oracle": "oracle/cvx.c, FP64, 1 thread", "seconds": time.perf_counter() - t0}


def wl_sides(instances):
    from voltax_gb300 import workloads
    return workloads.grid_sides(instances, *GRID_SIDES, seed=0)


def oracle_check_grids(batch, z, sides, seed, count=4):
    """oracle_check for an uneven grid batch: the first `count` grids, each
    solved alone by the compiled oracle and checked at the batch's solution
    (node voltages and pad currents of that grid)."""
    from oracle import cbase
    from oracle import plan as oplan
    from voltax_gb300 import symbolic, workloads
    worst = {"rel": 0.0, "kcl": 0.0, "ratio": 0.0}
    t0 = time.perf_counter()
    ts = np.zeros(1)
    n = min(count, len(sides))
    for k in range(n):
        c = workloads.power_grid(sides[k], seed=seed + k)
        st = symbolic.structure(c)
        cs = cbase.CSystem(c, st, oplan.make_plan_numpy(st))
        zr, _, _ = cs.run(ts, dc_first=True)
        zk = np.empty(c.size)
        zk[: c.n_nodes] = z[[batch.node(f"g{k}_{nm}") for nm in c.layout.node_names]]
        pads = c.devices("VoltageSource")
        zk[[c.layout.internal(p) for p in pads]] = \
            z[[batch.layout.internal(f"g{k}_{p}") for p in pads]]
        a, r = zk[: c.n_nodes], zr[0, : c.n_nodes]
        worst["rel"] = max(worst["rel"], float(np.max(np.abs(a - r) /
                                                      np.maximum(np.abs(r), 1e-3))))
        kcl, ratio = cs.check(ts, zk[None], method="dc", dc_first=True)
        worst["kcl"] = max(worst["kcl"], float(np.max(kcl)))
        worst["ratio"] = max(worst["ratio"], float(np.max(ratio)))
    return {"instances": n, "grids": [int(x) for x in sides[:n]], "time_points": 1,
            "max_rel_node_v": worst["rel"], "max_kcl_residual_a": worst["kcl"],
            "max_newton_step_ratio": worst["ratio"],
            "pass": bool(worst["rel"] <= 1e-9 and worst["ratio"] <= 1.0),
            "oracle": "oracle/cvx.c, FP64, 1 thread, each grid alone",
            "seconds": time.perf_counter() - t0}


def fused_phases(lib, torch, dev, run, total_iters):
    """Per-phase SM cycles of the fused kernel over one profiled run
    (vxg_fused_set_profile): shares of the kernel time and CTA cycles per
    Newton iteration."""
    cyc = torch.zeros(8, dtype=torch.int64, device=dev)
    lib.vxg_fused_set_profile(cyc.data_ptr())
    try:
        run()
        torch.cuda.synchronize()
    finally:
        lib.vxg_fused_set_profile(None)
    c = cyc.cpu().numpy().astype(float)
    names = ["eval", "assemble", "factor", "solve", "update"]
    total = c[5]
    out = {n: {"share": c[i] / total, "cycles_per_newton_iter": c[i] / total_iters}
           for i, n in enumerate(names)}
    rest = total - c[:5].sum()
    out["other"] = {"share": rest / total, "cycles_per_newton_iter": rest / total_iters}
    out["kernel_cta_cycles"] = total
    return out


# ----------------------------------------------------------------- GPU arm
class GPU:
    """The device, process group, library and helpers one GPU run shares."""

    def __init__(self):
        import torch
        from voltax_gb300 import _lib
        self.torch = torch
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(self.local)
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("nccl")
            self.dist = dist
        self.dev = torch.device("cuda", self.local)
        self.lib = _lib.load()
        self.peaks = {}
        pk = ROOT / "MEASURED_PEAKS.json"
        if pk.exists():
            self.peaks = json.loads(pk.read_text())
        # inputs and states are far below L2; a 256 MB write flushes it
        self.flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=self.dev)

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()
        self.torch.cuda.synchronize()

    def timed(self, fn, k):
        """Device time (s) of k calls of fn, L2 flushed before each, CUDA
        events on the current stream bracketed by a barrier and a
        synchronize; the maximum over ranks."""
        torch = self.torch
        ms = []
        for _ in range(k):
            self.flush.zero_()
            self.barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            self.barrier()
            ms.append(e0.elapsed_time(e1))
        return max_over_ranks(self.dist, float(np.sum(ms)) / 1e3, self.dev)


def max_over_ranks(dist, seconds: float, device) -> float:
    """The job's time: the largest of the ranks' `seconds` (an all-reduce
    MAX over the process group; the value itself with no group). Replicas
    process fixed work each, so the aggregate rate is ranks x per-rank work
    over this time."""
    if dist is None:
        return seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t)


# FP64 work of the fused kernel's chosen form per Newton iteration of one
# 4-bit mirror-adder instance: 2 DFMA + DADD + DMUL thread instructions that
# ncu counted on the 512-instance x 21-point launch (fused_kernel<float,128>,
# the committed ncu summary of that launch), 2.96e9 FLOP, divided by that
# launch's 95,827 Newton iterations. It is fixed by the algorithm (the same
# device equations, residual and update every iteration), so it is the
# roofline's per-unit work; the FP64 peak is the hardware rate ncu reports
# (2 DFMA per cycle per SM) at the SM clock sampled during the run.
FUSED_FP64_FLOP_PER_ITER = {"adder_mc": 30_907.0}
FUSED_NCU = {"source": "profiles/fused_kernel_adder_mc512.md", "issue_active_pct": 21.1,
             "fp64_pipe_active_pct": 32.3, "warps_eligible_per_scheduler_cycle": 0.24,
             "top_stalls_per_issue": {"barrier": 6.04, "short_scoreboard": 4.17,
                                      "wait": 3.20},
             "dram_bytes_per_launch_512x21": 5.89e6}


def measure_circuit(g, a, w, instances, n_t, steps, warmup, cpu=None, full=True):
    """One circuit workload (the adder Monte Carlo, the ring oscillator, the
    100 x 100 grid): the chosen form timed with inputs resident in HBM, the
    plain FP64 form, their match, the oracle check, the end-to-end figure
    through the public API, and (full) phase cycles and the roofline."""
    torch = g.torch
    import voltax_gb300 as vx
    from voltax_gb300 import symbolic
    from voltax_gb300.analysis import _Call
    lib = g.lib
    circuit = w.circuit(instances, seed=g.rank)
    B = circuit.batch
    ts = w.times(n_t)
    ic = w.ic(circuit)
    out_nodes = ([circuit.node(n) for n in w.outputs] if w.outputs
                 else list(range(circuit.n_nodes)))
    dev_circuit = to_device(circuit, g.dev)
    host_circuit = to_device(circuit, None, pin=True)
    opts32 = vx.Options(precision="f32", engine=a.engine, refine=a.refine, block=a.block)
    opts64 = vx.Options(precision="f64", engine=a.engine, block=a.block)
    st = symbolic.structure(circuit)
    call32 = _Call(dev_circuit, opts32)
    engine_used = "fused" if call32.fused else "generic"

    def step(c, opts):
        if w.analysis == "dc":
            return vx.dc(c, options=opts)
        return vx.transient(c, ts, ic=ic, method=w.method, options=opts)

    for _ in range(warmup):
        step(dev_circuit, opts32)
    n0 = lib.vxg_launch_count()
    with Clocks(g.local) as clk:
        t32 = g.timed(lambda: step(dev_circuit, opts32), steps)
    launches = (lib.vxg_launch_count() - n0) // steps
    solves_per_step = B * len(ts)
    value = g.world * solves_per_step * steps / t32

    # the plain FP64 form on the same workload (fewer steps), and the match
    step(dev_circuit, opts64)
    k64 = max(1, min(steps, 2))
    t64 = g.timed(lambda: step(dev_circuit, opts64), k64)
    value64 = g.world * solves_per_step * k64 / t64
    s32 = step(dev_circuit, opts32)
    s64 = step(dev_circuit, opts64)
    nv = circuit.n_nodes
    match = float((s32.z[..., :nv] - s64.z[..., :nv]).abs().max())
    it = s32.iterations.reshape(-1, len(ts)).double() if w.analysis == "transient" else \
        s32.iterations.reshape(-1, 1).double()
    iters = float(it[:, 1:].mean()) if w.analysis == "transient" else float(it.mean())
    total_iters = int(it.sum())  # Newton iterations of one step, all instances
    it64 = float(s64.iterations.double().sum())

    # end to end through the public API: parameters from pinned host memory,
    # the output node waveforms back to pinned host memory
    h2d = h2d_bytes(host_circuit)
    out_host = torch.empty(tuple(s32.z[..., out_nodes].shape), dtype=torch.float64,
                           pin_memory=True)

    def e2e_step():
        s = step(host_circuit, opts32)
        out_host.copy_(s.z[..., out_nodes], non_blocking=True)

    e2e_step()
    t_e2e = g.timed(e2e_step, steps)
    e2e_value = g.world * solves_per_step * steps / t_e2e

    phases = None
    if full and engine_used == "fused":
        phases = {"chosen": fused_phases(lib, torch, g.dev, lambda: step(dev_circuit, opts32),
                                         total_iters),
                  "plain_fp64": fused_phases(lib, torch, g.dev,
                                             lambda: step(dev_circuit, opts64), it64)}
    out = {
        "value": value, "unit": UNIT, "ms_per_step": 1e3 * t32 / steps, "steps": steps,
        "warmup": warmup,
        "config": {"workload": w.label(B, len(ts)), "instances": B, "time_points": len(ts),
                   "method": w.method or "dc", "t_stop_s": w.t_stop,
                   "solves_per_step": solves_per_step, "engine": engine_used,
                   "block": call32.block if engine_used == "fused" else None,
                   "refine": call32.refine,
                   "l2": "flushed between timed steps (256 MB write)",
                   "parallelism": "replicas" if g.world > 1 else "single GPU"},
        "plain_fp64": {"value": value64, "unit": UNIT, "speedup": value / value64},
        "match": {"max_abs_node_v_diff_vs_fp64": match, "converged": bool(s32.converged.all()),
                  "mean_newton_iters": iters},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(out_host.numel() * 8)},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if phases:
        out["phases"] = phases
    if full:
        out["roofline"] = roofline(g, w, st, engine_used, call32, B, len(ts), total_iters,
                                   t32 / steps, out["clocks"])
    if g.rank == 0:
        zs = s32.z.cpu().numpy()
        if zs.ndim == 1 or (w.analysis == "transient" and zs.ndim == 2):
            zs = zs[None]
        out["oracle_check"] = oracle_check(w, circuit, zs, ts, ic)
    if cpu is not None:
        out["cpu_baseline"] = cpu
    return out


def roofline(g, w, st, engine_used, call32, B, n_t, total_iters, step_s, clk):
    """Roofline of the dominant kernel. The fused kernel keeps every Newton
    iteration on chip (its DRAM traffic is the parameters in and the states
    out), and its busiest pipe is FP64 (device currents and charges, the
    residual, the update): it is placed against the FP64 rate. The HBM frame
    of an unfused implementation of the same step is kept for context."""
    fe = int(st.plan.stats["factor_entries"])
    bytes_per_iter = 8 * st.nnz + 4 * (st.nnz + 2 * fe) + 8 * 6 * st.size
    hbm_peak = float(g.peaks.get("hbm_gbs", 6800.0))
    hbm = {"achieved_gbs": bytes_per_iter * total_iters / step_s / 1e9, "peak_gbs": hbm_peak,
           "peak_source": "measured" if g.peaks else "fallback",
           "algorithmic_bytes_per_launch": bytes_per_iter * total_iters}
    flop = FUSED_FP64_FLOP_PER_ITER.get(w.name)
    if engine_used != "fused" or flop is None or call32.block == 32:
        return {"bound": "hbm", "kernel": "factor/solve level kernels"
                if engine_used != "fused" else "fused_kernel<float>",
                "achieved": hbm["achieved_gbs"], "peak": hbm_peak, "unit": "GB/s",
                "frac": hbm["achieved_gbs"] / hbm_peak, "traffic": None,
                "peak_source": hbm["peak_source"],
                "newton_iterations_per_launch": total_iters}
    sms = g.torch.cuda.get_device_properties(g.dev).multi_processor_count
    mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0
    peak = 2 * 2 * sms * mhz * 1e6 / 1e12
    achieved = flop * total_iters / step_s / 1e12
    packed = sum(t.numel() * 8 for t in call32.keep)
    return {"bound": "fp64", "kernel": f"fused_kernel<float,{call32.block}>",
            "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "traffic": packed + B * n_t * (8 * st.size + 8),
            "peak_source": f"FP64 pipe: 2 DFMA/cycle/SM (ncu peak) x {sms} SMs x {mhz:.0f} MHz",
            "fp64_flop_per_newton_iter": flop, "newton_iterations_per_launch": total_iters,
            "unfused_hbm_frame": hbm, "ncu": FUSED_NCU}


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
        return
    # CPU legs first (before any CUDA work), rank 0 only
    rank = int(os.environ.get("RANK", "0"))
    w = WORKLOADS[a.workload]
    cpu = cpu_baseline(w, a.time_points, a.instances) if rank == 0 and not a.no_cpu else None
    superlu = None
    if w.name not in ("ota_warm", "grids"):
        superlu = cpu_superlu(w, a.instances) if rank == 0 and not a.no_cpu else None
    g = GPU()
    if w.name == "ota_warm":
        res = measure_warm(g, a, w, a.instances, a.train or OTA_TRAIN, a.epochs, a.steps,
                           a.warmup, cpu)
    elif w.name == "grids":
        res = measure_grids(g, a, w, cpu)
    else:
        res = measure_circuit(g, a, w, a.instances, a.time_points, a.steps, a.warmup, cpu)
    if superlu:
        res["cpu_superlu"] = superlu
    if w.name == "adder_mc" and not a.no_extra:
        res["configs"] = other_configs(g, a)
    if g.rank != 0:
        return
    # voltax publishes one workload: 499 us per step on one CPU thread
    # (benchmarks/README.md:217), i.e. 2004 Newton solves/s
    vs_baseline = res["value"] / (1.0 / 499e-6) if w.name == "ring101_l1" else None
    dtype = "f32 LU + f64 residual/refinement"
    if w.name == "ota_warm":
        dtype += "; MLP bf16 x bf16 -> f32"
    line = {"metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": g.world,
            "steps": res["steps"], "warmup": res["warmup"], "ms_per_step": res["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": vs_baseline,
            "dtype": dtype, "data": "synthetic"}
    line.update({k: v for k, v in res.items() if k not in line})
    print(json.dumps(line))


def other_configs(g, a):
    """Bounded runs of the other single-GPU benchmark configurations, each
    with its own timing and oracle check: the 101-stage ring oscillator
    (one 2001-point trapezoidal transient per step), the 100 x 100 power
    grid DC, and the learned warm start on 10,000 held-out OTA-chain
    instances with a network trained first on 20,000 operating points of the
    plain solver (training reported separately, not timed)."""
    steps, warmup = max(1, min(a.steps, 5)), max(1, min(a.warmup, 3))
    out = {}
    ring = WORKLOADS["ring101"]
    out["ring101_trap2001"] = measure_circuit(g, a, ring, 1, ring.n_t, min(steps, 3), warmup,
                                              full=False)
    grid = WORKLOADS["grid100"]
    out["power_grid100_dc"] = measure_circuit(g, a, grid, 1, 1, 2 * steps, warmup, full=False)
    ota = WORKLOADS["ota_warm"]
    out["ota_chain_warm_start"] = measure_warm(g, a, ota, ota.default_instances, 20_000, 40,
                                               steps, warmup)
    return out



# --------------------------------------------------- learned warm start arm
def measure_warm(g, a, w, instances, n_train, epochs, steps, warmup, cpu=None):
    """DC operating points of held-out OTA-chain instances from the MLP's
    predicted guess (inference + Newton + fallback, one step) against Newton
    from the default guess. The network is trained first (untimed, reported
    separately) on operating points the plain FP64 solver produces for
    other parameters."""
    torch = g.torch
    import voltax_gb300 as vx
    from voltax_gb300 import warmstart, workloads

    rank, dev, lib = g.rank, g.dev, g.lib
    base = workloads.ota_chain(OTA_STAGES)

    def make(P):
        return workloads.apply_ota_params(base, P)

    plain = vx.Options(precision="f64")
    chosen = vx.Options(precision="f32")
    # training data by the plain solver (default guess, gmin stepping)
    Xtr = workloads.ota_params(n_train, seed=OTA_TRAIN_SEED + 1000 * rank)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    Vtr, conv_tr, it_tr = warmstart.solve_dataset(make, Xtr, chunk=25000, options=plain)
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    keep = conv_tr.cpu().numpy()
    model = warmstart.WarmStartMLP(Xtr.shape[1], Vtr.shape[1], hidden=512, seed=0)
    t0 = time.perf_counter()
    hist = model.fit(Xtr[keep], Vtr[torch.as_tensor(keep, device=Vtr.device)],
                     epochs=epochs, batch=1024, lr=2e-3, lr_final=2e-5)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0

    X = workloads.ota_params(instances, seed=OTA_TEST_SEED + rank)
    c_host = make(X)
    c = to_device(c_host, dev)  # parameters resident in HBM for `value`
    Xd = torch.as_tensor(X, device=dev)

    warm = lambda: warmstart.dc(c, Xd, model, options=chosen)  # noqa: E731
    cold = lambda: vx.dc(c, options=chosen)  # noqa: E731
    cold64 = lambda: vx.dc(c, options=plain)  # noqa: E731
    for _ in range(warmup):
        warm()
    n0 = lib.vxg_launch_count()
    with Clocks(g.local) as clk:
        t_warm = g.timed(warm, steps)
    launches = (lib.vxg_launch_count() - n0) // steps
    k_cold = max(1, min(steps, 2))
    cold()
    t_cold = g.timed(cold, k_cold)
    cold64()
    t_cold64 = g.timed(cold64, k_cold)
    B = instances
    value = B * steps / t_warm
    s_warm, s_cold, s_ref = warm(), cold(), cold64()
    nv = c.layout.n_nodes
    ref_v = s_ref.z[:, :nv]
    scale = ref_v.abs().amax(1, keepdim=True)
    rel = float(((s_warm.z[:, :nv] - ref_v).abs() / scale).max())
    it_w = s_warm.iterations.double()
    it_c = s_cold.iterations.double()

    # end to end: parameters and the MLP inputs from pinned host memory, node
    # voltages back to pinned host memory
    host_c = to_device(c_host, None, pin=True)
    Xh = torch.as_tensor(X).pin_memory()
    out = torch.empty((B, nv), dtype=torch.float64, pin_memory=True)
    h2d = Xh.numel() * 8 + h2d_bytes(host_c)

    def e2e():
        s = warmstart.dc(host_c, Xh.to(dev, non_blocking=True), model, options=chosen)
        out.copy_(s.z[:, :nv], non_blocking=True)

    e2e()
    t_e2e = g.timed(e2e, steps)
    res = {
        "value": value, "unit": UNIT, "ms_per_step": 1e3 * t_warm / steps, "steps": steps,
        "warmup": warmup,
        "config": {"workload": w.label(B, 1), "instances": B, "stages": OTA_STAGES,
                   "nodes": nv, "train_instances": n_train, "epochs": epochs,
                   "mlp": f"{Xtr.shape[1]}-512-512-{Vtr.shape[1]} GELU",
                   "l2": "flushed between timed steps (256 MB write)"},
        "default_guess": {"value": B * k_cold / t_cold, "unit": UNIT,
                          "mean_newton_iters": float(it_c.mean()),
                          "max_newton_iters": int(it_c.max())},
        "plain_fp64_default_guess": {"value": B * k_cold / t_cold64, "unit": UNIT},
        "warm_start": {"mean_newton_iters": float(it_w.mean()),
                       "max_newton_iters": int(it_w.max()),
                       "iteration_reduction": float(it_c.mean() / it_w.mean()),
                       "fallbacks": int((s_warm.iterations > chosen.direct_steps).sum()),
                       "converged": bool(s_warm.converged.all())},
        "match": {"max_rel_node_v_diff_vs_plain_fp64_default": rel},
        "training": {"data_gen_s": gen_s, "data_gen_solves_per_s": n_train / gen_s,
                     "data_mean_newton_iters": float(it_tr.double().mean()),
                     "train_s": train_s, "loss_first_epoch": hist[0],
                     "loss_last_epoch": hist[-1]},
        "e2e": {"value": B * steps / t_e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(out.numel() * 8)},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if rank == 0:
        res["oracle_check"] = oracle_check(w, c_host, s_warm.z.cpu().numpy(), np.zeros(1), "dc")
    if cpu is not None:
        res["cpu_baseline"] = cpu
    return res


# ------------------------------------------------------- uneven grid batch arm
def measure_grids(g, a, w, cpu=None):
    """An uneven batch of power grids in one segmented circuit: DC of every
    grid (one solve per grid), and the adjoint of each grid's largest IR drop
    with respect to all segment conductances (one transposed solve for the
    batch)."""
    torch = g.torch
    import voltax_gb300 as vx
    from voltax_gb300 import symbolic

    dev, lib = g.dev, g.lib
    t0 = time.perf_counter()
    circuit = w.circuit(a.instances, seed=0)
    st = symbolic.structure(circuit)
    st.plan  # the C++ planner (otherwise built lazily by the first analysis)
    plan_s = time.perf_counter() - t0
    n_grids = a.instances
    c_dev = to_device(circuit, dev)
    segs = torch.as_tensor(circuit.unknown_segments()[: circuit.n_nodes], device=dev,
                           dtype=torch.long)
    chosen = vx.Options(precision="f32")
    plain = vx.Options(precision="f64")
    timed = g.timed

    def drops(v):
        """largest IR drop (1 V - v) of each grid, by segment"""
        d = torch.full((n_grids,), -float("inf"), dtype=v.dtype, device=v.device)
        return d.scatter_reduce(0, segs, 1.0 - v, reduce="amax")

    def adjoint(opts):
        el = c_dev.elements["Resistor"]
        e2 = el.with_nodes(el.nodes)
        e2.log_r = el.log_r.detach().clone().requires_grad_(True)
        sol = vx.dc(c_dev.replace("Resistor", e2), options=opts)
        drops(sol.z[: circuit.n_nodes]).sum().backward()
        return e2.log_r.grad

    fwd = lambda: vx.dc(c_dev, options=chosen)  # noqa: E731
    for _ in range(a.warmup):
        fwd()
    n0 = lib.vxg_launch_count()
    with Clocks(g.local) as clk:
        t_fwd = timed(fwd, a.steps)
    launches = (lib.vxg_launch_count() - n0) // a.steps
    vx.dc(c_dev, options=plain)
    t_plain = timed(lambda: vx.dc(c_dev, options=plain), max(1, min(a.steps, 2)))
    adjoint(chosen)
    t_adj = timed(lambda: adjoint(chosen), max(1, min(a.steps, 2)))
    s32, s64 = fwd(), vx.dc(c_dev, options=plain)
    nv = circuit.n_nodes
    match = float((s32.z[:nv] - s64.z[:nv]).abs().max())
    g32, g64 = adjoint(chosen), adjoint(plain)
    grad_rel = float((g32 - g64).norm() / g64.norm())
    host_c = to_device(circuit, None, pin=True)
    out = torch.empty(nv, dtype=torch.float64, pin_memory=True)

    def e2e():
        s = vx.dc(host_c, options=chosen)
        out.copy_(s.z[:nv], non_blocking=True)

    e2e()
    t_e2e = timed(e2e, a.steps)
    sides = wl_sides(n_grids)
    res = {
        "value": n_grids * a.steps / t_fwd, "unit": UNIT, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": 1e3 * t_fwd / a.steps,
        "config": {"workload": w.label(n_grids, 1), "grids": n_grids, "sides": sides,
                   "unknowns": circuit.size, "nnz": st.nnz,
                   "factor_entries": int(st.plan.stats["factor_entries"]),
                   "largest_supernode": int(st.plan.stats["largest_supernode"]),
                   "host_plan_s": plan_s,
                   "l2": "flushed between timed steps (256 MB write)"},
        "plain_fp64": {"value": n_grids / (t_plain / max(1, min(a.steps, 2))), "unit": UNIT},
        "adjoint": {"value": n_grids / (t_adj / max(1, min(a.steps, 2))), "unit":
                    "grids/s (DC + transposed solve + d max-drop / d log r)",
                    "rel_diff_vs_fp64": grad_rel},
        "match": {"max_abs_node_v_diff_vs_fp64": match,
                  "converged": bool(s32.converged.all()),
                  "newton_iters": [int(x) for x in s32.iterations.reshape(-1)[:4]]},
        "e2e": {"value": n_grids * a.steps / t_e2e, "unit": UNIT,
                "h2d_bytes_per_step": int(h2d_bytes(host_c)), "d2h_bytes_per_step": nv * 8},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    res["plain_fp64"]["speedup"] = res["value"] / res["plain_fp64"]["value"]
    if g.rank == 0:
        res["oracle_check"] = oracle_check_grids(circuit, s32.z.cpu().numpy(),
                                                 wl_sides(a.instances), seed=0)
    if cpu is not None:
        res["cpu_baseline"] = cpu
    return res


if __name__ == "__main__":
    main()
