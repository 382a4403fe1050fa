"""Device models on the Newton hot path, as vectorized element groups.

Each class mirrors a voltax element (same terminals, internal unknowns and
parameter names; log-space storage of positive quantities):

* `Resistor`, `Capacitor`      -- voltax/elements/passive.py:13-59
* `Conductance`                -- voltax/elements/behavioral.py:29-99
* `VoltageSource`, `CurrentSource` -- voltax/elements/sources.py:58-115
* `MOSProcess`, `EKVMOSFET`    -- voltax/elements/mosfet.py:26-205

The physics itself is evaluated by the CUDA device kernels
(``voltax_gb300/csrc/devices.cuh``). On the host an element only knows its
nodes, its parameters (float64 torch tensors, ``(N,)`` or ``(B, N)`` for a
batch of B circuit instances) and how to turn them into the kernel's
per-device parameter rows (`gpu_params`). Those rows are computed with torch
ops, so gradients flow from the kernel's parameter VJP back to the user's
parameters through ordinary torch autograd.
"""

from __future__ import annotations

from typing import Any, Sequence

import math

import numpy as np
import torch

from .signals import Constant, Signal, as_signal

_F64 = torch.float64
VT_300K = 0.025852
"""Thermal voltage kT/q at 300 K (voltax/elements/semiconductor.py:13)."""

# kernel codes of the device table (must match include/vxg.h)
KIND_CONDUCTANCE = 0
KIND_CAPACITOR = 1
KIND_VSOURCE = 2
KIND_ISOURCE = 3
KIND_EKV = 4
KIND_L1 = 5
KIND_DIODE = 6
KIND_INDUCTOR = 7
KIND_VCCS = 8
KIND_BJT = 9
KIND_VCVS = 10
KIND_CCCS = 11
KIND_CCVS = 12
KIND_XFMR = 13
KIND_IDEAL_OPAMP = 14
KIND_OPAMP = 15
KIND_SWITCH = 16
KIND_COUPLED_L = 17


def _t(x) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x.to(_F64)
    return torch.as_tensor(np.asarray(x, dtype=np.float64))


def positive_log(x) -> torch.Tensor:
    """``log(x)``, validating that `x` is positive (voltax/element.py:40-45)."""
    x = _t(x)
    if not x.requires_grad and bool(torch.any(x <= 0)):
        raise ValueError(f"expected a positive value, got {x}")
    return torch.log(x)


def _is_single(nodes: Sequence[Any]) -> bool:
    return len(nodes) > 0 and isinstance(nodes[0], (int, str, np.integer))


class Element:
    """A vectorized group of ``N`` devices of one type (voltax/element.py:66-131).

    Subclasses declare ``terminals``, ``n_internal``, ``internal_names``,
    ``shared`` (fields common to all devices), ``fields`` (per-device
    parameter tensors) and the kernel ``kind``.
    """

    terminals: tuple[str, ...] = ()
    n_internal: int = 0
    internal_names: tuple[str, ...] = ()
    shared: tuple[str, ...] = ()
    fields: tuple[str, ...] = ()
    static: tuple[str, ...] = ()
    local: bool = True
    kind: int = -1
    has_charges: bool = False

    nodes: tuple[tuple[Any, ...], ...]

    # ------------------------------------------------------------ structure
    @property
    def size(self) -> int:
        return len(self.nodes)

    def node_array(self) -> np.ndarray:
        """The node table as a read-only ``(N, T)`` int64 array, converted
        once per node table (a copy made by `with_nodes` that keeps the
        table keeps the array)."""
        held = self.__dict__.get("_node_table")
        if held is not None and held[0] is self.nodes:
            return held[1]
        table = np.asarray(self.nodes, dtype=np.int64).reshape(self.size, -1)
        table.setflags(write=False)
        self.__dict__["_node_table"] = (self.nodes, table)
        return table

    def with_nodes(self, nodes) -> "Element":
        new = object.__new__(type(self))
        new.__dict__.update(self.__dict__)
        # the same node table keeps its identity (a circuit then keeps its topology key)
        new.nodes = self.nodes if nodes is self.nodes else tuple(map(tuple, nodes))
        return new

    @staticmethod
    def _devices(nodes) -> tuple[tuple[Any, ...], ...]:
        if _is_single(nodes):
            return (tuple(nodes),)
        return tuple(map(tuple, nodes))

    def _per_device(self, value) -> torch.Tensor:
        value = _t(value)
        if value.ndim == 0:
            return value.expand(self.size).clone()
        if value.shape[-1] != self.size:
            raise ValueError(f"expected a scalar or shape (..., {self.size}) value, "
                             f"got {tuple(value.shape)}")
        return value

    def _log_per_device(self, value) -> torch.Tensor:
        return self._per_device(positive_log(value))

    # ------------------------------------------------------------ parameters
    def param_tensors(self) -> dict[str, torch.Tensor]:
        return {f: getattr(self, f) for f in self.fields}

    def batch_size(self) -> int:
        """Instances in the parameters' leading axis (1 when unbatched)."""
        sizes = {p.shape[0] for p in self._all_params() if p.ndim == 2}
        if len(sizes) > 1:
            raise ValueError(f"inconsistent batch sizes {sizes}")
        return sizes.pop() if sizes else 1

    def _all_params(self) -> list[torch.Tensor]:
        return list(self.param_tensors().values())

    def get(self, field: str, index=slice(None)):
        return getattr(self, field)[..., index]

    def set(self, index: int, **values) -> "Element":
        """Copy with device `index`'s parameters replaced (physical units;
        log-space fields handled as in voltax/element.py:143-163)."""
        out = self.with_nodes(self.nodes)
        for key, value in values.items():
            log_attr = f"log_{key.rstrip('_')}"
            if log_attr in self.fields:
                attr, value = log_attr, torch.log(_t(value))
            elif key in self.fields:
                attr, value = key, _t(value)
            else:
                settable = sorted(f.removeprefix("log_") for f in self.fields)
                raise AttributeError(f"{type(self).__name__} has no per-device "
                                     f"parameter {key!r}; settable: {settable}")
            new = getattr(out, attr).clone()
            new[..., index] = value
            setattr(out, attr, new)
        return out

    def gpu_params(self) -> list[torch.Tensor]:
        """Kernel parameter rows, each ``(N,)`` or ``(B, N)`` float64."""
        raise NotImplementedError

    def group_key(self) -> tuple:
        """Elements with equal keys can be fused (voltax/element.py:218-242)."""
        static = tuple((s, getattr(self, s)) for s in self.static)
        shared = tuple(id(getattr(self, s)) for s in self.shared)
        return (type(self), static, shared)


def concatenate(elements: Sequence[Element]) -> Element:
    """Fuse same-type elements into one group (voltax/element.py:198-215)."""
    first = elements[0]
    if len(elements) == 1:
        return first
    out = first.with_nodes([d for e in elements for d in e.nodes])
    for f in first.fields:
        xs = [getattr(e, f) for e in elements]
        batched = max(x.ndim for x in xs) == 2
        if batched:
            B = max(x.shape[0] for x in xs if x.ndim == 2)
            xs = [x if x.ndim == 2 else x.expand(B, x.shape[-1]) for x in xs]
        setattr(out, f, torch.cat(xs, dim=-1))
    for f in ("ac", "ac_phase"):
        if hasattr(first, f):
            setattr(out, f, torch.cat([_t(getattr(e, f)).reshape(-1) for e in elements]))
    if hasattr(first, "value") and isinstance(first.value, Signal):
        sigs = [e.value for e in elements]
        params = []
        for i in range(len(first.value.fields)):
            xs = [s.params()[i] for s in sigs]
            batched = max(x.ndim for x in xs) == 2
            if batched:
                B = max(x.shape[0] for x in xs if x.ndim == 2)
                xs = [x if x.ndim == 2 else x.expand(B, x.shape[-1]) for x in xs]
            params.append(torch.cat(xs, dim=-1))
        out.value = first.value.replace_params(params)
    return out


# =============================================================================
# Linear two-terminal elements
# =============================================================================


class Resistor(Element):
    """Linear resistor, ``i = (v_p - v_n) exp(-log_r)`` (passive.py:13-38)."""

    terminals = ("p", "n")
    fields = ("log_r",)
    kind = KIND_CONDUCTANCE

    def __init__(self, nodes, r):
        self.nodes = self._devices(nodes)
        self.log_r = self._log_per_device(r)

    @property
    def r(self):
        return torch.exp(self.log_r)

    @property
    def g(self):
        return torch.exp(-self.log_r)

    def gpu_params(self):
        return [torch.exp(-self.log_r)]


class Conductance(Element):
    """Linear conductance ``i = g(theta) (v_p - v_n)`` with a chosen map from
    ``theta`` to ``g`` (behavioral.py:29-99): log, softplus, sigmoid, linear."""

    terminals = ("p", "n")
    fields = ("theta",)
    static = ("transform", "g_min", "g_max")
    kind = KIND_CONDUCTANCE

    def __init__(self, nodes, g, transform: str = "log", g_min: float = 0.0,
                 g_max: float = 1.0):
        if transform not in ("log", "softplus", "sigmoid", "linear"):
            raise ValueError(f"unknown transform {transform!r}")
        self.nodes = self._devices(nodes)
        self.transform, self.g_min, self.g_max = transform, g_min, g_max
        self.theta = self._per_device(self.to_theta(g))

    def to_theta(self, g):
        g = _t(g)
        if self.transform == "log":
            return torch.log(g)
        if self.transform == "softplus":
            y = g - self.g_min
            return y + torch.log(-torch.expm1(-y))
        if self.transform == "sigmoid":
            u = (g - self.g_min) / (self.g_max - self.g_min)
            return torch.log(u) - torch.log1p(-u)
        return g

    @property
    def g(self):
        th = self.theta
        if self.transform == "log":
            return torch.exp(th)
        if self.transform == "softplus":
            return self.g_min + torch.logaddexp(th, torch.zeros_like(th))
        if self.transform == "sigmoid":
            return self.g_min + (self.g_max - self.g_min) * torch.sigmoid(th)
        return th

    def set(self, index, **values):
        if "g" in values:
            values["theta"] = self.to_theta(values.pop("g"))
        if "r" in values:
            values["theta"] = self.to_theta(1.0 / _t(values.pop("r")))
        return super().set(index, **values)

    def gpu_params(self):
        return [self.g]


class Capacitor(Element):
    """Linear capacitor, ``q = c (v_p - v_n)`` (passive.py:41-59)."""

    terminals = ("p", "n")
    fields = ("log_c",)
    kind = KIND_CAPACITOR
    has_charges = True

    def __init__(self, nodes, c):
        self.nodes = self._devices(nodes)
        self.log_c = self._log_per_device(c)

    @property
    def c(self):
        return torch.exp(self.log_c)

    def gpu_params(self):
        return [torch.exp(self.log_c)]


# =============================================================================
# Sources
# =============================================================================


class _Source(Element):
    terminals = ("p", "n")
    fields = ()

    def _init_source(self, nodes, value, ac=0.0, ac_phase=0.0):
        self.nodes = self._devices(nodes)
        sig = as_signal(value)
        single = _is_single(nodes)
        self.value = sig.map(lambda x: x.reshape(1) if single and x.ndim == 0
                             else self._per_device(x))
        # small-signal stimulus (host side only: AC analysis)
        self.ac = self._per_device(ac)
        self.ac_phase = self._per_device(ac_phase)

    def phasor(self):
        """``ac exp(j ac_phase)`` per device (numpy complex, sources.py:30-36)."""
        ac = np.asarray(getattr(self, "ac", np.zeros(self.size)), dtype=float)
        ph = np.asarray(getattr(self, "ac_phase", np.zeros(self.size)), dtype=float)
        return np.broadcast_to(ac * np.exp(1j * np.deg2rad(ph)), (self.size,))

    @property
    def static(self):  # waveform type decides the kernel branch
        return ("wave_kind",)

    @property
    def wave_kind(self) -> int:
        return self.value.kind

    def _all_params(self):
        return self.value.params()

    def with_dc(self, values) -> "_Source":
        out = self.with_nodes(self.nodes)
        out.value = Constant(self._per_device(values))
        return out

    def set(self, index, **values):
        out = self.with_nodes(self.nodes)
        out.value = self.value.map(lambda x: x.clone())
        for key in [k for k in values if k in self.value.fields and k != "value"]:
            getattr(out.value, key)[..., index] = _t(values.pop(key))
        if "value" in values:
            dc = _t(values.pop("value"))
            if isinstance(out.value, Constant):
                v = out.value.value.clone()
                if dc.ndim == 1 and v.ndim == 1 and dc.shape[0] != v.shape[0]:
                    v = v.expand(dc.shape[0], v.shape[0]).clone()
                    v[:, index] = dc
                else:
                    v[..., index] = dc
                out.value = Constant(v)
            elif self.size == 1:
                out.value = Constant(dc.reshape(-1) if dc.ndim else dc.reshape(1))
            else:
                raise TypeError("set(value=...) on a batched non-DC source")
        if values:
            raise AttributeError(f"unknown source parameters {sorted(values)}")
        return out

    def gpu_params(self):
        return self.value.params()


class VoltageSource(_Source):
    """Independent voltage source ``v_p - v_n = value(t)``; internal unknown
    ``i`` flows p -> n through the source (sources.py:58-87)."""

    n_internal = 1
    internal_names = ("i",)
    kind = KIND_VSOURCE

    def __init__(self, nodes, value: Signal | Any = 0.0, ac=0.0, ac_phase=0.0):
        self._init_source(nodes, value, ac, ac_phase)


class CurrentSource(_Source):
    """Independent current source driving ``value(t)`` from p to n through
    the source (sources.py:90-115)."""

    kind = KIND_ISOURCE

    def __init__(self, nodes, value: Signal | Any = 0.0, ac=0.0, ac_phase=0.0):
        self._init_source(nodes, value, ac, ac_phase)


# =============================================================================
# EKV MOSFET
# =============================================================================


class MOSProcess:
    """Shared technology parameters (mosfet.py:26-87)."""

    def __init__(self, kp=400e-6, vth=0.4, n=1.3, lam=0.04, vt=VT_300K, gamma=0.0,
                 phi=0.7, cox=8.6e-3, cov=0.3e-9):
        self.log_kp = positive_log(kp)
        self.vth, self.n, self.lam, self.vt = _t(vth), _t(n), _t(lam), _t(vt)
        self.gamma, self.phi = _t(gamma), _t(phi)
        self.log_cox = positive_log(cox)
        self.log_cov = positive_log(cov)

    @classmethod
    def nmos(cls, **overrides) -> "MOSProcess":
        return cls(**{"kp": 400e-6, **overrides})

    @classmethod
    def pmos(cls, **overrides) -> "MOSProcess":
        return cls(**{"kp": 200e-6, **overrides})

    @property
    def kp(self):
        return torch.exp(self.log_kp)

    @property
    def cox(self):
        return torch.exp(self.log_cox)

    @property
    def cov(self):
        return torch.exp(self.log_cov)


class EKVMOSFET(Element):
    """EKV 2.6-style MOSFET (mosfet.py:155-205); terminals ``(d, g, s, b)``.

    Kernel parameter rows (all per device): sign, i_spec = 2 n kp (W/L) vt^2,
    vth, dvth, n, vt, lam, c_ox = cox W L, cov W, then the derived 1/n,
    1/(2 vt), c_ox n vt and -(n - 1)/n.
    """

    terminals = ("d", "g", "s", "b")
    shared = ("process",)
    fields = ("log_w", "log_l", "dvth")
    static = ("polarity",)
    kind = KIND_EKV
    has_charges = True

    def __init__(self, nodes, w=1e-6, l=0.13e-6, process: MOSProcess | None = None,
                 polarity: str = "n", dvth=0.0):
        if polarity not in ("n", "p"):
            raise ValueError(f"polarity must be 'n' or 'p', got {polarity!r}")
        self.nodes = self._devices(nodes)
        self.polarity = polarity
        self.log_w = self._log_per_device(w)
        self.log_l = self._log_per_device(l)
        self.dvth = self._per_device(dvth)
        if process is None:
            process = MOSProcess.nmos() if polarity == "n" else MOSProcess.pmos()
        self.process = process

    @property
    def w(self):
        return torch.exp(self.log_w)

    @property
    def l(self):
        return torch.exp(self.log_l)

    @property
    def sign(self) -> float:
        return 1.0 if self.polarity == "n" else -1.0

    def gpu_params(self):
        p = self.process
        w, l = self.w, self.l
        i_spec = 2 * p.n * p.kp * (w / l) * p.vt ** 2
        shape = i_spec.shape

        def full(x):
            return _t(x).expand(shape)

        c_ox = p.cox * w * l
        # rows 9-12 are derived from rows 4, 5 and 7 so the kernel multiplies
        # instead of dividing; gradients flow through rows 0-8
        return [full(self.sign), i_spec, full(p.vth), self.dvth.expand(shape),
                full(p.n), full(p.vt), full(p.lam), c_ox, p.cov * w,
                full(1.0 / p.n), full(1.0 / (2.0 * p.vt)), c_ox * p.n * p.vt,
                full(-(p.n - 1.0) / p.n)]


class Level1MOSFET(EKVMOSFET):
    """Shichman-Hodges (SPICE Level 1) square-law MOSFET, smoothed
    (mosfet.py:208-257); terminals ``(d, g, s, b)``.

    ``I_ds = kp (W/L) (v_ov v_ds - v_ds^2/2)`` in triode and
    ``kp (W/L) v_ov^2 / 2`` in saturation, times ``(1 + lam v_ds)``, with
    ``v_ov = smooth softplus((v_gs - v_t)/smooth)`` (``smooth=0``: the exact
    SPICE model), drain and source swapped for ``v_ds < 0``, the body effect
    ``gamma (sqrt(phi + v_sb) - sqrt(phi))`` linearised under forward bias,
    and overlap charges only.

    Kernel parameter rows (per device): sign, kp W/L, vth, dvth, lam, gamma,
    phi, smooth, cov W, then the derived sqrt(phi), 1/(2 sqrt(phi)) and
    1/smooth (0 when smooth = 0).
    """

    static = ("polarity", "smooth")
    kind = KIND_L1

    def __init__(self, nodes, w=1e-6, l=0.13e-6, process: MOSProcess | None = None,
                 polarity: str = "n", dvth=0.0, smooth: float = 0.02):
        super().__init__(nodes, w, l, process, polarity, dvth)
        self.smooth = float(smooth)

    def gpu_params(self):
        p = self.process
        w, l = self.w, self.l
        k = p.kp * (w / l)
        shape = k.shape

        def full(x):
            return _t(x).expand(shape)

        sphi = torch.sqrt(p.phi)
        # rows 9-11 are derived from rows 6 and 7 so the kernel multiplies
        # instead of dividing; gradients flow through rows 0-8
        return [full(self.sign), k, full(p.vth), self.dvth.expand(shape), full(p.lam),
                full(p.gamma), full(p.phi), full(self.smooth), p.cov * w, full(sphi),
                full(0.5 / sphi), full(1.0 / self.smooth if self.smooth > 0 else 0.0)]


class Inductor(Element):
    """Inductor with series resistance (passive.py:62-87). Internal unknown:
    the branch current ``i`` (``p -> n``); ``l di/dt + rs i - (v_p - v_n) = 0``.

    Kernel parameter rows: l, rs."""

    terminals = ("p", "n")
    n_internal = 1
    internal_names = ("i",)
    fields = ("log_l", "rs")
    kind = KIND_INDUCTOR
    has_charges = True

    def __init__(self, nodes, l, rs=0.0):
        self.nodes = self._devices(nodes)
        self.log_l = self._log_per_device(l)
        self.rs = self._per_device(rs)

    @property
    def l(self):
        return torch.exp(self.log_l)

    def gpu_params(self):
        return [torch.exp(self.log_l), self.rs.expand(self.log_l.shape)]


class CoupledInductors(Element):
    """``N`` inductors with a full mutual-inductance matrix across the group,
    ``M = k sqrt(l l^T)`` off the diagonal and ``l`` on it: the flux of
    device d is ``sum_e M_de i_e``. Its devices interact, so the group is
    non-local (``local = False``, voltax/element.py:30-34, 76-79): its
    Jacobian is one block over all ``3 N`` group unknowns, stamped at the
    positions voltax gives a non-local group (voltax/sparse.py:87, 245-247).
    Terminals ``(p, n)``, internal unknown the branch current ``i``; the
    branch equation is ``d/dt sum_e M_de i_e - (v_p - v_n) = 0``.

    Kernel parameter rows: l, sqrt(l), k (k shared by the group)."""

    terminals = ("p", "n")
    n_internal = 1
    internal_names = ("i",)
    fields = ("log_l",)
    static = ("k",)
    local = False
    kind = KIND_COUPLED_L
    has_charges = True

    def __init__(self, nodes, l, k=0.5):
        self.nodes = self._devices(nodes)
        self.log_l = self._log_per_device(l)
        self.k = float(k)

    @property
    def l(self):
        return torch.exp(self.log_l)

    def gpu_params(self):
        l = torch.exp(self.log_l)
        return [l, torch.sqrt(l), torch.full_like(l, self.k)]

    def group_key(self) -> tuple:
        """A coupled block never fuses with another one: each is its own
        mutual-inductance matrix."""
        return (type(self), id(self))


class Diode(Element):
    """Shockley diode (semiconductor.py:27-70): ``i = is (explin(v/(n vt)) - 1)``
    with ``explin`` continuing ``exp`` linearly above 40, ``q = tt i + cj v``,
    ``v = v_anode - v_cathode``.

    Kernel parameter rows: is, 1/(n vt), tt, cj."""

    terminals = ("a", "k")
    fields = ("log_is", "n", "cj", "tt", "vt")
    kind = KIND_DIODE
    has_charges = True

    def __init__(self, nodes, is_=1e-14, n=1.0, cj=0.0, tt=0.0, vt=VT_300K):
        self.nodes = self._devices(nodes)
        self.log_is = self._log_per_device(is_)
        self.n = self._per_device(n)
        self.cj = self._per_device(cj)
        self.tt = self._per_device(tt)
        self.vt = self._per_device(vt)

    def gpu_params(self):
        i_s = torch.exp(self.log_is)
        shape = i_s.shape
        return [i_s, (1.0 / (self.n * self.vt)).expand(shape), self.tt.expand(shape),
                self.cj.expand(shape)]


class VCCS(Element):
    """Voltage-controlled current source (controlled.py:46-60):
    ``i = gm (v_cp - v_cn)`` flowing ``p -> n`` through the source.

    Kernel parameter rows: gm."""

    terminals = ("p", "n", "cp", "cn")
    fields = ("gm",)
    kind = KIND_VCCS

    def __init__(self, nodes, gm):
        self.nodes = self._devices(nodes)
        self.gm = self._per_device(gm)

    def gpu_params(self):
        return [self.gm]


class BJT(Element):
    """Ebers-Moll (transport form) bipolar transistor with Early effect
    (semiconductor.py:73-135); terminals ``(c, b, e)``::

        i_f = is (explin(v_be/vt) - 1),   i_r = is (explin(v_bc/vt) - 1)
        i_c = (i_f - i_r)(1 + v_ce/vaf) - i_r/br,   i_b = i_f/bf + i_r/br
        q_be = tf i_f + cje v_be,   q_bc = tr i_r + cjc v_bc

    PNP mirrors all voltages and currents. Kernel parameter rows: sign, is,
    1/vt, 1/bf, 1/br, 1/vaf, tf, tr, cje, cjc."""

    terminals = ("c", "b", "e")
    fields = ("log_is", "log_bf", "log_br", "inv_vaf", "tf", "tr", "cje", "cjc", "vt")
    static = ("polarity",)
    kind = KIND_BJT
    has_charges = True

    def __init__(self, nodes, polarity: str = "npn", is_=1e-16, bf=100.0, br=1.0,
                 vaf=float("inf"), tf=0.0, tr=0.0, cje=0.0, cjc=0.0, vt=VT_300K):
        if polarity not in ("npn", "pnp"):
            raise ValueError(f"polarity must be 'npn' or 'pnp', got {polarity!r}")
        self.nodes = self._devices(nodes)
        self.polarity = polarity
        self.log_is = self._log_per_device(is_)
        self.log_bf = self._log_per_device(bf)
        self.log_br = self._log_per_device(br)
        self.inv_vaf = self._per_device(1.0 / _t(vaf))
        self.tf, self.tr = self._per_device(tf), self._per_device(tr)
        self.cje, self.cjc = self._per_device(cje), self._per_device(cjc)
        self.vt = self._per_device(vt)

    @property
    def sign(self) -> float:
        return 1.0 if self.polarity == "npn" else -1.0

    def gpu_params(self):
        i_s = torch.exp(self.log_is)
        shape = i_s.shape

        def full(x):
            return _t(x).expand(shape)

        return [full(self.sign), i_s, (1.0 / self.vt).expand(shape),
                torch.exp(-self.log_bf).expand(shape), torch.exp(-self.log_br).expand(shape),
                self.inv_vaf.expand(shape), self.tf.expand(shape), self.tr.expand(shape),
                self.cje.expand(shape), self.cjc.expand(shape)]


class _Linear4(Element):
    """Four-terminal linear controlled source: ``(p, n)`` output port,
    ``(cp, cn)`` control / sense port (controlled.py:1-98)."""

    terminals = ("p", "n", "cp", "cn")

    def gpu_params(self):
        return [getattr(self, self.fields[0])]


class VCVS(_Linear4):
    """Voltage-controlled voltage source (E): ``v_out = gain v_ctrl``; internal
    unknown: the output current (controlled.py:27-43). Kernel row: gain."""

    n_internal = 1
    internal_names = ("i",)
    fields = ("gain",)
    kind = KIND_VCVS

    def __init__(self, nodes, gain):
        self.nodes = self._devices(nodes)
        self.gain = self._per_device(gain)


class CCCS(_Linear4):
    """Current-controlled current source (F): ``i_out = gain i_sense``, the
    sense current through a zero-volt ammeter ``cp -> cn``
    (controlled.py:63-79). Kernel row: gain."""

    n_internal = 1
    internal_names = ("i_sense",)
    fields = ("gain",)
    kind = KIND_CCCS

    def __init__(self, nodes, gain):
        self.nodes = self._devices(nodes)
        self.gain = self._per_device(gain)


class CCVS(_Linear4):
    """Current-controlled voltage source (H): ``v_out = r i_sense``
    (controlled.py:82-98). Kernel row: r."""

    n_internal = 2
    internal_names = ("i", "i_sense")
    fields = ("r",)
    kind = KIND_CCVS

    def __init__(self, nodes, r):
        self.nodes = self._devices(nodes)
        self.r = self._per_device(r)


class Transformer(Element):
    """Two coupled inductors, mutual inductance ``k sqrt(l1 l2)``; terminals
    ``(p1, n1, p2, n2)``, internal unknowns the winding currents
    (passive.py:90-129). Kernel rows: l1, l2, k sqrt(l1 l2)."""

    terminals = ("p1", "n1", "p2", "n2")
    n_internal = 2
    internal_names = ("i1", "i2")
    fields = ("log_l1", "log_l2", "k")
    kind = KIND_XFMR
    has_charges = True

    def __init__(self, nodes, l1, l2, k=1.0):
        self.nodes = self._devices(nodes)
        self.log_l1 = self._log_per_device(l1)
        self.log_l2 = self._log_per_device(l2)
        self.k = self._per_device(k)

    def gpu_params(self):
        l1, l2 = torch.exp(self.log_l1), torch.exp(self.log_l2)
        return [l1, l2, self.k * torch.sqrt(l1 * l2)]


class IdealOpAmp(Element):
    """Ideal op-amp (nullor), terminals ``(inp, inn, out)``: the output
    sources the current ``i_out`` (from ground into ``out``) that enforces
    ``v_inp = v_inn`` (opamp.py:13-32). One unused kernel parameter row."""

    terminals = ("inp", "inn", "out")
    n_internal = 1
    internal_names = ("i_out",)
    fields = ()
    kind = KIND_IDEAL_OPAMP

    def __init__(self, nodes):
        self.nodes = self._devices(nodes)

    def gpu_params(self):
        return [torch.zeros(self.size, dtype=torch.float64)]  # no parameters: one unused row


class OpAmp(Element):
    """Single-pole op-amp macromodel with soft output rails (opamp.py:35-103):
    ``tau dx/dt + x = clip(a0 (v_inp - v_inn))``, ``clip(u) = mid + half
    tanh((u - mid)/half)``, the output driving ``out`` through ``rout``;
    ``tau = a0 / (2 pi gbw)``. Kernel rows: a0, 1/rout, tau, mid, half,
    1/half."""

    terminals = ("inp", "inn", "out")
    n_internal = 1
    internal_names = ("x",)
    fields = ("log_a0", "log_gbw", "log_rout", "vmin", "vmax")
    kind = KIND_OPAMP
    has_charges = True

    def __init__(self, nodes, a0=1e5, gbw=1e6, rout=1.0, vmin=-15.0, vmax=15.0):
        self.nodes = self._devices(nodes)
        self.log_a0 = self._log_per_device(a0)
        self.log_gbw = self._log_per_device(gbw)
        self.log_rout = self._log_per_device(rout)
        self.vmin = self._per_device(vmin)
        self.vmax = self._per_device(vmax)

    def gpu_params(self):
        a0 = torch.exp(self.log_a0)
        shape = a0.shape
        half = (0.5 * (self.vmax - self.vmin)).expand(shape)
        return [a0, torch.exp(-self.log_rout).expand(shape),
                (a0 / (2 * math.pi * torch.exp(self.log_gbw))).expand(shape),
                (0.5 * (self.vmax + self.vmin)).expand(shape), half, 1.0 / half]


class Switch(Element):
    """Voltage-controlled switch, smoothed (switch.py:14-50): terminals
    ``(p, n, cp, cn)``, ``log g = -log roff + sigmoid((v_c - vth)/vwidth)
    log(roff/ron)``. Kernel rows: log roff, log(roff/ron), vth, 1/vwidth."""

    terminals = ("p", "n", "cp", "cn")
    fields = ("log_ron", "log_roff", "vth", "vwidth")
    kind = KIND_SWITCH

    def __init__(self, nodes, ron=1.0, roff=1e9, vth=0.5, vwidth=0.05):
        self.nodes = self._devices(nodes)
        self.log_ron = self._log_per_device(ron)
        self.log_roff = self._log_per_device(roff)
        self.vth = self._per_device(vth)
        self.vwidth = self._per_device(vwidth)

    def gpu_params(self):
        shape = torch.broadcast_shapes(self.log_ron.shape, self.log_roff.shape)
        return [self.log_roff.expand(shape), (self.log_roff - self.log_ron).expand(shape),
                self.vth.expand(shape), (1.0 / self.vwidth).expand(shape)]


ELEMENT_TYPES = (Resistor, Conductance, Capacitor, VoltageSource, CurrentSource,
                 EKVMOSFET, Level1MOSFET, Inductor, Diode, VCCS, BJT, VCVS, CCCS, CCVS,
                 Transformer, IdealOpAmp, OpAmp, Switch)
