"""ctypes wrapper of ``cvx.c``, the compiled CPU restatement used as the
timed CPU baseline (TEST INFRASTRUCTURE; see oracle/__init__.py).

`CSystem(circuit, st, plan, b)` flattens one circuit instance (kernel
parameter rows of instance ``b``, stamp positions, the supernodal plan) and
`run` executes DC + transient on one CPU thread. ctypes releases the GIL
during the call, so several `CSystem`s can run in parallel threads.
"""

from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libcvx.so"


def build() -> Path:
    LIB.parent.mkdir(exist_ok=True)
    src = HERE / "cvx.c"
    if not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["gcc", "-O3", "-std=c11", "-shared", "-fPIC", "-o", str(LIB), str(src),
                        "-lm"], check=True)
    return LIB


class Group(C.Structure):
    _fields_ = [("kind", C.c_int), ("n", C.c_int), ("T", C.c_int), ("K", C.c_int),
                ("wave", C.c_int), ("n_params", C.c_int), ("int_offset", C.c_int),
                ("nodes", C.c_void_p), ("params", C.c_void_p), ("jpos", C.c_void_p)]


class Sys(C.Structure):
    _fields_ = [("S", C.c_int), ("nv", C.c_int), ("nnz", C.c_int), ("n_groups", C.c_int),
                ("groups", C.POINTER(Group)), ("indptr", C.c_void_p), ("indices", C.c_void_p),
                ("rows", C.c_void_p), ("n_sn", C.c_int), ("k", C.c_void_p), ("r", C.c_void_p),
                ("panel", C.c_void_p), ("piv_ptr", C.c_void_p), ("piv", C.c_void_p),
                ("bord_ptr", C.c_void_p), ("bord", C.c_void_p), ("a_pos", C.c_void_p),
                ("work", C.c_longlong), ("schur_ptr", C.c_void_p), ("schur_tgt", C.c_void_p)]


class Opts(C.Structure):
    _fields_ = [("max_steps", C.c_int), ("rtol", C.c_double), ("atol", C.c_double),
                ("max_dv", C.c_double), ("gmin", C.c_double), ("gmin_steps", C.c_int),
                ("direct_steps", C.c_int), ("gmins", C.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        _lib.cvx_run.argtypes = [C.POINTER(Sys), C.POINTER(Opts), C.c_int, C.c_int, C.c_void_p,
                                 C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.cvx_run.restype = C.c_int
        _lib.cvx_check.argtypes = [C.POINTER(Sys), C.POINTER(Opts), C.c_int, C.c_int,
                                   C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        _lib.cvx_check.restype = C.c_int
    return _lib


KINDS = {"Resistor": 0, "Conductance": 0, "Capacitor": 1, "VoltageSource": 2,
         "CurrentSource": 3, "EKVMOSFET": 4, "Level1MOSFET": 5, "Diode": 6, "Inductor": 7,
         "VCCS": 8, "BJT": 9, "VCVS": 10, "CCCS": 11, "CCVS": 12, "Transformer": 13,
         "IdealOpAmp": 14, "OpAmp": 15, "Switch": 16}
WAVES = {"Constant": 0, "Step": 1, "Pulse": 2}


def _rows_of(el, b):
    """Kernel parameter rows of instance ``b`` (physical values, float64)."""
    import torch
    name = type(el).__name__

    def inst(x):
        x = torch.as_tensor(x, dtype=torch.float64).detach().cpu()
        return x[b] if x.ndim == 2 else x

    n = el.size
    if name == "Resistor":
        return [torch.exp(-inst(el.log_r))]
    if name == "Conductance":
        th = inst(el.theta)
        g = {"log": lambda: torch.exp(th),
             "softplus": lambda: el.g_min + torch.logaddexp(th, torch.zeros_like(th)),
             "sigmoid": lambda: el.g_min + (el.g_max - el.g_min) * torch.sigmoid(th),
             "linear": lambda: th}[el.transform]()
        return [g]
    if name == "Capacitor":
        return [torch.exp(inst(el.log_c))]
    if name in ("VoltageSource", "CurrentSource"):
        return [inst(getattr(el.value, f)).expand(n) for f in el.value.fields]
    if name == "EKVMOSFET":
        p = el.process
        w, l = torch.exp(inst(el.log_w)), torch.exp(inst(el.log_l))
        nn, vt = torch.as_tensor(p.n).double(), torch.as_tensor(p.vt).double()
        kp = torch.exp(torch.as_tensor(p.log_kp).double())
        sign = 1.0 if el.polarity == "n" else -1.0
        i_spec = 2 * nn * kp * (w / l) * vt ** 2
        full = lambda x: torch.as_tensor(x, dtype=torch.float64).expand(n)  # noqa: E731
        return [full(sign), i_spec, full(p.vth), inst(el.dvth).expand(n), full(nn), full(vt),
                full(p.lam), torch.exp(torch.as_tensor(p.log_cox).double()) * w * l,
                torch.exp(torch.as_tensor(p.log_cov).double()) * w]
    if name == "Diode":
        full = lambda x: inst(x).expand(n)  # noqa: E731
        return [torch.exp(full(el.log_is)), 1.0 / (full(el.n) * full(el.vt)), full(el.tt),
                full(el.cj)]
    if name == "Inductor":
        return [torch.exp(inst(el.log_l)).expand(n), inst(el.rs).expand(n)]
    if name == "VCCS":
        return [inst(el.gm).expand(n)]
    if name == "IdealOpAmp":
        return [torch.zeros(n, dtype=torch.float64)]
    if name == "OpAmp":
        import math
        full = lambda x: inst(x).expand(n)  # noqa: E731
        a0 = torch.exp(full(el.log_a0))
        half = 0.5 * (full(el.vmax) - full(el.vmin))
        return [a0, torch.exp(-full(el.log_rout)), a0 / (2 * math.pi * torch.exp(full(el.log_gbw))),
                0.5 * (full(el.vmax) + full(el.vmin)), half, 1.0 / half]
    if name == "Switch":
        full = lambda x: inst(x).expand(n)  # noqa: E731
        return [full(el.log_roff), full(el.log_roff) - full(el.log_ron), full(el.vth),
                1.0 / full(el.vwidth)]
    if name in ("VCVS", "CCCS"):
        return [inst(el.gain).expand(n)]
    if name == "CCVS":
        return [inst(el.r).expand(n)]
    if name == "Transformer":
        l1, l2 = torch.exp(inst(el.log_l1)).expand(n), torch.exp(inst(el.log_l2)).expand(n)
        return [l1, l2, inst(el.k).expand(n) * torch.sqrt(l1 * l2)]
    if name == "BJT":
        full = lambda x: inst(x).expand(n)  # noqa: E731
        sign = 1.0 if el.polarity == "npn" else -1.0
        return [torch.full((n,), sign, dtype=torch.float64), torch.exp(full(el.log_is)),
                1.0 / full(el.vt), torch.exp(-full(el.log_bf)), torch.exp(-full(el.log_br)),
                full(el.inv_vaf), full(el.tf), full(el.tr), full(el.cje), full(el.cjc)]
    if name == "Level1MOSFET":  # voltax/elements/mosfet.py:208-257
        p = el.process
        w, l = torch.exp(inst(el.log_w)), torch.exp(inst(el.log_l))
        kp = torch.exp(torch.as_tensor(p.log_kp).double())
        sign = 1.0 if el.polarity == "n" else -1.0
        full = lambda x: torch.as_tensor(x, dtype=torch.float64).expand(n)  # noqa: E731
        return [full(sign), kp * (w / l), full(p.vth), inst(el.dvth).expand(n), full(p.lam),
                full(p.gamma), full(p.phi), full(float(el.smooth)),
                torch.exp(torch.as_tensor(p.log_cov).double()) * w]
    raise NotImplementedError(name)


def schur_targets(plan, S):
    """Per supernode, the r x r panel positions of its border x border block
    (the targets of voltax/sparse.py:514-527 in the unpadded layout)."""
    k, r, panel = plan.k, plan.r, plan.panel
    sn_of, pos_in = plan.sn_of, plan.pos_in
    bkeys = np.concatenate([np.int64(i) * S + np.asarray(b, np.int64)
                            for i, b in enumerate(plan.borders)])
    bidx = np.concatenate([np.arange(len(b)) for b in plan.borders])
    order = np.argsort(bkeys)
    bkeys, bidx = bkeys[order], bidx[order]

    def position(u, v):
        su, sv = sn_of[u], sn_of[v]
        out = np.empty(u.shape, np.int64)
        same = su == sv
        out[same] = panel[su[same]] + pos_in[u[same]] * k[su[same]] + pos_in[v[same]]
        up = su < sv
        o = su[up]
        out[up] = panel[o] + k[o] * k[o] + pos_in[u[up]] * r[o] + \
            bidx[np.searchsorted(bkeys, np.asarray(o, np.int64) * S + np.asarray(v[up], np.int64))]
        lo = su > sv
        o = sv[lo]
        out[lo] = panel[o] + k[o] * k[o] + k[o] * r[o] + \
            bidx[np.searchsorted(bkeys, np.asarray(o, np.int64) * S + np.asarray(u[lo], np.int64))] * k[o] + \
                pos_in[v[lo]]
        return out

    ptr, tg = [0], []
    for b in plan.borders:
        if len(b):
            u, v = np.broadcast_arrays(b[:, None], b[None, :])
            tg.append(position(u.ravel(), v.ravel()))
        ptr.append(ptr[-1] + len(b) * len(b))
    return (np.asarray(ptr, np.int64),
            np.concatenate(tg).astype(np.int64) if tg else np.zeros(0, np.int64))


class CSystem:
    """One circuit instance flattened for ``cvx_run``."""

    def __init__(self, circuit, st, plan, b: int = 0):
        self._keep = []
        keep = self._keep.append

        def arr(x, dt):
            a = np.ascontiguousarray(x, dtype=dt)
            keep(a)
            return a.ctypes.data

        self.S = st.size
        groups = (Group * len(st.devices))()
        for gi, ((name, allv, T, local), (_, pos, _)) in enumerate(zip(st.devices, st.stamps)):
            el = circuit.elements[name]
            rows = _rows_of(el, b)
            n, m = allv.shape
            K = m - T
            off = [o for g, _, _, o in circuit.layout.groups if g == name][0]
            wave = WAVES[type(el.value).__name__] if hasattr(el, "value") else -1
            prm = np.stack([np.asarray(r, np.float64).reshape(n) for r in rows])
            groups[gi] = Group(KINDS[type(el).__name__], n, T, K, wave, len(rows), off,
                               arr(allv[:, :T], np.int32), arr(prm, np.float64),
                               arr(pos.reshape(n, m * m), np.int32))
        keep(groups)
        sp, stg = schur_targets(plan, st.size)
        s = Sys()
        s.S, s.nv, s.nnz, s.n_groups = st.size, st.n_nodes, st.nnz, len(st.devices)
        s.groups = groups
        s.indptr = arr(st.indptr, np.int64)
        s.indices = arr(st.indices, np.int32)
        s.rows = arr(st.rows, np.int32)
        s.n_sn = len(plan.k)
        s.k, s.r = arr(plan.k, np.int32), arr(plan.r, np.int32)
        s.panel = arr(plan.panel, np.int64)
        s.piv_ptr = arr(np.concatenate([[0], np.cumsum(plan.k)]), np.int64)
        s.piv = arr(np.concatenate(plan.supernodes), np.int32)
        s.bord_ptr = arr(np.concatenate([[0], np.cumsum(plan.r)]), np.int64)
        s.bord = arr(np.concatenate(plan.borders), np.int32)
        s.a_pos = arr(plan.a_pos, np.int64)
        s.work = int(plan.work)
        s.schur_ptr, s.schur_tgt = arr(sp, np.int64), arr(stg, np.int64)
        self.sys = s

    def run(self, ts, z0=None, method="be", dc_first=True, max_steps=100, rtol=1e-6,
            atol=1e-9, max_dv=1.0, gmin=1e-12, gmin_steps=10, gmin_start=1e-2,
            direct_steps=25):
        ts = np.ascontiguousarray(np.atleast_1d(np.asarray(ts, np.float64)))
        z0 = np.zeros(self.S) if z0 is None else np.ascontiguousarray(z0, np.float64)
        gm = np.ascontiguousarray(np.concatenate(
            [[gmin], np.logspace(np.log10(gmin_start), np.log10(gmin), gmin_steps)]))
        o = Opts(max_steps, rtol, atol, max_dv, gmin, gmin_steps, direct_steps,
                 gm.ctypes.data)
        n_t = len(ts)
        z_out = np.zeros((n_t, self.S))
        conv = np.zeros(n_t, np.int32)
        iters = np.zeros(n_t, np.int32)
        mode = {"dc": 0, "be": 1, "trap": 2}[method]
        rc = lib().cvx_run(C.byref(self.sys), C.byref(o), mode, n_t, ts.ctypes.data,
                           z0.ctypes.data, int(dc_first), z_out.ctypes.data, conv.ctypes.data,
                           iters.ctypes.data)
        if rc:
            raise MemoryError("cvx_run could not allocate its workspace")
        return z_out, conv.astype(bool), iters

    def check(self, ts, z_traj, method="be", dc_first=True, rtol=1e-6, atol=1e-9,
              gmin=1e-12):
        """Acceptance of a trajectory computed elsewhere: per time point the
        largest FP64 residual entry |r(z_n)| (the KCL residual, in A on node
        rows) and the largest |dz_i| / (atol + rtol |z_i|) of one more
        Newton step from z_n (<= 1: voltax's convergence test passes,
        voltax/analysis.py:224-229). Point 0 is checked as a DC solve when
        `dc_first`, else skipped (an initial condition)."""
        ts = np.ascontiguousarray(np.atleast_1d(np.asarray(ts, np.float64)))
        z = np.ascontiguousarray(np.asarray(z_traj, np.float64).reshape(len(ts), self.S))
        o = Opts(100, rtol, atol, 1.0, gmin, 0, 0, None)
        kcl = np.zeros(len(ts))
        ratio = np.zeros(len(ts))
        mode = {"dc": 0, "be": 1, "trap": 2}[method]
        rc = lib().cvx_check(C.byref(self.sys), C.byref(o), mode, len(ts), ts.ctypes.data,
                             z.ctypes.data, int(dc_first), kcl.ctypes.data, ratio.ctypes.data)
        if rc:
            raise MemoryError("cvx_check could not allocate its workspace")
        return kcl, ratio
