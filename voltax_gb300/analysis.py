"""Drop-in for ``voltax.dc`` / ``voltax.transient`` on the GPU
(voltax/analysis.py).

`dc` runs damped Newton with the gmin-stepping fallback
(voltax/analysis.py:208-266, 410-431); `transient` runs backward Euler or
trapezoidal steps, each a Newton solve warm-started from the previous state
(voltax/analysis.py:434-480). The Newton loop, stamping, refactorization and
solves run in ``libvxg.so``; this module only sequences the gmin stages and
packs arguments.

Differentiation: `dc` is differentiable in every element parameter (torch
autograd). The backward pass is the implicit-function adjoint of
voltax/analysis.py:282-288 -- one transposed solve ``J^T lam = g`` at the
root, then the parameter VJP ``-lam^T dF/dp`` on the GPU -- and it reuses the
factors of the Jacobian at the returned root instead of re-forming them.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib as L
from . import autotune
from .runtime import engine_for, stream_ptr
from .symbolic import structure

SPARSE_THRESHOLD = 200


@dataclass(frozen=True)
class Options:
    """Newton settings (voltax/analysis.py:50-89) plus the factorization
    format: ``precision="f64"`` is the plain FP64 form; ``"f32"`` factors in
    FP32 and recovers FP64 accuracy through the FP64 residual: every Newton
    step solves ``J dz = -r(z)`` with the FP32 factors and the FP64 residual
    of the current iterate, i.e. the Newton iteration itself is the
    iterative refinement (measured on the 4096-instance adder: the same
    iteration counts and 8.7e-13 V agreement with the plain form). `refine`
    adds inner refinement sweeps ``dz += J^-1 (b - J dz)`` per solve against
    the FP64 Jacobian values; ``None`` picks 0 for the fused kernel (small
    systems, where a sweep costs as much as a Newton iteration) and 1 for
    the generic engine (large systems, where it saves a refactorization:
    the 100 x 100 grid converges in 2 Newton iterations with it, 3 without).
    Adjoint (transposed) solves always refine, since no Newton loop follows. `solver` is accepted for compatibility: every solve
    uses the supernodal GPU factorization (a circuit of at most ``2 * leaf``
    unknowns is one dense supernode).

    `engine` picks the fused persistent kernel or the generic level kernels;
    with ``"auto"`` and `autotune`, the faster one (and the fused kernel's
    CTA width) is timed per topology and batch size (`autotune.choose`), and
    on the generic engine `autotune` also times each elimination level's
    factor CTA width (`autotune.tune_factor`).
    `block` pins the fused kernel's threads per instance: 64, 128, 256 or 512
    (one CTA per instance), 32 (one warp per instance, several instances per
    CTA; topologies whose supernodes are at most 32 wide), 0: library
    choice."""

    max_steps: int = 100
    rtol: float = 1e-6
    atol: float = 1e-9
    max_dv: float = 1.0
    gmin: float = 1e-12
    gmin_steps: int = 10
    gmin_start: float = 1e-2
    direct_steps: int = 25
    solver: str = "auto"
    sparse_threshold: int = SPARSE_THRESHOLD
    precision: str = "f64"
    refine: int | None = None
    engine: str = "auto"
    block: int = 0
    autotune: bool = True

    def __post_init__(self):
        if self.engine not in ("auto", "fused", "generic"):
            raise ValueError(f"engine must be 'auto', 'fused' or 'generic', got {self.engine!r}")
        if self.solver not in ("auto", "dense", "sparse"):
            raise ValueError("solver must be 'auto', 'dense' or 'sparse', "
                             f"got {self.solver!r}")
        if self.block not in (0, 32, 64, 128, 256, 512):
            raise ValueError(f"block must be 0, 32, 64, 128, 256 or 512, got {self.block!r}")
        if self.precision not in ("f64", "f32"):
            raise ValueError(f"precision must be 'f64' or 'f32', got {self.precision!r}")

    def native(self, max_steps: int | None = None, refine: int | None = None
               ) -> L.NewtonOpts:
        r = refine if refine is not None else (self.refine or 0)
        return L.NewtonOpts(self.max_steps if max_steps is None else max_steps, self.rtol,
                            self.atol, self.max_dv,
                            L.VXG_F32 if self.precision == "f32" else L.VXG_F64,
                            r, self.block)


class Solution:
    """Result of `dc` or `transient` (voltax/analysis.py:92-139).

    ``z``: ``(S,)`` / ``(T, S)`` for one circuit, ``(B, S)`` / ``(B, T, S)``
    for a batch of B instances; ``converged`` and ``iterations`` likewise
    without the state axis.
    """

    def __init__(self, t, z, converged, layout, iterations=None):
        self.t, self.z, self.converged, self.layout = t, z, converged, layout
        self.iterations = iterations

    def v(self, node: str | None = None):
        if node is None:
            return self.z[..., : self.layout.n_nodes]
        idx = self.layout.node(node)
        return torch.zeros(self.z.shape[:-1], dtype=self.z.dtype,
                           device=self.z.device) if idx < 0 else self.z[..., idx]

    def i(self, device: str, which: str | None = None):
        return self.z[..., self.layout.internal(device, which)]

    def check(self) -> "Solution":
        bad = ~(self.converged.bool() & torch.all(torch.isfinite(self.z), dim=-1))
        if bool(torch.any(bad)):
            where = ""
            if bad.ndim and torch.is_tensor(self.t) and self.t.ndim:
                flat = bad.reshape(-1, bad.shape[-1]).any(0) if bad.ndim > 1 else bad
                where = f" at t={float(self.t[int(torch.argmax(flat.int()))])}"
            raise RuntimeError(
                f"Newton did not converge{where}. Common causes: a node without "
                "a DC path to ground, a loop of voltage sources/inductors, or "
                "time steps too coarse for an edge (see docs: Analyses).")
        return self

    def __getitem__(self, name: str):
        if "." in name:
            device, which = name.rsplit(".", 1)
            return self.i(device, which)
        return self.v(name)


# =============================================================================
# Newton through the C ABI
# =============================================================================


class _Call:
    """Arguments shared by the native Newton calls of one analysis."""

    def __init__(self, circuit, options: Options):
        self.c, self.o = circuit, options
        self.st = structure(circuit)
        self.eng = engine_for(self.st, circuit)
        self.B = circuit.batch
        self.params, self.keep, self.rows = self.eng.pack_params(circuit, self.B)
        self.prec = L.VXG_F32 if options.precision == "f32" else L.VXG_F64
        self.ws = self.eng.workspace(self.B, self.prec)
        self.n_inst = self.B * self.eng.n_seg
        dev = self.eng.device
        self.conv = torch.zeros(self.n_inst, dtype=torch.int32, device=dev)
        self.iters = torch.zeros(self.n_inst, dtype=torch.int32, device=dev)
        self.block = options.block
        self.fused = self._use_fused()
        if self.fused and options.engine == "auto" and options.autotune and not options.block:
            engine, self.block = autotune.choose(self)
            self.fused = engine == "fused"
        if not self.fused and options.autotune:
            autotune.tune_factor(self)
        self.refine = options.refine if options.refine is not None else (0 if self.fused else 1)

    def _use_fused(self) -> bool:
        if self.o.engine == "generic":
            return False
        n = C.c_size_t()
        ok = self.eng.lib.vxg_fused_smem(self.eng.handle, self.prec, C.byref(n)) == L.VXG_OK
        if self.o.engine == "fused" and not ok:
            raise L.VxgError("this topology is not eligible for the fused kernel")
        return ok

    def fused_run(self, mode, ts_np, z0, dc_first):
        """One persistent launch: [DC at ts[0]] + one Newton solve per time point."""
        o = self.o
        dev = self.eng.device
        T = len(ts_np)
        ts_d = torch.as_tensor(ts_np, dtype=torch.float64, device=dev)
        gmins = np.concatenate([[o.gmin], np.logspace(np.log10(o.gmin_start),
                                                      np.log10(o.gmin), o.gmin_steps)])
        gm_d = torch.as_tensor(gmins, dtype=torch.float64, device=dev)
        z_out = torch.empty((T, self.B, self.eng.S), dtype=torch.float64, device=dev)
        conv = torch.empty((T, self.B), dtype=torch.int32, device=dev)
        iters = torch.empty((T, self.B), dtype=torch.int32, device=dev)
        nat = o.native(refine=self.refine)
        nat.block = self.block
        L.check(self.eng.lib.vxg_fused_run(
            self.eng.handle, self.B, self.params, mode, T, ts_d.data_ptr(), z0.data_ptr(),
            int(dc_first), gm_d.data_ptr(), o.gmin_steps, o.direct_steps, o.gmin,
            C.byref(nat), z_out.data_ptr(), conv.data_ptr(), iters.data_ptr(), stream_ptr()),
            "vxg_fused_run")
        return z_out, conv, iters

    def newton(self, mode, z, t, t_prev=0.0, z_prev=None, gmin=None, max_steps=None,
               mask=None, factors=None):
        o = self.o.native(max_steps, refine=self.refine)
        gmin_t = None
        gmin_s = self.o.gmin
        if torch.is_tensor(gmin):
            gmin_t = gmin.to(self.eng.device, torch.float64).contiguous()
        elif gmin is not None:
            gmin_s = float(gmin)
        args = (self.eng.handle, self.B, self.params, mode, float(t), float(t_prev),
                None if z_prev is None else z_prev.data_ptr(),
                None if gmin_t is None else gmin_t.data_ptr(), gmin_s, C.byref(o),
                z.data_ptr(), self.conv.data_ptr(), self.iters.data_ptr())
        if mask is None:
            L.check(self.eng.lib.vxg_newton(*args, None if factors is None else
                                            factors.data_ptr(), self.ws.data_ptr(),
                                            stream_ptr()), "vxg_newton")
        else:
            L.check(self.eng.lib.vxg_newton_masked(*args, mask.data_ptr(), self.ws.data_ptr(),
                                                   stream_ptr()), "vxg_newton_masked")
        return self.conv.clone(), self.iters.clone()


def _gmin_stepping(call: _Call, t, guess: torch.Tensor, factors=None):
    """voltax/analysis.py:236-266 for a batch: instances that fail the
    direct attempt run the gmin stages; the others stay frozen."""
    o = call.o
    if call.fused:
        z_out, conv, iters = call.fused_run(L.VXG_MODE_DC, np.array([float(t)]),
                                            guess.contiguous(), True)
        z = z_out[0]
        data = _refactor(call, z, t, factors) if factors is not None else None
        return z, conv[0], iters[0], data
    z = guess.clone()
    conv, iters = call.newton(L.VXG_MODE_DC, z, t, gmin=o.gmin,
                              max_steps=o.direct_steps if o.gmin_steps else None)
    total = iters.clone()
    if o.gmin_steps and not bool(conv.all()):
        failed = (conv == 0).to(torch.int32)
        seg_of = torch.as_tensor(call.eng.tables.seg_of, device=z.device, dtype=torch.long)
        restart = failed.bool().reshape(call.B, -1)[:, seg_of]  # (B, S) per unknown
        z = torch.where(restart, guess, z).contiguous()
        gmins = np.concatenate([[o.gmin], np.logspace(np.log10(o.gmin_start),
                                                      np.log10(o.gmin), o.gmin_steps)])
        for k in range(1, o.gmin_steps + 1):
            conv_k, it_k = call.newton(L.VXG_MODE_DC, z, t, gmin=gmins[k], mask=failed)
            total = total + torch.where(failed.bool(), it_k, torch.zeros_like(it_k))
            conv = torch.where(failed.bool(), conv_k, conv)
    data = None
    if factors is not None:  # factors of J at the returned root (adjoint)
        data = _refactor(call, z, t, factors)
    return z, conv, total, data


def _refactor(call: _Call, z, t, factors):
    eng = call.eng
    data = torch.empty((call.B, eng.nnz), dtype=torch.float64, device=eng.device)
    L.check(eng.lib.vxg_eval(eng.handle, call.B, call.params, z.data_ptr(), float(t), 1.0, 0.0,
                             None, call.o.gmin, None, None, data.data_ptr(), call.ws.data_ptr(),
                             stream_ptr()), "vxg_eval")
    L.check(eng.lib.vxg_factor(eng.handle, call.B, call.prec, data.data_ptr(),
                               factors.data_ptr(), call.ws.data_ptr(), stream_ptr()),
            "vxg_factor")
    return data


class _DCRoot(torch.autograd.Function):
    """z* = root of f(z, t) + gmin v; backward by the implicit function
    theorem with the factors at z*."""

    @staticmethod
    def forward(ctx, call, t, guess, *rows):
        fac = call.eng.factor_buffer(call.B, call.prec)
        z, conv, iters, data = _gmin_stepping(call, t, guess, factors=fac)
        ctx.call, ctx.t, ctx.fac, ctx.data = call, t, fac, data
        ctx.conv, ctx.iters = conv, iters
        ctx.save_for_backward(z)
        ctx.mark_non_differentiable(conv, iters)
        return z, conv, iters

    @staticmethod
    def backward(ctx, gz, _gc, _gi):
        (z,) = ctx.saved_tensors
        call = ctx.call
        eng = call.eng
        gz = gz.contiguous()
        lam = torch.empty_like(gz)
        data = ctx.data if call.prec == L.VXG_F32 else None
        L.check(eng.lib.vxg_solve(eng.handle, call.B, call.prec, ctx.fac.data_ptr(),
                                  None if data is None else data.data_ptr(), gz.data_ptr(),
                                  lam.data_ptr(), 1, max(call.refine, 2) if data is not None
                                  else 0,
                                  call.ws.data_ptr(), stream_ptr()), "vxg_solve")
        grads_out = []
        bufs = []
        for name, rows in zip(eng.tables.group_names, call.rows):
            n = call.c.elements[name].size
            bufs.append(torch.zeros((len(rows), call.B, n), dtype=torch.float64,
                                    device=eng.device))
        ptrs = (C.c_void_p * max(len(bufs), 1))(*[b.data_ptr() for b in bufs])
        L.check(eng.lib.vxg_param_vjp(eng.handle, call.B, call.params, z.data_ptr(),
                                      float(ctx.t), 1.0, 0.0, lam.data_ptr(), ptrs,
                                      stream_ptr()), "vxg_param_vjp")
        for rows, buf in zip(call.rows, bufs):
            for r, row in enumerate(rows):
                g = buf[r]
                g = g.sum(0) if row.ndim == 1 else g
                grads_out.append(g.to(row.device))
        return (None, None, None, *grads_out)


def _flat_rows(call):
    return [row for rows in call.rows for row in rows]


def dc(circuit, t: float = 0.0, guess=None, options: Options = Options()) -> Solution:
    """DC operating point: ``f(z, t) + gmin v = 0`` (voltax/analysis.py:410-431).

    Differentiable in the circuit's parameters (torch autograd)."""
    call = _Call(circuit, options)
    S, B = call.eng.S, call.B
    if guess is None:
        g = torch.zeros((B, S), dtype=torch.float64, device=call.eng.device)
    else:
        g = torch.as_tensor(guess, dtype=torch.float64, device=call.eng.device)
        g = g.reshape(-1, S).expand(B, S).contiguous()
    rows = _flat_rows(call)
    if any(r.requires_grad for r in rows):
        z, conv, iters = _DCRoot.apply(call, float(t), g, *rows)
    else:
        z, conv, iters, _ = _gmin_stepping(call, float(t), g)
    single = circuit.batch == 1
    shape = (call.eng.n_seg,) if call.eng.n_seg > 1 else ()
    conv = conv.reshape(B, *shape).bool()
    iters = iters.reshape(B, *shape)
    if single:
        z, conv, iters = z[0], conv[0], iters[0]
    return Solution(torch.as_tensor(t, dtype=torch.float64), z, conv, circuit.layout, iters)


def _attach_adjoint(call, ts_np, mode, dc_first, options, z_out):
    rows = _flat_rows(call)
    if not any(r.requires_grad for r in rows):
        return z_out
    return _TransientAdjoint.apply(call, ts_np, mode, dc_first, options.gmin, z_out, *rows)


def _param_vjp(call: _Call, z, t, cf, cq, lam):
    """Per group ``(P, B, n)`` of ``-lam^T d(cf f(z, t) + cq q(z))/d rows``."""
    eng = call.eng
    bufs = [torch.zeros((len(rows), call.B, call.c.elements[name].size), dtype=torch.float64,
                        device=eng.device)
            for name, rows in zip(eng.tables.group_names, call.rows)]
    ptrs = (C.c_void_p * max(len(bufs), 1))(*[b.data_ptr() for b in bufs])
    L.check(eng.lib.vxg_param_vjp(eng.handle, call.B, call.params, z.contiguous().data_ptr(),
                                  float(t), float(cf), float(cq), lam.contiguous().data_ptr(),
                                  ptrs, stream_ptr()), "vxg_param_vjp")
    return bufs


class _TransientAdjoint(torch.autograd.Function):
    """Reverse sweep of the implicit-function adjoint over the time steps
    (voltax differentiates its ``lax.scan`` of ``_root`` solves,
    voltax/analysis.py:269-288, 470-477). With R_n the step residual:
    ``J_n^T lam_n = g_n - (dR_{n+1}/dz_n)^T lam_{n+1}`` from the last step
    back (to the DC point when ``ic="dc"``), and
    ``dL/dp = -sum_n lam_n^T dR_n/dp``."""

    @staticmethod
    def forward(ctx, call, ts, mode, dc_first, gmin, z_out, *rows):
        ctx.call, ctx.ts, ctx.mode, ctx.dc_first, ctx.gmin = call, ts, mode, dc_first, gmin
        ctx.save_for_backward(z_out)
        return z_out.clone()

    @staticmethod
    def backward(ctx, gz):
        (z,) = ctx.saved_tensors
        call, ts, trap = ctx.call, ctx.ts, ctx.mode == L.VXG_MODE_TRAP
        eng, B = call.eng, call.B
        f64 = L.VXG_F64
        ws = eng.workspace(B, f64)
        fac = eng.factor_buffer(B, f64)
        data = torch.empty((B, eng.nnz), dtype=torch.float64, device=eng.device)
        tmp = torch.empty((B, eng.S), dtype=torch.float64, device=eng.device)
        gz = gz.contiguous()
        acc = None
        lam_next = None

        def stamp(zn, t, cf, cq, gm):
            L.check(eng.lib.vxg_eval(eng.handle, B, call.params, zn.data_ptr(), float(t),
                                     float(cf), float(cq), None, float(gm), None, None,
                                     data.data_ptr(), ws.data_ptr(), stream_ptr()), "vxg_eval")

        for n in range(len(ts) - 1, -1, -1):
            if n == 0 and not ctx.dc_first:
                break
            zn = z[n].contiguous()
            rhs = gz[n].clone()
            if lam_next is not None:  # - (dR_{n+1}/dz_n)^T lam_{n+1}
                h1 = ts[n + 1] - ts[n]
                stamp(zn, ts[n], 0.5 if trap else 0.0, -1.0 / h1, 0.0)
                L.check(eng.lib.vxg_spmv(eng.handle, B, data.data_ptr(), lam_next.data_ptr(),
                                         tmp.data_ptr(), 1, stream_ptr()), "vxg_spmv")
                rhs -= tmp
            if n == 0:
                cf, cq = 1.0, 0.0
            else:
                h = ts[n] - ts[n - 1]
                cf, cq = (0.5 if trap else 1.0), 1.0 / h
            stamp(zn, ts[n], cf, cq, ctx.gmin)
            L.check(eng.lib.vxg_factor(eng.handle, B, f64, data.data_ptr(), fac.data_ptr(),
                                       ws.data_ptr(), stream_ptr()), "vxg_factor")
            lam = torch.empty_like(rhs)
            L.check(eng.lib.vxg_solve(eng.handle, B, f64, fac.data_ptr(), None, rhs.data_ptr(),
                                      lam.data_ptr(), 1, 0, ws.data_ptr(), stream_ptr()),
                    "vxg_solve")
            parts = [_param_vjp(call, zn, ts[n], cf, cq, lam)]
            if n > 0:
                parts.append(_param_vjp(call, z[n - 1], ts[n - 1], 0.5 if trap else 0.0,
                                        -cq, lam))
            for bufs in parts:
                acc = bufs if acc is None else [a + b for a, b in zip(acc, bufs)]
            lam_next = lam
        grads = []
        for rows, buf in zip(call.rows, acc if acc is not None else
                             [None] * len(call.rows)):
            for r, row in enumerate(rows):
                if buf is None:
                    grads.append(None)
                    continue
                g = buf[r]
                g = g.sum(0) if row.ndim == 1 else g
                grads.append(g.to(row.device))
        return (None, None, None, None, None, None, *grads)


def transient(circuit, ts, ic="dc", method: str = "be",
              options: Options = Options()) -> Solution:
    """Transient analysis on the time grid `ts` (voltax/analysis.py:434-480)."""
    if method not in ("be", "trap"):
        raise ValueError(f"method must be 'be' or 'trap', got {method!r}")
    ts_np = np.ascontiguousarray(np.asarray(ts, dtype=np.float64))
    call = _Call(circuit, options)
    S, B = call.eng.S, call.B
    dev = call.eng.device
    mode = L.VXG_MODE_BE if method == "be" else L.VXG_MODE_TRAP
    if call.fused and (isinstance(ic, Solution) or not isinstance(ic, str) or ic in ("dc", "zero")):
        dc_first = isinstance(ic, str) and ic == "dc"
        if isinstance(ic, Solution):
            z0 = ic.z
        elif isinstance(ic, str):
            z0 = torch.zeros((B, S), dtype=torch.float64, device=dev)
        else:
            z0 = torch.as_tensor(ic, dtype=torch.float64)
        z0 = torch.as_tensor(z0, dtype=torch.float64, device=dev).detach()
        z0 = z0.reshape(-1, S).expand(B, S).contiguous()
        z_out, conv, iters = call.fused_run(mode, ts_np, z0, dc_first)
        conv[0] = 1  # the initial state counts as converged (voltax/analysis.py:479)
        z_out = _attach_adjoint(call, ts_np, mode, dc_first, options, z_out)
        tt = torch.as_tensor(ts_np)
        if circuit.batch == 1:
            return Solution(tt, z_out[:, 0], conv[:, 0].bool(), circuit.layout, iters[:, 0])
        return Solution(tt, z_out.permute(1, 0, 2), conv.T.bool(), circuit.layout, iters.T)
    dc_sol = None
    if isinstance(ic, Solution):
        z0 = ic.z
    elif isinstance(ic, str):
        if ic == "dc":
            dc_sol = dc(circuit, float(ts_np[0]), options=options)
            z0 = dc_sol.z
        elif ic == "zero":
            z0 = torch.zeros((B, S), dtype=torch.float64, device=dev)
        else:
            raise ValueError(f"ic must be 'dc', 'zero' or an array, got {ic!r}")
    else:
        z0 = torch.as_tensor(ic, dtype=torch.float64)
    z0 = torch.as_tensor(z0, dtype=torch.float64, device=dev).detach()
    z0 = z0.reshape(-1, S).expand(B, S).contiguous()
    T = len(ts_np)
    n_inst = call.n_inst
    z_out = torch.empty((T, B, S), dtype=torch.float64, device=dev)
    conv = torch.empty((T, n_inst), dtype=torch.int32, device=dev)
    iters = torch.empty((T, n_inst), dtype=torch.int32, device=dev)
    o = options.native(refine=call.refine)
    L.check(call.eng.lib.vxg_transient(
        call.eng.handle, B, call.params, mode, T, ts_np.ctypes.data_as(L.PF64), z0.data_ptr(),
        options.gmin, C.byref(o), z_out.data_ptr(), conv.data_ptr(), iters.data_ptr(),
        call.ws.data_ptr(), stream_ptr()), "vxg_transient")
    if dc_sol is not None:  # row 0 reports the DC solve, as the fused engine does
        conv[0] = 1
        iters[0] = dc_sol.iterations.reshape(-1).to(torch.int32)
    z_out = _attach_adjoint(call, ts_np, mode, isinstance(ic, str) and ic == "dc", options, z_out)
    tt = torch.as_tensor(ts_np)
    if circuit.batch == 1:
        return Solution(tt, z_out[:, 0], conv[:, 0].bool(), circuit.layout, iters[:, 0])
    return Solution(tt, z_out.permute(1, 0, 2), conv.T.bool(), circuit.layout, iters.T)


# =============================================================================
# Sweeps and time grids
# =============================================================================


def dc_sweep(circuit, values, apply, t: float = 0.0, guess=None,
             options: Options = Options()) -> Solution:
    """DC sweep with continuation (SPICE ``.dc``, voltax/analysis.py:530-568):
    point k starts Newton from point k-1's operating point, so one solution
    branch is followed (hysteresis shows when sweeping up and down).

    `apply` is a source name (its DC value is set) or ``fn(circuit, value)``.
    Returns a `Solution` whose ``t`` holds the sweep values and whose ``z``
    has the sweep axis first. A DC source swept on the fused engine runs the
    whole sweep in one persistent launch (`vxg_fused_sweep`); otherwise each
    point is one Newton launch, warm-started from the previous state left on
    the device."""
    if isinstance(apply, str):
        swept = _device_sweep(circuit, values, apply, t, guess, options)
        if swept is not None:
            return swept
        device = apply
        apply = lambda c, v: c.set(device, value=v)  # noqa: E731
    vals = torch.as_tensor(np.array(values, dtype=np.float64))  # a copy: any strides
    z = guess
    zs, oks, its = [], [], []
    for v in vals:
        sol = dc(apply(circuit, float(v)), t, guess=z, options=options)
        z = sol.z
        zs.append(sol.z)
        oks.append(sol.converged)
        its.append(sol.iterations)
    return Solution(vals, torch.stack(zs), torch.stack(oks), circuit.layout,
                    torch.stack(its))


def _device_sweep(circuit, values, name: str, t, guess, options: Options):
    """`dc_sweep` of the DC value of source `name` in one launch: the fused
    kernel writes each point's value into a private per-instance copy of the
    source group's parameter rows and solves from the previous point. None
    when that path does not apply (not a constant-valued source, the generic
    engine, or a parameter that needs a gradient): the caller then sweeps
    point by point."""
    from .elements import _Source
    from .signals import Constant
    try:
        gname, idx = circuit.layout.device(name)
    except KeyError:
        return None
    el = circuit.elements[gname]
    if not isinstance(el, _Source) or not isinstance(el.value, Constant):
        return None
    vals = np.array(values, dtype=np.float64).reshape(-1)
    if vals.size == 0:
        return None
    call = _Call(circuit, options)
    if not call.fused or any(r.requires_grad for r in _flat_rows(call)):
        return None
    eng, o = call.eng, call.o
    S, B = eng.S, call.B
    dev = eng.device
    gi = eng.tables.group_names.index(gname)
    packed = call.keep[gi]  # (rows, 1 or B, n)
    rows_n, _, n = packed.shape
    own = packed.expand(rows_n, B, n).clone()  # written by the kernel
    call.keep.append(own)
    call.params[gi] = L.GroupParams(own.data_ptr(), B * n, n)
    if guess is None:
        z0 = torch.zeros((B, S), dtype=torch.float64, device=dev)
    else:
        z0 = torch.as_tensor(guess, dtype=torch.float64, device=dev)
        z0 = z0.reshape(-1, S).expand(B, S).contiguous()
    K = vals.size
    vals_d = torch.as_tensor(vals, device=dev)
    gmins = np.concatenate([[o.gmin], np.logspace(np.log10(o.gmin_start), np.log10(o.gmin),
                                                  o.gmin_steps)])
    gm_d = torch.as_tensor(gmins, dtype=torch.float64, device=dev)
    z_out = torch.empty((K, B, S), dtype=torch.float64, device=dev)
    conv = torch.empty((K, B), dtype=torch.int32, device=dev)
    iters = torch.empty((K, B), dtype=torch.int32, device=dev)
    nat = o.native(refine=call.refine)
    nat.block = call.block
    L.check(eng.lib.vxg_fused_sweep(
        eng.handle, B, call.params, gi, 0, idx, K, vals_d.data_ptr(), float(t), z0.data_ptr(),
        gm_d.data_ptr(), o.gmin_steps, o.direct_steps, o.gmin, C.byref(nat), z_out.data_ptr(),
        conv.data_ptr(), iters.data_ptr(), stream_ptr()), "vxg_fused_sweep")
    conv = conv.bool()
    if circuit.batch == 1:
        z_out, conv, iters = z_out[:, 0], conv[:, 0], iters[:, 0]
    return Solution(torch.as_tensor(vals), z_out, conv, circuit.layout, iters)


def time_grid(circuit, t_stop: float, dt_max: float, dt_min: float | None = None,
              ramp_points: int = 10, growth: float = 1.2) -> np.ndarray:
    """A transient time grid refined at the sources' corners
    (voltax/analysis.py:571-620): every waveform breakpoint is a grid point,
    each interval between breakpoints starts with a step of `dt_min`
    (default: the shortest interval / `ramp_points`) that grows by `growth`
    up to `dt_max`, with at least `ramp_points` steps per interval."""
    from .signals import Signal
    corners = [np.array([0.0, t_stop])]
    for el in circuit.elements.values():
        sig = getattr(el, "value", None)
        if isinstance(sig, Signal):
            corners.append(np.asarray(sig.breakpoints(t_stop), dtype=float))
    corners = np.unique(np.concatenate(corners))
    gaps = np.diff(corners)
    gaps = gaps[gaps > 0]
    if dt_min is None:
        dt_min = min(dt_max, gaps.min() / ramp_points) if gaps.size else dt_max
    times = [0.0]
    for a, b in zip(corners[:-1], corners[1:]):
        span = b - a
        step = min(dt_min, span / ramp_points)
        cap = min(dt_max, max(span / ramp_points, dt_min))
        now = a
        while b - now > 1e-9 * step:
            now = min(now + step, b)
            times.append(now)
            step = min(step * growth, cap)
    return np.unique(np.asarray(times))


# =============================================================================
# AC small-signal analysis
# =============================================================================


def linearize(circuit, z, t: float = 0.0):
    """Small-signal matrices ``G = df/dz`` and ``C = dq/dz`` at state `z` as
    dense ``(S, S)`` tensors (voltax/analysis.py:483-491); the stamped sparse
    values come from `sparse.jacobian`."""
    from . import sparse
    st = structure(circuit)
    G = sparse.jacobian(circuit, z, t, 1.0, 0.0, structure=st)
    C = sparse.jacobian(circuit, z, t, 0.0, 1.0, structure=st)
    return sparse.to_dense(st, G), sparse.to_dense(st, C)


class ACSolution:
    """Result of `ac` (voltax/analysis.py:142-178): complex phasors
    ``z`` of shape ``(F, S)`` at the frequencies ``freqs`` (Hz)."""

    def __init__(self, freqs, z, op, layout):
        self.freqs, self.z, self.op, self.layout = freqs, z, op, layout

    def v(self, node: str | None = None):
        if node is None:
            return self.z[..., : self.layout.n_nodes]
        idx = self.layout.node(node)
        if idx < 0:
            return torch.zeros(self.z.shape[:-1], dtype=self.z.dtype, device=self.z.device)
        return self.z[..., idx]

    def i(self, device: str, which: str | None = None):
        return self.z[..., self.layout.internal(device, which)]

    def db(self, node: str):
        """``20 log10 |v(node)|``."""
        return 20 * torch.log10(self.v(node).abs())

    def phase(self, node: str, unwrap: bool = True):
        """Phase of `v(node)` in degrees, unwrapped along frequency."""
        ang = torch.angle(self.v(node)).cpu().numpy()
        if unwrap:
            ang = np.unwrap(ang, axis=0)
        return torch.as_tensor(np.rad2deg(ang))


def ac(circuit, freqs, op: Solution | None = None, options: Options = Options(),
       max_factor_bytes: float = 2e9) -> ACSolution:
    """Small-signal AC analysis around the DC operating point
    (voltax/analysis.py:494-524): solves ``(G + j 2 pi f C) z = -b`` for every
    frequency, ``b`` the sources' ``ac`` / ``ac_phase`` stimulus.

    ``G`` and ``C`` are stamped once at the operating point; the frequencies
    are the batch of one complex factorization + solve launch sequence
    (`vxg_ac_factor` / `vxg_ac_solve`) under the circuit's own plan, in
    chunks whose factors fit `max_factor_bytes`."""
    if circuit.batch != 1:
        raise ValueError("ac() takes one circuit instance")
    op = dc(circuit, options=options) if op is None else op
    st = structure(circuit)
    eng = engine_for(st, circuit)
    from . import sparse
    t0 = float(op.t)
    G = sparse.jacobian(circuit, op.z, t0, 1.0, 0.0, structure=st).contiguous()
    Cq = sparse.jacobian(circuit, op.z, t0, 0.0, 1.0, structure=st).contiguous()
    b = torch.as_tensor(-circuit.ac_stimulus(), dtype=torch.complex128)
    rhs = torch.view_as_real(b).contiguous().to(eng.device)
    f = np.asarray(freqs, dtype=np.float64).reshape(-1)
    omega = torch.as_tensor(2 * np.pi * f, dtype=torch.float64, device=eng.device)
    chunk = max(1, int(max_factor_bytes // max(16 * eng.tables.work, 1)))
    out = []
    for s0 in range(0, len(f), chunk):
        F = min(chunk, len(f) - s0)
        fac = eng.factor_buffer(F, L.VXG_C128)
        ws = eng.workspace(F, L.VXG_C128)
        L.check(eng.lib.vxg_ac_factor(eng.handle, F, G.data_ptr(), Cq.data_ptr(),
                                      omega[s0:s0 + F].data_ptr(), fac.data_ptr(),
                                      ws.data_ptr(), stream_ptr()), "vxg_ac_factor")
        x = torch.empty((F, eng.S, 2), dtype=torch.float64, device=eng.device)
        L.check(eng.lib.vxg_ac_solve(eng.handle, F, fac.data_ptr(), rhs.data_ptr(), 0,
                                     x.data_ptr(), ws.data_ptr(), stream_ptr()), "vxg_ac_solve")
        out.append(torch.view_as_complex(x))
    return ACSolution(torch.as_tensor(f), torch.cat(out), op, circuit.layout)
