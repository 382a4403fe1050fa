"""Drop-in for ``voltax.sparse`` on the GPU (voltax/sparse.py).

Same names and argument meaning:

* `structure(circuit)` -> `Structure` (cached per topology), ``.plan``
* `jacobian(circuit, z, t, f, q, structure)` -> CSR values of
  ``f df/dz + q dq/dz`` (voltax/sparse.py:220-249)
* `factor(plan, data)` -> `Factors` (voltax/sparse.py:549-572)
* `solve(plan, factors, b, transpose)` (voltax/sparse.py:575-595)
* `spsolve(st, data, b)`, differentiable in ``data`` and ``b`` with the
  adjoint reusing the forward factors (voltax/sparse.py:598-621)

Arrays are float64 torch tensors on the GPU; a leading axis batches
instances that share the pattern. Everything runs in the CUDA kernels of
``libvxg.so``; nothing here computes on the CPU.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib as L
from .runtime import engine_for, stream_ptr, tptr
from .symbolic import (LEAF_SIZE, Plan, Structure, build_structure, make_plan,  # noqa: F401
                       positions, structure)

PRECISIONS = {"f64": L.VXG_F64, "f32": L.VXG_F32}


def _prec(precision) -> int:
    if isinstance(precision, int):
        return precision
    try:
        return PRECISIONS[precision]
    except KeyError:
        raise ValueError(f"precision must be 'f64' or 'f32', got {precision!r}") from None


def _batched(x: torch.Tensor, n: int, what: str):
    """``(B, n)`` view of a ``(n,)`` or ``(B, n)`` tensor, and whether it was 1-D."""
    if x.shape[-1] != n or x.ndim not in (1, 2):
        raise ValueError(f"{what} must have shape ({n},) or (B, {n}), got {tuple(x.shape)}")
    single = x.ndim == 1
    return (x[None] if single else x), single


def _dev(x, eng):
    return torch.as_tensor(x, dtype=torch.float64, device=eng.device).contiguous()


def residual(circuit, z, t=0.0, cf=1.0, cq=0.0) -> torch.Tensor:
    """``cf f(z, t) + cq q(z)`` on the GPU (voltax/circuit.py:196-226)."""
    st = structure(circuit)
    eng = engine_for(st, circuit)
    z = _dev(z, eng)
    zb, single = _batched(z, st.size, "z")
    B = max(zb.shape[0], circuit.batch)
    zb = zb.expand(B, st.size).contiguous()
    params, keep, _ = eng.pack_params(circuit, B)
    ws = eng.workspace(B, L.VXG_F64)
    f = torch.empty_like(zb) if cf != 0 else None
    q = torch.empty_like(zb) if cq != 0 else None
    L.check(eng.lib.vxg_eval(eng.handle, B, params, zb.data_ptr(), float(t), 1.0, 0.0, None,
                             0.0, tptr(f), tptr(q), None, ws.data_ptr(), stream_ptr()),
            "vxg_eval")
    out = torch.zeros_like(zb)
    if f is not None:
        out = out + cf * f
    if q is not None:
        out = out + cq * q
    return out[0] if single and B == 1 else out


def jacobian(circuit, z, t=0.0, f=1.0, q=0.0, structure: Structure | None = None,
             gmin: float = 0.0) -> torch.Tensor:
    """Stamped values of ``f df/dz + q dq/dz`` at state `z` and time `t`
    on `structure`'s pattern (plus `gmin` on node diagonals)."""
    from .symbolic import structure as _structure_of
    st = _structure_of(circuit) if structure is None else structure
    eng = engine_for(st, circuit)
    z = _dev(z, eng)
    zb, single = _batched(z, st.size, "z")
    B = max(zb.shape[0], circuit.batch)
    zb = zb.expand(B, st.size).contiguous()
    params, keep, _ = eng.pack_params(circuit, B)
    ws = eng.workspace(B, L.VXG_F64)
    data = torch.empty((B, st.nnz), dtype=torch.float64, device=eng.device)
    L.check(eng.lib.vxg_eval(eng.handle, B, params, zb.data_ptr(), float(t), float(f),
                             float(q), None, float(gmin), None, None, data.data_ptr(),
                             ws.data_ptr(), stream_ptr()), "vxg_eval")
    return data[0] if single and B == 1 else data


class Factors:
    """Numeric factors of a batch of matrices on one plan (opaque; per
    supernode W = F11^-1, Ub = W F12, Lb = F21 W in unpadded panels)."""

    def __init__(self, engine, precision: int, batch: int, buffer: torch.Tensor, data):
        self.engine, self.precision, self.batch = engine, precision, batch
        self.buffer, self.data = buffer, data


def _engine_of(plan_or_st):
    if isinstance(plan_or_st, Structure):
        return engine_for(plan_or_st)
    st = getattr(plan_or_st, "structure", None)
    if st is None:
        raise TypeError("factor/solve need a Plan from make_plan / Structure.plan "
                        "or the Structure itself")
    return engine_for(st, plan=plan_or_st)


def factor(plan, data, precision="f64") -> Factors:
    """Refactor the matrix with pattern values `data` ((nnz,) or (B, nnz))."""
    eng = _engine_of(plan)
    p = _prec(precision)
    data = _dev(data, eng)
    db, _ = _batched(data, eng.nnz, "data")
    B = db.shape[0]
    buf = eng.factor_buffer(B, p)
    ws = eng.workspace(B, p)
    L.check(eng.lib.vxg_factor(eng.handle, B, p, db.data_ptr(), buf.data_ptr(), ws.data_ptr(),
                               stream_ptr()), "vxg_factor")
    return Factors(eng, p, B, buf, db)


def solve(plan, factors: Factors, b, transpose: bool = False, refine: int = 2):
    """``A x = b`` (or ``A^T x = b``) with `factor`'s output. With FP32
    factors, `refine` FP64 refinement sweeps follow."""
    eng = factors.engine
    b = _dev(b, eng)
    bb, single = _batched(b, eng.S, "b")
    B = factors.batch
    bb = bb.expand(B, eng.S).contiguous()
    x = torch.empty_like(bb)
    ws = eng.workspace(B, factors.precision)
    L.check(eng.lib.vxg_solve(eng.handle, B, factors.precision, factors.buffer.data_ptr(),
                              factors.data.data_ptr(), bb.data_ptr(), x.data_ptr(),
                              int(bool(transpose)),
                              refine if factors.precision == L.VXG_F32 else 0,
                              ws.data_ptr(), stream_ptr()), "vxg_solve")
    return x[0] if single and B == 1 else x


def to_dense(st: Structure, data) -> torch.Tensor:
    """Dense ``(..., S, S)`` matrix of CSR values on `st`'s pattern
    (voltax/sparse.py:135-140)."""
    data = torch.as_tensor(data)
    rows = torch.as_tensor(np.repeat(np.arange(st.size), np.diff(st.indptr)),
                           device=data.device)
    cols = torch.as_tensor(np.asarray(st.indices), device=data.device)
    out = torch.zeros((*data.shape[:-1], st.size, st.size), dtype=data.dtype,
                      device=data.device)
    out[..., rows, cols] = data
    return out


def matvec(st: Structure, data, x):
    """``A @ x`` (voltax/sparse.py:130-133)."""
    eng = engine_for(st)
    data = _dev(data, eng)
    x = _dev(x, eng)
    db, single = _batched(data, st.nnz, "data")
    xb, _ = _batched(x, st.size, "x")
    B = max(db.shape[0], xb.shape[0])
    db = db.expand(B, st.nnz).contiguous()
    xb = xb.expand(B, st.size).contiguous()
    y = torch.empty_like(xb)
    L.check(eng.lib.vxg_spmv(eng.handle, B, db.data_ptr(), xb.data_ptr(), y.data_ptr(), 0,
                             stream_ptr()), "vxg_spmv")
    return y[0] if single and B == 1 else y


class _SpSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, data, b, st, precision):
        fac = factor(st, data, precision)
        x = solve(st, fac, b)
        ctx.fac, ctx.st = fac, st
        ctx.save_for_backward(x)
        return x

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        fac, st = ctx.fac, ctx.st
        eng = fac.engine
        gb = solve(st, fac, g.contiguous(), transpose=True)
        gbb, _ = _batched(gb, st.size, "g")
        xb, _ = _batched(x, st.size, "x")
        B = fac.batch
        gdata = torch.empty((B, st.nnz), dtype=torch.float64, device=eng.device)
        L.check(eng.lib.vxg_spsolve_gdata(eng.handle, B, gbb.contiguous().data_ptr(),
                                          xb.contiguous().data_ptr(), gdata.data_ptr(),
                                          stream_ptr()), "vxg_spsolve_gdata")
        if fac.data.shape[0] == 1 and ctx.needs_input_grad[0]:
            gdata = gdata.reshape(-1) if x.ndim == 1 else gdata
        return gdata, gb, None, None


def spsolve(st: Structure, data, b, precision="f64"):
    """``x = A^-1 b``, differentiable in `data` and `b` (one transposed solve
    with the forward factors)."""
    return _SpSolve.apply(data, b, st, precision)
