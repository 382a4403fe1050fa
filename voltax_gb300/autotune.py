"""Launch-shape autotuners for the Newton engines.

Which engine and CTA width run a batched analysis fastest depends on the
topology and the batch: the fused persistent kernel keeps an instance on
one CTA (best when several CTAs fit an SM), the generic level kernels
spread every instance over the whole GPU (best when the fused kernel's
shared-memory footprint leaves one narrow CTA per SM). `choose` times the
candidates -- the fused kernel at 128, 256 and 512 threads per instance
(one CTA each) and the generic engine -- on a few DC Newton iterations of
the caller's own
instances, and keeps the fastest per (topology, precision, batch size
class). Each trial runs on scratch copies; nothing the caller owns is
written.

The choice changes only speed, never the algorithm: every candidate
computes the same Newton iterates up to rounding (the engines agree to
1e-11 relative). For bit-for-bit repeatable results across processes, pin
``Options(engine=..., block=...)``, which bypasses the tuner.

`tune_factor` picks the generic engine's tile shape: the CTA width (128,
256 or 512 threads) of each elimination level's factor kernel, timed level
by level by `vxg_tune_factor` on the Jacobian of the caller's instances,
once per (topology, precision, batch size class). The width changes no sum's
order, so the factors are bitwise those of the built-in size rule.
"""

from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L
from .runtime import stream_ptr

TRIAL_STEPS = 3
TRIAL_INSTANCES = 4096
# The fused kernel with one warp per instance (block 32) or 64 threads per
# instance is not a candidate: a DC trial favours them, but on the
# transients they run slower than 128-thread CTAs (4-bit adder, 4096
# instances: 2.35 M and 2.18 M vs 2.56 M solves/s). Pin them with
# Options(block=32) or Options(block=64).
BLOCKS = (128, 256, 512)

_cache: dict[tuple, tuple[str, int]] = {}
_widths: dict[tuple, tuple[int, ...]] = {}


def _bucket(batch: int) -> int:
    return 1 << max(0, (batch - 1).bit_length())


def _time(fn) -> float:
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fn()  # warm: first-launch attribute setup, caches
    torch.cuda.synchronize()
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def choose(call) -> tuple[str, int]:
    """("fused", block) or ("generic", 0) for this call's topology and batch."""
    key = (call.c.topology_key(), call.prec, _bucket(call.B))
    if key in _cache:
        return _cache[key]
    eng, o = call.eng, call.o
    n = min(call.B, TRIAL_INSTANCES)
    S = eng.S
    dev = eng.device
    z0 = torch.zeros((n, S), dtype=torch.float64, device=dev)
    ts = torch.zeros(1, dtype=torch.float64, device=dev)
    z_out = torch.empty((1, n, S), dtype=torch.float64, device=dev)
    conv = torch.empty(n * eng.n_seg, dtype=torch.int32, device=dev)
    iters = torch.empty(n * eng.n_seg, dtype=torch.int32, device=dev)
    results = {}
    for block in BLOCKS:
        nat = o.native(TRIAL_STEPS)
        nat.block = block

        def fused():
            return eng.lib.vxg_fused_run(
                eng.handle, n, call.params, L.VXG_MODE_DC, 1, ts.data_ptr(), z0.data_ptr(), 1,
                None, 0, TRIAL_STEPS, o.gmin, C.byref(nat), z_out.data_ptr(), conv.data_ptr(),
                iters.data_ptr(), stream_ptr())

        status = fused()
        if status == L.VXG_ERR_TOO_LARGE:  # the warp kernel: a supernode wider than 32
            continue
        L.check(status, "vxg_fused_run")
        ms = _time(fused)
        results[("fused", block)] = ms / max(int(iters.sum()), 1)
    z = torch.empty_like(z0)
    nat = o.native(TRIAL_STEPS)

    def generic():
        z.copy_(z0)
        L.check(eng.lib.vxg_newton(eng.handle, n, call.params, L.VXG_MODE_DC, 0.0, 0.0, None,
                                   None, o.gmin, C.byref(nat), z.data_ptr(), conv.data_ptr(),
                                   iters.data_ptr(), None, call.ws.data_ptr(), stream_ptr()),
                "vxg_newton")

    ms = _time(generic)
    results[("generic", 0)] = ms / max(int(iters.sum()), 1)
    best = min(results, key=results.get)
    _cache[key] = best
    return best


def tune_factor(call) -> tuple[int, ...]:
    """Per-level factor CTA widths (0: fixed shape) for this call's topology,
    precision and batch, set on the call's engine handle."""
    eng = call.eng
    key = (call.c.topology_key(), call.prec, _bucket(call.B))
    applied = eng.__dict__.setdefault("factor_widths_key", {})  # precision -> key held
    widths = _widths.get(key)
    if widths is not None:
        if applied.get(call.prec) != key:
            arr = (C.c_int32 * len(widths))(*widths)
            L.check(eng.lib.vxg_set_factor_shapes(eng.handle, call.prec, arr),
                    "vxg_set_factor_shapes")
            applied[call.prec] = key
        return widths
    n = min(call.B, TRIAL_INSTANCES)
    dev = eng.device
    z = torch.zeros((n, eng.S), dtype=torch.float64, device=dev)
    data = torch.empty((n, eng.nnz), dtype=torch.float64, device=dev)
    ws = call.ws if n == call.B else eng.workspace(n, call.prec)
    fac = eng.factor_buffer(n, call.prec)
    L.check(eng.lib.vxg_eval(eng.handle, n, call.params, z.data_ptr(), 0.0, 1.0, 0.0, None,
                             call.o.gmin, None, None, data.data_ptr(), ws.data_ptr(),
                             stream_ptr()), "vxg_eval")
    nl = C.c_int32()
    L.check(eng.lib.vxg_level_count(eng.handle, C.byref(nl)), "vxg_level_count")
    out = (C.c_int32 * max(nl.value, 1))()
    L.check(eng.lib.vxg_tune_factor(eng.handle, n, call.prec, data.data_ptr(), fac.data_ptr(),
                                    ws.data_ptr(), out, stream_ptr()), "vxg_tune_factor")
    widths = tuple(out[i] for i in range(nl.value))
    _widths[key] = widths
    applied[call.prec] = key
    return widths


def clear() -> None:
    _cache.clear()
    _widths.clear()
