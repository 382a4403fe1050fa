"""Launch-shape autotuner for the Newton engines.

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


def clear() -> None:
    _cache.clear()
