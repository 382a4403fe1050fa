"""The launch-shape autotuner: it returns one of its candidates, caches the
choice per (topology, precision, batch size class), writes nothing the
caller owns, and a tuned analysis agrees with every pinned engine/width."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_choice_is_cached_and_results_agree_across_shapes():
    import voltax_gb300 as vx
    from voltax_gb300 import autotune, workloads
    from voltax_gb300.analysis import _Call
    autotune.clear()
    c = workloads.mirror_adder_mc(64, seed=4)
    call = _Call(c, vx.Options(precision="f32"))
    choice = autotune.choose(call)
    assert choice in [("fused", b) for b in autotune.BLOCKS] + [("generic", 0)]
    assert autotune.choose(call) == choice and len(autotune._cache) == 1
    ts = np.linspace(0, 100e-12, 11)
    ref = vx.transient(c, ts, ic="dc", options=vx.Options(precision="f32"))
    for engine, block in [("fused", 32), ("fused", 64), ("fused", 128), ("fused", 256),
                          ("fused", 512), ("generic", 0)]:
        o = vx.Options(precision="f32", engine=engine, block=block)
        s = vx.transient(c, ts, ic="dc", options=o)
        assert bool(s.converged.all())
        assert float((s.z - ref.z).abs().max()) < 1e-11, (engine, block)


def test_fused_block_widths_agree():
    """The CTA width -- or one warp per instance -- changes which threads do
    the work (and, through the level dispatch, thread- or warp-level
    factorization of small supernodes), not the arithmetic: the results
    agree to rounding."""
    import voltax_gb300 as vx
    from voltax_gb300 import workloads
    c = workloads.mirror_adder_mc(8, seed=5)
    ts = np.linspace(0, 50e-12, 6)
    out = [vx.transient(c, ts, ic="dc", options=vx.Options(precision="f32", engine="fused",
                                                            block=b)).z
           for b in (128, 64, 256, 512, 32)]
    for other in out[1:]:
        assert float((out[0] - other).abs().max()) < 1e-12


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_factor_widths_are_tuned_and_change_no_bits(precision):
    """The generic engine's tile-shape tuner: one width per elimination
    level (0 for a level of fixed shape), cached per (topology, precision,
    batch class); and every width gives bitwise the same factors."""
    import ctypes as C
    import torch
    import voltax_gb300 as vx
    from voltax_gb300 import _lib as L
    from voltax_gb300 import autotune, workloads
    from voltax_gb300.analysis import _Call
    from voltax_gb300.runtime import stream_ptr
    autotune.clear()
    c = workloads.power_grid(100)
    call = _Call(c, vx.Options(precision=precision, engine="generic"))
    widths = autotune.tune_factor(call)
    eng = call.eng
    nl = C.c_int32()
    L.check(eng.lib.vxg_level_count(eng.handle, C.byref(nl)), "vxg_level_count")
    assert len(widths) == nl.value > 0
    assert set(widths) <= {0, 128, 256, 512} and any(widths)
    assert autotune.tune_factor(call) == widths and len(autotune._widths) == 1
    z = torch.zeros((1, eng.S), dtype=torch.float64, device=eng.device)
    data = torch.empty((1, eng.nnz), dtype=torch.float64, device=eng.device)
    L.check(eng.lib.vxg_eval(eng.handle, 1, call.params, z.data_ptr(), 0.0, 1.0, 0.0, None,
                             1e-12, None, None, data.data_ptr(), call.ws.data_ptr(),
                             stream_ptr()), "vxg_eval")
    facs = []
    for w in (None, 128, 256, 512):
        arr = None if w is None else (C.c_int32 * nl.value)(*[w if x else 0 for x in widths])
        L.check(eng.lib.vxg_set_factor_shapes(eng.handle, call.prec, arr),
                "vxg_set_factor_shapes")
        fac = eng.factor_buffer(1, call.prec)
        L.check(eng.lib.vxg_factor(eng.handle, 1, call.prec, data.data_ptr(), fac.data_ptr(),
                                   call.ws.data_ptr(), stream_ptr()), "vxg_factor")
        facs.append(fac)
    for other in facs[1:]:
        assert torch.equal(facs[0], other)
    bad = (C.c_int32 * nl.value)(*([96] * nl.value))
    assert eng.lib.vxg_set_factor_shapes(eng.handle, call.prec, bad) == L.VXG_ERR_INVALID
    autotune.clear()
    L.check(eng.lib.vxg_set_factor_shapes(eng.handle, call.prec, None), "vxg_set_factor_shapes")
    s = vx.dc(c, options=vx.Options(precision=precision, engine="generic"))
    assert bool(s.converged.all())
