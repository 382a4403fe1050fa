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
