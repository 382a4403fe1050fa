"""Learned warm start: the MLP kernels against the float64 oracle
(oracle/mlp.py, which rounds to bfloat16 where the kernels store BF16), and
what the trained network gains over Newton from the default guess."""

import numpy as np
import pytest
import torch

from oracle import mlp as om

pytestmark = pytest.mark.gpu


def _model(n_in=64, hidden=96, n_out=37, seed=3):
    from voltax_gb300.warmstart import WarmStartMLP
    m = WarmStartMLP(n_in, n_out, hidden=hidden, seed=seed)
    rng = np.random.default_rng(seed + 1)
    X = rng.normal(size=(300, n_in)) * rng.uniform(0.5, 2.0, n_in) + rng.normal(size=n_in)
    V = rng.normal(size=(300, n_out)) * rng.uniform(0.1, 1.0, n_out)
    m.set_normalization(X, V)
    # nonzero biases, so the bias paths are exercised
    for i, (ow, ob) in enumerate(m.offsets):
        n = m.dims[i + 1]
        m.w[ob:ob + n] = torch.as_tensor(rng.normal(size=n) * 0.1, dtype=torch.float32)
    L = m.lib
    assert L.vxg_mlp_adam(m.n_params, m.w.data_ptr(), m.wb.data_ptr(), None, None, None, 0.0,
                          0.0, 0.0, 0.0, 0, torch.cuda.current_stream().cuda_stream) == 0
    return m, X, V


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_forward_loss_and_gradients_match_oracle():
    m, X, V = _model()
    rows_np = np.random.default_rng(7).permutation(300)[:150]  # M = 150: ragged tiles
    x = torch.as_tensor(X, dtype=torch.float64, device="cuda")
    T = ((torch.as_tensor(V) - m.y_mean.double().cpu()) / m.y_std.double().cpu()).float()
    t = T.cuda().contiguous()
    rows = torch.as_tensor(rows_np, dtype=torch.int64, device="cuda")
    M = len(rows_np)
    b = m._buffers(M, True)
    m._forward(x, rows, b, M, train=True)
    from voltax_gb300.runtime import stream_ptr
    assert m.lib.vxg_mlp_mse(M, m.dims[-1], b["y"].data_ptr(), t.data_ptr(), rows.data_ptr(),
                             b["dy"].data_ptr(), m.loss.data_ptr(), m._scratch.data_ptr(),
                             stream_ptr()) == 0
    m.backward(b, M)
    torch.cuda.synchronize()

    layers = m.layers()
    xb = om.normalize(X[rows_np], m.x_mean.cpu().numpy(), m.x_istd.cpu().numpy())
    np.testing.assert_array_equal(b["x"].float().cpu().numpy(), xb)  # same rounding, bitwise
    cache = om.forward(layers, xb)
    y = b["y"].cpu().numpy()
    assert _rel(y, cache["y"]) < 5e-3
    loss, dy = om.mse(cache["y"], T.numpy()[rows_np].astype(np.float64))
    assert abs(float(m.loss) - loss) <= 1e-2 * loss
    grads = om.backward(layers, cache, dy)
    for (gw, gb), (rw, rb) in zip(m.grads(), grads):
        assert _rel(gw, rw) < 2e-2, _rel(gw, rw)
        assert _rel(gb, rb) < 2e-2, _rel(gb, rb)


def test_adam_matches_oracle():
    m, _, _ = _model(n_in=16, hidden=64, n_out=9)
    rng = np.random.default_rng(11)
    g = rng.normal(size=m.n_params).astype(np.float32)
    m.g.copy_(torch.as_tensor(g))
    w0 = m.w.cpu().numpy().astype(np.float64)
    mm, vv = np.zeros(m.n_params), np.zeros(m.n_params)
    w = w0
    from voltax_gb300.runtime import stream_ptr
    for step in (1, 2, 3):
        assert m.lib.vxg_mlp_adam(m.n_params, m.w.data_ptr(), m.wb.data_ptr(), m.g.data_ptr(),
                                  m.m.data_ptr(), m.v.data_ptr(), 1e-3, 0.9, 0.999, 1e-8, step,
                                  stream_ptr()) == 0
        w, mm, vv = om.adam(w, g.astype(np.float64), mm, vv, step, 1e-3)
    torch.cuda.synchronize()
    np.testing.assert_allclose(m.w.cpu().numpy(), w, rtol=1e-5, atol=1e-6)
    np.testing.assert_array_equal(m.wb.float().cpu().numpy(), om.bf16(m.w.cpu().numpy()))


def _fit_smooth(seed):
    from voltax_gb300.warmstart import WarmStartMLP
    rng = np.random.default_rng(0)
    X = rng.normal(size=(4096, 8))
    A = rng.normal(size=(8, 5)) / 3
    V = np.sin(X @ A) + 0.1 * (X[:, :5] ** 2)
    m = WarmStartMLP(8, 5, hidden=64, seed=seed)
    hist = m.fit(X, V, epochs=15, batch=256, lr=3e-3, lr_final=1e-4, seed=seed)
    return m, hist


def test_training_reduces_loss_and_is_reproducible():
    m1, h1 = _fit_smooth(0)
    assert h1[-1] < 0.1 * h1[0], h1
    m2, h2 = _fit_smooth(0)
    assert h1 == h2
    assert torch.equal(m1.w, m2.w)  # fixed-order reductions: same bits


@pytest.fixture(scope="module")
def ota_setup():
    from voltax_gb300 import analysis, warmstart, workloads
    base = workloads.ota_chain(stages=8)
    make = lambda P: workloads.apply_ota_params(base, P)  # noqa: E731
    opts = analysis.Options(engine="generic")
    Xtr = workloads.ota_params(4000, seed=1)
    Vtr, conv, _ = warmstart.solve_dataset(make, Xtr, chunk=2000, options=opts)
    assert bool(conv.all())
    model = warmstart.WarmStartMLP(Xtr.shape[1], Vtr.shape[1], hidden=128, seed=0)
    hist = model.fit(Xtr, Vtr.cpu().numpy(), epochs=40, batch=256, lr=3e-3, lr_final=3e-5)
    assert hist[-1] < 0.05 * hist[0]
    Xte = workloads.ota_params(300, seed=2)
    return base, make, model, Xte, opts


@pytest.mark.parametrize("engine", ["generic", "auto"])
def test_warm_start_halves_newton_iterations(ota_setup, engine):
    from voltax_gb300 import analysis, warmstart
    base, make, model, Xte, _ = ota_setup
    opts = analysis.Options(engine=engine)
    c = make(Xte)
    ref = analysis.dc(c, options=opts)
    warm = warmstart.dc(c, Xte, model, options=opts)
    assert bool(ref.converged.all()) and bool(warm.converged.all())
    it_ref = ref.iterations.double().mean().item()
    it_warm = warm.iterations.double().mean().item()
    assert 2 * it_warm <= it_ref, (it_warm, it_ref)
    nv = c.layout.n_nodes
    v_ref, v_warm = ref.z[:, :nv], warm.z[:, :nv]
    scale = v_ref.abs().amax(1, keepdim=True)
    assert float(((v_warm - v_ref).abs() / scale).max()) <= 1e-9


def test_fallback_to_default_guess(ota_setup):
    """A network that predicts nonsense (40 V everywhere) fails the direct
    attempt on every instance; the plain path from zeros takes over."""
    from voltax_gb300 import analysis, warmstart
    base, make, model, Xte, opts = ota_setup
    X = Xte[:64]
    c = make(X)
    saved = model.y_mean.clone()
    try:
        model.y_mean.fill_(40.0)
        warm = warmstart.dc(c, X, model, options=opts)
    finally:
        model.y_mean.copy_(saved)
    ref = analysis.dc(c, options=opts)
    assert bool(warm.converged.all())
    assert torch.equal(warm.iterations, ref.iterations + opts.direct_steps)
    nv = c.layout.n_nodes
    assert float((warm.z[:, :nv] - ref.z[:, :nv]).abs().max()) <= 1e-12
