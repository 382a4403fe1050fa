"""The XLA FFI drop-in (voltax_gb300/xla.py over csrc/vxg_xla.cc).

Without jax (this container and, so far, the GPU hosts) the module must
import and report itself unavailable, and the shim's handlers must name the
C entry points they forward to. Where jax with jax.ffi is installed, the GPU
test runs spsolve through XLA custom calls and its custom VJP against the
torch path and dense linear algebra.
"""

import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_module_imports_and_reports_availability():
    from voltax_gb300 import xla
    try:
        import jax  # noqa: F401
        has_jax = True
    except ImportError:
        has_jax = False
    if not has_jax:
        assert xla.available() is False
    assert xla.TARGETS == ("vxg_eval", "vxg_factor", "vxg_solve")


def test_shim_forwards_to_declared_entry_points():
    src = (ROOT / "voltax_gb300" / "csrc" / "vxg_xla.cc").read_text()
    header = (ROOT / "include" / "vxg.h").read_text()
    for name in ("vxg_eval", "vxg_factor", "vxg_solve"):
        assert re.search(rf"\b{name}\(", src), name
        assert re.search(rf"XLA_FFI_DEFINE_HANDLER_SYMBOL\({name}_ffi,", src), name
        assert re.search(rf"\bint {name}\(", header), name


@pytest.mark.gpu
def test_spsolve_through_xla_matches_dense_and_gradient():
    jax = pytest.importorskip("jax")
    import jax.numpy as jnp
    from voltax_gb300 import symbolic, workloads, xla
    if not xla.available():
        pytest.skip("libvxg_xla.so not built (no jax FFI headers)")
    jax.config.update("jax_enable_x64", True)
    from oracle import stamp as ost
    c = workloads.power_grid(8, seed=3)
    st = symbolic.structure(c)
    topo = xla.Topology(c, st, st.plan)
    A = ost.add_gmin(ost.jacobian(c, st, np.zeros(c.size), 0.0), st, c.n_nodes, 1e-12)
    b = np.random.default_rng(0).standard_normal(c.size)
    x = np.asarray(xla.spsolve(topo, jnp.asarray(A)[None], jnp.asarray(b)[None]))[0]
    dense = st.to_scipy(A).toarray()
    np.testing.assert_allclose(x, np.linalg.solve(dense, b), rtol=1e-10, atol=1e-12)

    def loss(data):
        return jnp.sum(xla.spsolve(topo, data[None], jnp.asarray(b)[None]) ** 2)

    g = np.asarray(jax.grad(loss)(jnp.asarray(A)))
    xs = np.linalg.solve(dense, b)
    lam = np.linalg.solve(dense.T, 2 * xs)
    ref = -lam[st.rows] * xs[st.indices]
    np.testing.assert_allclose(g, ref, rtol=1e-8, atol=1e-12)
