"""A non-local element group (voltax/element.py:30-34, sparse.py:245-247):
`CoupledInductors`, whose devices share one mutual-inductance matrix, so the
group's Jacobian is one block over all its unknowns. The CPU tests check the
stamping tables and the oracle's group Jacobian; the GPU tests compare the
stamped G and C, DC and trapezoidal transients (voltax
tests/test_sparse.py:267-287's coupled case) and the transient adjoint with
the oracle."""

import numpy as np
import pytest
import torch

from circuits import coupled_circuit
from oracle import analysis as oa
from oracle import stamp as ost


def _dense(st, data):
    rows = np.repeat(np.arange(st.size), np.diff(st.indptr))
    out = np.zeros((st.size, st.size))
    out[rows, st.indices] = data
    return out


def test_coupled_group_tables():
    from voltax_gb300 import symbolic
    from voltax_gb300.runtime import Tables
    c = coupled_circuit()
    st = symbolic.structure(c)
    assert [(name, local) for name, _, _, local in st.devices] == \
        [("K", False), ("R", True), ("V", True)]
    tb = Tables(c, st, st.plan)
    # K: 3 devices x 3 rows x 9 group columns; R: 3 x 2 x 2; V: 1 x 3 x 3
    assert tb.n_res_slots == 9 + 6 + 3
    assert tb.n_jac_slots == 81 + 12 + 9
    # contributions kept (those touching ground dropped): K's block over its
    # 6 non-ground unknowns (every n terminal is ground), R 4 + 1 + 1, V 2 x 2
    assert tb.jac_ptr[-1] == 6 * 6 + 6 + 4


def test_oracle_group_jacobian_matches_finite_differences():
    from voltax_gb300 import symbolic
    c = coupled_circuit()
    st = symbolic.structure(c)
    z = np.random.default_rng(0).normal(size=c.size)
    cf, cq = 1.0, 2.0
    J = _dense(st, ost.jacobian(c, st, z, 0.0, cf, cq))
    F = lambda zz: cf * ost.f(c, zz, 0.0) + cq * ost.q(c, zz)  # noqa: E731
    eye = np.eye(c.size)
    fd = np.stack([(F(z + 1e-6 * eye[j]) - F(z - 1e-6 * eye[j])) / 2e-6
                   for j in range(c.size)], 1)
    np.testing.assert_allclose(J, fd, rtol=1e-7, atol=1e-9)


@pytest.mark.gpu
def test_coupled_stamped_jacobians_match_oracle():
    import voltax_gb300 as vx
    from voltax_gb300 import symbolic
    c = coupled_circuit()
    st = symbolic.structure(c)
    z = np.random.default_rng(1).uniform(-0.5, 0.5, c.size)
    G, C = vx.linearize(c, torch.as_tensor(z), 0.0)
    for M, (cf, cq) in ((G, (1.0, 0.0)), (C, (0.0, 1.0))):
        ref = _dense(st, ost.jacobian(c, st, z, 0.0, cf, cq))
        np.testing.assert_allclose(M.cpu().numpy(), ref, rtol=1e-13,
                                   atol=1e-15 * max(1.0, np.abs(ref).max()))


@pytest.mark.gpu
@pytest.mark.parametrize("engine", ["fused", "generic"])
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_coupled_transient_matches_oracle(engine, precision):
    import voltax_gb300 as vx
    from voltax_gb300 import symbolic
    c = coupled_circuit()
    st = symbolic.structure(c)
    ts = np.linspace(0.0, 5e-6, 101)
    o = vx.Options(engine=engine, precision=precision)
    sol = vx.transient(c, ts, ic="dc", method="trap", options=o)
    assert bool(sol.converged.all())
    ref = oa.transient(oa.System(c, st, st.plan), ts, method="trap")[0]
    np.testing.assert_allclose(sol.z.cpu().numpy(), ref, rtol=1e-9, atol=1e-11)
    dc = vx.dc(c, options=o)
    np.testing.assert_allclose(dc.z.cpu().numpy(),
                               oa.dc(oa.System(c, st, st.plan))[0], rtol=1e-10, atol=1e-12)


@pytest.mark.gpu
def test_coupled_transient_gradient_matches_finite_differences():
    """d(sum of v(b) over the run)/d log l through the transient adjoint, whose
    parameter terms for a coupled group span every device of the group."""
    import voltax_gb300 as vx
    ts = np.linspace(0.0, 5e-6, 51)
    c = coupled_circuit()
    K = c.elements["K"]
    log_l = torch.log(torch.tensor([1e-3, 2e-3, 0.5e-3], dtype=torch.float64))

    def loss(p):
        k = K.with_nodes(K.nodes)
        k.log_l = p
        sol = vx.transient(c.replace("K", k), ts, ic="dc", method="trap",
                           options=vx.Options(precision="f64"))
        return sol.v("b").sum()

    p = log_l.clone().requires_grad_(True)
    (g,) = torch.autograd.grad(loss(p), p)
    fd = torch.stack([(loss(log_l + 1e-6 * e) - loss(log_l - 1e-6 * e)) / 2e-6
                      for e in torch.eye(3, dtype=torch.float64)])
    np.testing.assert_allclose(g.cpu().numpy(), fd.cpu().numpy(), rtol=1e-5,
                               atol=1e-8 * float(fd.abs().max()))
