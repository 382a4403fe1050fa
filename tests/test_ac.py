"""AC small-signal analysis (voltax/analysis.py:483-524) on the GPU against
closed forms and the oracle's dense complex solves."""

import numpy as np
import pytest
import torch

from oracle import analysis as oa

pytestmark = pytest.mark.gpu


def _rc(R=1e3, C=1e-7):
    from voltax_gb300.builder import CircuitBuilder
    b = CircuitBuilder()
    b.vsource("in", "0", 0.0, ac=1.0, name="Vin")
    b.resistor("in", "out", R, name="R1")
    b.capacitor("out", "0", C, name="C1")
    return b.build()


def test_rc_lowpass_closed_form():
    import voltax_gb300 as vx
    R, C = 1e3, 1e-7
    f = np.logspace(1, 6, 41)
    sol = vx.ac(_rc(R, C), f)
    w = 2 * np.pi * f * R * C
    h = sol.v("out").cpu().numpy()
    np.testing.assert_allclose(np.abs(h), 1 / np.sqrt(1 + w ** 2), rtol=1e-12)
    np.testing.assert_allclose(np.angle(h), -np.arctan(w), rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(sol.db("out").cpu().numpy(),
                               -10 * np.log10(1 + w ** 2), atol=1e-10)
    # the stimulus source's branch current: i = -(v_in - v_out)/R through the source
    i = sol.i("Vin").cpu().numpy()
    np.testing.assert_allclose(i, -(1 - h) / R, rtol=1e-10)


def test_phase_unwrapped_through_four_poles():
    """voltax tests/test_analysis.py:240-249, buffered by VCCS stages
    (gm = -1 mS into 1 kOhm: gain +1)."""
    import voltax_gb300 as vx
    from voltax_gb300.builder import CircuitBuilder
    b = CircuitBuilder()
    b.vsource("in", "0", 0.0, ac=1.0, name="Vin")
    for k in range(4):
        b.resistor("in" if k == 0 else f"b{k}", f"n{k}", 1e3, name=f"R{k}")
        b.capacitor(f"n{k}", "0", 1e-9, name=f"C{k}")
        b.vccs(f"b{k + 1}", "0", f"n{k}", "0", -1e-3, name=f"G{k}")
        b.resistor(f"b{k + 1}", "0", 1e3, name=f"RL{k}")
    sol = vx.ac(b.build(), np.logspace(3, 8, 200))
    ph = sol.phase("b4").numpy()
    assert ph[-1] < -300
    assert np.all(np.diff(ph) < 1.0)


@pytest.mark.parametrize("name", ["mixed", "ota", "controlled"])
def test_ac_matches_oracle(name):
    import voltax_gb300 as vx
    from voltax_gb300 import symbolic, workloads
    if name == "controlled":  # transformer and controlled sources; Vin carries ac=1
        from circuits import controlled_sources_circuit
        c = controlled_sources_circuit()
    elif name == "ota":
        c = workloads.ota_chain(6)
        c = c.replace("VoltageSource", _with_ac(c.elements["VoltageSource"],
                                                 c.layout.device("Vin")[1]))
    else:
        from circuits import mixed_circuit
        c = mixed_circuit()
        c = c.replace("VoltageSource_Pulse", _with_ac(c.elements["VoltageSource_Pulse"], 0))
    f = np.logspace(6, 11, 17)
    sol = vx.ac(c, f)
    st = symbolic.structure(c)
    z_op = sol.op.z.cpu().numpy()
    ref = oa.ac(oa.System(c, st, st.plan), f, z_op)
    z = sol.z.cpu().numpy()
    scale = np.abs(ref).max(axis=1, keepdims=True)
    assert np.max(np.abs(z - ref) / scale) < 1e-10


def _with_ac(el, idx):
    e = el.with_nodes(el.nodes)
    ac = torch.zeros(el.size, dtype=torch.float64)
    ac[idx] = 1.0
    e.ac, e.ac_phase = ac, torch.full((el.size,), 30.0, dtype=torch.float64)
    return e


def test_linearize_matches_oracle_jacobians():
    import voltax_gb300 as vx
    from oracle import stamp as ost
    from voltax_gb300 import symbolic
    from circuits import mixed_circuit
    c = mixed_circuit()
    st = symbolic.structure(c)
    z = np.random.default_rng(3).uniform(-0.3, 0.8, c.size)
    G, C = vx.linearize(c, torch.as_tensor(z), 0.0)
    rows = np.repeat(np.arange(st.size), np.diff(st.indptr))
    for M, (cf, cq) in ((G, (1.0, 0.0)), (C, (0.0, 1.0))):
        ref = np.zeros((st.size, st.size))
        ref[rows, st.indices] = ost.jacobian(c, st, z, 0.0, cf, cq)
        np.testing.assert_allclose(M.cpu().numpy(), ref, rtol=1e-12,
                                   atol=1e-15 * max(1.0, np.abs(ref).max()))


def _rc_mesh(n, seed=0):
    """An n x n RC mesh (lognormal branch conductances, a capacitor at every
    node) driven at one corner by an AC source and tied down at the other."""
    from voltax_gb300.builder import CircuitBuilder
    rng = np.random.default_rng(seed)
    b = CircuitBuilder()
    b.vsource("n0_0", "0", 1.0, ac=1.0, name="Vin")
    b.vsource(f"n{n - 1}_{n - 1}", "0", 0.0, name="Vgnd")
    g = np.exp(rng.normal(0.0, 0.3, (2, n, n)))
    cap = 1e-12 * (1.0 + rng.random((n, n)))
    for i in range(n):
        for j in range(n):
            if j + 1 < n:
                b.resistor(f"n{i}_{j}", f"n{i}_{j + 1}", 1.0 / g[0, i, j])
            if i + 1 < n:
                b.resistor(f"n{i}_{j}", f"n{i + 1}_{j}", 1.0 / g[1, i, j])
            b.capacitor(f"n{i}_{j}", "0", cap[i, j])
    return b.build()


def test_ac_wide_supernode_matches_sparse_oracle():
    """A 140 x 140 RC mesh: its root separator (k = 115) is too wide for the
    complex factorization's shared memory, so the wide kernel (F11 left in
    its panel) factors it. Reference: the oracle's stamped G and C solved by
    scipy's sparse LU at each frequency."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    import voltax_gb300 as vx
    from voltax_gb300 import symbolic
    from oracle import stamp as ost
    c = _rc_mesh(140)
    st = symbolic.structure(c)
    assert int(np.max(st.plan.k)) > 104
    f = np.array([1e8, 1e10])
    sol = vx.ac(c, f)
    z_op = sol.op.z.cpu().numpy()
    rows = np.repeat(np.arange(st.size), np.diff(st.indptr))
    shape = (st.size, st.size)
    G = sp.csr_matrix((ost.jacobian(c, st, z_op, 0.0, 1.0, 0.0), (rows, st.indices)), shape)
    Cm = sp.csr_matrix((ost.jacobian(c, st, z_op, 0.0, 0.0, 1.0), (rows, st.indices)), shape)
    rhs = -oa._ac_stimulus(c)
    ref = np.stack([spl.splu((G + 2j * np.pi * fk * Cm).tocsc(), permc_spec="COLAMD").solve(rhs)
                    for fk in f])
    z = sol.z.cpu().numpy()
    scale = np.abs(ref).max(axis=1, keepdims=True)
    assert np.max(np.abs(z - ref) / scale) < 1e-10
