"""Pins of the CPU oracle to the reference's known answers and invariants.

* RC ladder transient and its gradient: values recorded by voltax
  (tests/test_analysis.py:33-49).
* EKV square law, symmetry, PMOS mirror, charge conservation and C_gg
  (voltax tests/test_elements.py:188-220).
* gmin stepping rescues a CMOS full adder (voltax tests/test_analysis.py:138-149).
* Block-LDU factor/solve equals dense LAPACK for real and transposed systems
  with leaf 1 and 16 (voltax tests/test_sparse.py:208-230).
* Stamped Jacobian equals the Jacobian of the assembled residual
  (voltax tests/test_sparse.py:174-189), and spsolve's VJP equals the dense one
  (voltax tests/test_sparse.py:245-261).
"""

import numpy as np
import pytest
import torch

from oracle import analysis as oa
from oracle import devices as od
from oracle import lu as olu
from oracle import stamp as ost
from voltax_gb300 import elements as el
from voltax_gb300 import symbolic, workloads
from voltax_gb300.builder import CircuitBuilder
from voltax_gb300.library import cmos


def rc_ladder(R1=1e3, R2=2e3, C1=1e-9, C2=0.5e-9, Rload=1e4):
    b = CircuitBuilder()
    b.vsource("in", "0", 1.0, name="Vin")
    b.resistor("in", "a", R1, name="R1")
    b.resistor("a", "out", R2, name="R2")
    b.resistor("out", "0", Rload, name="Rload")
    b.capacitor("a", "0", C1, name="C1")
    b.capacitor("out", "0", C2, name="C2")
    return b.build()


def system(c, leaf=None):
    st = symbolic.structure(c, leaf)
    return oa.System(c, st, st.plan)


def test_rc_ladder_matches_recorded_values():
    c = rc_ladder()
    ts = np.linspace(0, 1e-5, 101)
    z, ok, _ = oa.transient(system(c), ts, ic="zero")
    assert ok.all()
    np.testing.assert_allclose(z[-1], [1.0, 0.921635241, 0.766714055, -7.83647588e-05],
                               atol=1e-8)


def test_rc_ladder_gradient_matches_recorded_values():
    """d sum(v_out) / d log r, by central differences of the oracle."""
    ts = np.linspace(0, 1e-5, 101)
    names = ["R1", "R2", "Rload"]
    base = np.log([1e3, 2e3, 1e4])

    def loss(log_r):
        c = rc_ladder(*np.exp(log_r[:2]), Rload=np.exp(log_r[2]))
        z, _, _ = oa.transient(system(c), ts, ic="zero")
        return z[:, c.node("out")].sum()

    eps = 1e-5
    g = []
    for i in range(3):
        d = np.zeros(3)
        d[i] = eps
        g.append((loss(base + d) - loss(base - d)) / (2 * eps))
    np.testing.assert_allclose(g, -np.array([13.35247162, 13.96802873, -11.62111701]),
                               rtol=1e-6)
    assert names


def _ekv_model(**kw):
    m = el.EKVMOSFET((0, 1, 2, 3), **kw)
    return od.GroupModel(m)


def test_ekv_strong_inversion_square_law():
    p = el.MOSProcess.nmos(kp=200e-6, vth=0.4, n=1.0, lam=0.0)
    m = _ekv_model(w=2e-6, l=1e-6, process=p)
    v = torch.tensor([[1.5, 1.4, 0.0, 0.0]], dtype=torch.float64)
    I, _ = m.currents(v, None, 0.0)
    sq = 0.5 * 200e-6 * 2 * (1.4 - 0.4) ** 2
    assert np.isclose(I[0, 0].item(), sq, rtol=0.05)


def test_ekv_symmetry_and_pmos_mirror():
    n = _ekv_model()
    v = torch.tensor([[0.3, 0.9, 0.1, 0.0]], dtype=torch.float64)
    vs = torch.tensor([[0.1, 0.9, 0.3, 0.0]], dtype=torch.float64)
    assert np.isclose(n.currents(v, None, 0)[0][0, 0], -n.currents(vs, None, 0)[0][0, 0])
    pm = od.GroupModel(el.EKVMOSFET((0, 1, 2, 3), polarity="p", process=n.el.process))
    assert np.isclose(pm.currents(-v, None, 0)[0][0, 0], -n.currents(v, None, 0)[0][0, 0])
    p = _ekv_model(polarity="p")
    on = torch.tensor([[0.0, 0.0, 1.2, 1.2]], dtype=torch.float64)
    assert p.currents(on, None, 0)[0][0, 0] < 0


def test_ekv_charge_conservation_and_saturation_cgg():
    m = _ekv_model(w=10e-6, l=1e-6)
    v = torch.tensor([[1.2, 1.2, 0.0, 0.0]], dtype=torch.float64)
    Q, _ = m.charges(v, None)
    assert abs(Q.sum().item()) < 1e-25
    vg = torch.tensor(1.2, dtype=torch.float64, requires_grad=True)
    vv = torch.stack([v[0, 0], vg, v[0, 2], v[0, 3]])[None]
    cgg = torch.autograd.grad(m.charges(vv, None)[0][0, 1], vg)[0].item()
    p = m.el.process
    n = float(p.n)
    expected = (2 / 3 + (n - 1) / (3 * n)) * float(p.cox) * 10e-12 + 2 * float(p.cov) * 10e-6
    assert np.isclose(cgg, expected, rtol=0.01)


def test_gmin_stepping_rescues_cmos_full_adder():
    b = CircuitBuilder()
    b.vsource("vdd", "0", 1.2)
    for n in ["a", "c"]:
        b.vsource(n, "0", 0.0)
    cmos.full_adder(b, "a", "c", "0", "s", "co", "vdd")
    c = b.build()
    sys = system(c)
    _, plain_ok, _ = oa.dc(sys, opts=oa.Options(gmin_steps=0))
    z, ok, _ = oa.dc(sys)
    assert not plain_ok
    assert ok
    assert z[c.node("s")] < 0.01 and z[c.node("co")] < 0.01


def test_conflicting_sources_do_not_converge():
    b = CircuitBuilder()
    b.vsource("a", "0", 1.0)
    b.vsource("a", "0", 2.0)
    b.resistor("a", "0", 1e3)
    _, ok, _ = oa.dc(system(b.build()))
    assert not ok


def test_rc_ladder_dc_sweep_values():
    for r in (1e3, 1e4, 1e5):
        c = rc_ladder(Rload=r)
        z, ok, _ = oa.dc(system(c))
        assert ok and np.isclose(z[c.node("out")], r / (r + 3e3))


from circuits import (bjt_amplifier, controlled_sources_circuit, mixed_circuit,  # noqa: E402
                      opamp_switch_circuit)


def _cases():
    return {
        "grid": lambda: workloads.power_grid(10, seed=3),
        "adder": lambda: workloads.mirror_adder(2),
        "ring": lambda: workloads.ring_oscillator(9)[0],
        "ring_l1": lambda: workloads.ring_oscillator_level1(9, gamma=0.3)[0],
        "mixed": mixed_circuit,
        "bjt": bjt_amplifier,
        "controlled": controlled_sources_circuit,
        "opamp_switch": opamp_switch_circuit,
    }


@pytest.mark.parametrize("name,leaf", [("grid", 1), ("grid", 16), ("adder", 1),
                                       ("adder", 16), ("ring", 2)])
def test_factor_solve_matches_dense(name, leaf):
    c = _cases()[name]()
    st = symbolic.structure(c)
    plan = symbolic.make_plan(st, leaf)
    pp = olu.from_plan(plan, st)
    z = np.random.default_rng(0).uniform(-0.5, 1.5, c.size)
    G = ost.add_gmin(ost.jacobian(c, st, z, 0.0), st, c.n_nodes, 1e-12)
    C = ost.jacobian(c, st, z, 0.0, 0.0, 1.0)
    rhs = np.random.default_rng(1).standard_normal(c.size)
    for A in (G, G + C / 1e-9):
        dense = st.to_scipy(A).toarray()
        fac = olu.factor(pp, A)
        for tr in (False, True):
            x = olu.solve(pp, fac, rhs, tr)
            ref = np.linalg.solve(dense.T if tr else dense, rhs)
            np.testing.assert_allclose(x, ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max())


@pytest.mark.parametrize("name", ["grid", "adder", "ring"])
def test_stamped_jacobian_equals_full_jacobian(name):
    c = _cases()[name]()
    st = symbolic.structure(c)
    z = np.random.default_rng(0).uniform(-0.5, 1.5, c.size)
    t = 0.3e-9
    for cf, cq, fn in ((1.0, 0.0, lambda zz: ost.f(c, zz, t)), (0.0, 1.0, lambda zz: ost.q(c, zz))):
        A = st.to_scipy(ost.jacobian(c, st, z, t, cf, cq)).toarray()
        h = 1e-7
        ref = np.stack([(fn(z + h * e) - fn(z - h * e)) / (2 * h)
                        for e in np.eye(c.size)], 1)
        scale = np.abs(ref).max()
        np.testing.assert_allclose(A, ref, rtol=1e-5, atol=1e-7 * scale)


def test_spsolve_vjp_matches_dense():
    c = workloads.power_grid(6, seed=2)
    st = symbolic.structure(c)
    pp = olu.from_plan(st.plan, st)
    z = np.zeros(c.size)
    A = ost.add_gmin(ost.jacobian(c, st, z, 0.0), st, c.n_nodes, 1e-12)
    b = np.random.default_rng(2).standard_normal(c.size)
    g = np.random.default_rng(3).standard_normal(c.size)
    gdata, gb = olu.spsolve_vjp(pp, st, A, b, g)
    dense = st.to_scipy(A).toarray()
    x = np.linalg.solve(dense, b)
    gb_ref = np.linalg.solve(dense.T, g)
    np.testing.assert_allclose(gb, gb_ref, rtol=1e-9)
    np.testing.assert_allclose(gdata, -gb_ref[st.rows] * x[st.indices], rtol=1e-8,
                               atol=1e-12)


def test_power_grid_dc_matches_superlu():
    import scipy.sparse.linalg as spla
    c = workloads.power_grid(20, seed=1)
    st = symbolic.structure(c)
    sys = oa.System(c, st, st.plan)
    z, ok, _ = oa.dc(sys)
    assert ok
    A = ost.add_gmin(ost.jacobian(c, st, z, 0.0), st, c.n_nodes, 1e-12)
    r0 = ost.dc_residual(c, np.zeros(c.size), 0.0, 1e-12)
    ref = spla.splu(st.to_scipy(A).tocsc()).solve(-r0)
    np.testing.assert_allclose(z, ref, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("name,method", [("grid", "be"), ("adder", "be"), ("ring", "trap"),
                                         ("ring_l1", "be"), ("mixed", "trap"),
                                         ("bjt", "trap"), ("controlled", "be"),
                                         ("opamp_switch", "be")])
def test_compiled_baseline_matches_oracle(name, method):
    """oracle/cvx.c (the timed CPU baseline) equals the torch restatement."""
    from oracle import cbase
    c = _cases()[name]()
    st = symbolic.structure(c)
    ts = np.linspace(0.0, 40e-12, 9)
    z0 = None
    if name == "ring":
        z0 = workloads.ring_initial_state(c, [f"n{k}" for k in range(9)]).numpy()
    if name == "ring_l1":
        z0 = workloads.ring_level1_initial_state(
            c, [f"n{k}" for k in range(1, 10)]).numpy()
    zc, okc, itc = cbase.CSystem(c, st, st.plan).run(ts, z0=z0, method=method,
                                                      dc_first=z0 is None)
    zr, okr, itr = oa.transient(oa.System(c, st, st.plan), ts, ic="dc" if z0 is None else z0,
                                method=method)
    assert okc.all() and okr.all()
    assert np.array_equal(itc[1:], itr[1:])
    np.testing.assert_allclose(zc, zr, rtol=1e-10, atol=1e-12)


def _l1(v, **kw):
    m = od.GroupModel(el.Level1MOSFET((0, 1, 2, 3), **kw))
    return m.currents(torch.tensor([v], dtype=torch.float64), None, 0.0)[0][0, 0].item()


def test_level1_exact_square_law_and_body_effect():
    """voltax tests/test_elements.py:222-231 (known answers)."""
    p = el.MOSProcess.nmos(kp=100e-6, vth=0.5, lam=0.02, gamma=0.4, phi=0.7)
    kw = dict(w=4e-6, l=1e-6, process=p, smooth=0.0)
    k = 100e-6 * 4
    assert np.isclose(_l1([2.0, 1.5, 0.0, 0.0], **kw), 0.5 * k * 1.0 * (1 + 0.04))
    assert np.isclose(_l1([0.2, 1.5, 0.0, 0.0], **kw), k * (1.0 - 0.1) * 0.2 * 1.004)
    assert _l1([1.0, 0.4, 0.0, 0.0], **kw) == 0.0
    vth_body = 0.5 + 0.4 * (np.sqrt(0.7 + 0.5) - np.sqrt(0.7))
    assert np.isclose(_l1([3.0, 2.0, 0.5, 0.0], **kw),
                      0.5 * k * (1.5 - vth_body) ** 2 * (1 + 0.02 * 2.5))


def test_level1_reverse_mode_smooth_and_pmos_mirror():
    p = el.MOSProcess.nmos(kp=100e-6, vth=0.5, lam=0.02)
    kw = dict(w=4e-6, l=1e-6, process=p, smooth=0.0)
    # drain and source swap for vds < 0
    assert np.isclose(_l1([0.0, 1.5, 0.3, 0.0], **kw), -_l1([0.3, 1.5, 0.0, 0.0], **kw))
    # smoothing only matters near cutoff
    assert np.isclose(_l1([1.0, 1.5, 0.0, 0.0], **{**kw, "smooth": 0.02}),
                      _l1([1.0, 1.5, 0.0, 0.0], **kw), rtol=1e-6)
    assert _l1([1.0, 0.5, 0.0, 0.0], **{**kw, "smooth": 0.02}) > 0.0
    pm = dict(kw, polarity="p", process=el.MOSProcess.pmos(kp=100e-6, vth=0.5, lam=0.02))
    assert np.isclose(_l1([-1.0, -1.5, 0.0, 0.0], **pm), -_l1([1.0, 1.5, 0.0, 0.0], **kw))
