"""GPU parity against the CPU oracle, through the C ABI.

* stamping: f, q and the CSR Jacobian equal the oracle; bit for bit on
  linear circuits (same device values, same canonical summation order), to
  1e-12 relative on EKV circuits (analytic vs forward-mode derivatives), and
  bitwise reproducible run to run (voltax tests/test_sparse.py:174-189);
* factor/solve: real and transposed solves equal dense LAPACK for plans with
  leaf 1, 2 and 16, in FP64 and in FP32 + FP64 refinement
  (voltax tests/test_sparse.py:208-230);
* analyses: DC and transient node voltages within 1e-9 relative of the
  oracle, the same convergence flags and the same Newton iteration counts
  (voltax tests/test_sparse.py:264-295);
* adjoints: spsolve and dc gradients equal dense / finite differences
  (voltax tests/test_sparse.py:245-261, 336-353).
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from oracle import analysis as oa  # noqa: E402
from oracle import stamp as ost  # noqa: E402
import voltax_gb300 as vx  # noqa: E402
from voltax_gb300 import sparse, symbolic, workloads  # noqa: E402
from voltax_gb300.builder import CircuitBuilder  # noqa: E402
from voltax_gb300.library import cmos  # noqa: E402


def rc_ladder(R1=1e3, R2=2e3, C1=1e-9, C2=0.5e-9, Rload=1e4):
    b = CircuitBuilder()
    b.vsource("in", "0", 1.0, name="Vin")
    b.resistor("in", "a", R1, name="R1")
    b.resistor("a", "out", R2, name="R2")
    b.resistor("out", "0", Rload, name="Rload")
    b.capacitor("a", "0", C1, name="C1")
    b.capacitor("out", "0", C2, name="C2")
    return b.build()


CIRCUITS = {
    "rc_ladder": rc_ladder,
    "grid": lambda: workloads.power_grid(10, seed=3),
    "adder": lambda: workloads.mirror_adder(2),
    "ring": lambda: workloads.ring_oscillator(9)[0],
    "ring_l1": lambda: workloads.ring_oscillator_level1(5, gamma=0.3)[0],
    "ring_l1_smooth": lambda: workloads.ring_oscillator_level1(5, smooth=0.02, gamma=0.3)[0],
}
from circuits import (bjt_amplifier, controlled_sources_circuit, mixed_circuit,  # noqa: E402
                      opamp_switch_circuit)

CIRCUITS["mixed"] = mixed_circuit
CIRCUITS["bjt"] = bjt_amplifier
CIRCUITS["controlled"] = controlled_sources_circuit
CIRCUITS["opamp_switch"] = opamp_switch_circuit
LINEAR = ("rc_ladder", "grid")


def rel(a, b, floor=1e-3):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if a.size else 0.0


@pytest.mark.parametrize("name", list(CIRCUITS))
def test_stamping_matches_oracle(name):
    c = CIRCUITS[name]()
    st = symbolic.structure(c)
    z = np.random.default_rng(0).uniform(-0.5, 1.5, c.size)
    t = 0.3e-9
    zt = torch.as_tensor(z)
    f_gpu = c.f(zt, t).cpu().numpy()
    q_gpu = c.q(zt).cpu().numpy()
    f_ref, q_ref = ost.f(c, z, t), ost.q(c, z)
    for cf, cq in ((1.0, 0.0), (0.0, 1.0), (0.5, 1e9)):
        J = sparse.jacobian(c, zt, t, cf, cq, structure=st).cpu().numpy()
        J2 = sparse.jacobian(c, zt, t, cf, cq, structure=st).cpu().numpy()
        J_ref = ost.jacobian(c, st, z, t, cf, cq)
        assert np.array_equal(J, J2), "stamping is not bitwise reproducible"
        if name in LINEAR:
            assert np.array_equal(J, J_ref), "linear stamps differ from the canonical sum"
        else:
            scale = np.abs(J_ref).max()
            np.testing.assert_allclose(J, J_ref, rtol=1e-12, atol=1e-14 * scale)
    if name in LINEAR:
        assert np.array_equal(f_gpu, f_ref) and np.array_equal(q_gpu, q_ref)
    else:
        np.testing.assert_allclose(f_gpu, f_ref, rtol=1e-12, atol=1e-15 * np.abs(f_ref).max())
        np.testing.assert_allclose(q_gpu, q_ref, rtol=1e-12, atol=1e-15 * np.abs(q_ref).max())


@pytest.mark.parametrize("name,leaf", [("grid", 1), ("grid", 16), ("adder", 1),
                                       ("adder", 16), ("ring", 2), ("rc_ladder", 16)])
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_factor_solve_matches_dense(name, leaf, precision):
    c = CIRCUITS[name]()
    st = symbolic.structure(c)
    plan = symbolic.make_plan(st, leaf)
    z = np.random.default_rng(0).uniform(-0.5, 1.5, c.size)
    G = ost.add_gmin(ost.jacobian(c, st, z, 0.0), st, c.n_nodes, 1e-12)
    C = ost.jacobian(c, st, z, 0.0, 0.0, 1.0)
    rhs = np.random.default_rng(1).standard_normal(c.size)
    for A in (G, G + C / 1e-9):
        dense = st.to_scipy(A).toarray()
        fac = sparse.factor(plan, torch.as_tensor(A), precision)
        for tr in (False, True):
            x = sparse.solve(plan, fac, torch.as_tensor(rhs), tr).cpu().numpy()
            ref = np.linalg.solve(dense.T if tr else dense, rhs)
            np.testing.assert_allclose(x, ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max())


def _oracle_dc(c):
    st = symbolic.structure(c)
    return oa.dc(oa.System(c, st, st.plan))


ENGINES = ["fused", "generic"]


@pytest.mark.parametrize("name", ["rc_ladder", "grid", "adder"])
@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("engine", ENGINES)
def test_dc_matches_oracle(name, precision, engine):
    c = CIRCUITS[name]()
    sol = vx.dc(c, options=vx.Options(precision=precision, engine=engine))
    z_ref, ok_ref, it_ref = _oracle_dc(c)
    assert bool(sol.converged) == ok_ref
    assert rel(sol.z.cpu().numpy(), z_ref) < 1e-9
    if precision == "f64":
        assert int(sol.iterations) == it_ref


@pytest.mark.parametrize("engine", ENGINES)
def test_cmos_full_adder_needs_gmin_stepping(engine):
    """voltax tests/test_analysis.py:138-149 on the GPU."""
    b = CircuitBuilder()
    b.vsource("vdd", "0", 1.2)
    for n in ["a", "c"]:
        b.vsource(n, "0", 0.0)
    cmos.full_adder(b, "a", "c", "0", "s", "co", "vdd")
    c = b.build()
    plain = vx.dc(c, options=vx.Options(gmin_steps=0, engine=engine))
    rescued = vx.dc(c, options=vx.Options(engine=engine))
    assert not bool(plain.converged)
    assert bool(rescued.converged)
    z_ref, ok_ref, it_ref = _oracle_dc(c)
    assert ok_ref and rel(rescued.z.cpu().numpy(), z_ref) < 1e-9
    assert float(rescued.v("s")) < 0.01 and float(rescued.v("co")) < 0.01


def test_singular_circuit_fails_check():
    b = CircuitBuilder()
    b.vsource("a", "0", 1.0)
    b.vsource("a", "0", 2.0)
    b.resistor("a", "0", 1e3)
    with pytest.raises(RuntimeError, match="did not converge"):
        vx.dc(b.build()).check()


@pytest.mark.parametrize("method", ["be", "trap"])
@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("engine", ENGINES)
def test_ring_transient_matches_oracle(method, precision, engine):
    c, nodes = workloads.ring_oscillator(9)
    z0 = workloads.ring_initial_state(c, nodes)
    ts = np.linspace(0.0, 60e-12, 31)
    sol = vx.transient(c, ts, ic=z0, method=method,
                       options=vx.Options(precision=precision, engine=engine))
    st = symbolic.structure(c)
    zr, okr, itr = oa.transient(oa.System(c, st, st.plan), ts, ic=z0.numpy(), method=method)
    assert bool(sol.converged.all()) and okr.all()
    v, vr = sol.z.cpu().numpy(), zr
    assert np.max(np.abs(v[:, : c.n_nodes] - vr[:, : c.n_nodes])) < 1e-9
    if precision == "f64":
        assert np.array_equal(sol.iterations.cpu().numpy()[1:], itr[1:])


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("engine", ENGINES)
def test_level1_ring_transient_matches_oracle(precision, engine):
    """The reference's own ring benchmark circuit (exact Level 1, body
    effect on, backward Euler): node voltages and Newton iterations."""
    c, nodes = workloads.ring_oscillator_level1(9, gamma=0.3)
    z0 = workloads.ring_level1_initial_state(c, nodes)
    ts = np.linspace(0.0, 40e-12, 41)
    sol = vx.transient(c, ts, ic=z0, method="be",
                       options=vx.Options(precision=precision, engine=engine))
    st = symbolic.structure(c)
    zr, okr, itr = oa.transient(oa.System(c, st, st.plan), ts, ic=z0.numpy(), method="be")
    assert bool(sol.converged.all()) and okr.all()
    v = sol.z.cpu().numpy()
    assert np.max(np.abs(v[:, : c.n_nodes] - zr[:, : c.n_nodes])) < 1e-9
    if precision == "f64":
        assert np.array_equal(sol.iterations.cpu().numpy()[1:], itr[1:])


def test_level1_dc_gradient_matches_finite_differences():
    """Parameter VJP of the Level-1 kernel (dual numbers) through the DC
    adjoint: d v(out) / d (dvth, log W) of an inverter with body effect."""
    import functools
    from voltax_gb300.elements import Level1MOSFET, MOSProcess
    b = CircuitBuilder(nmos=MOSProcess.nmos(gamma=0.4), pmos=MOSProcess.pmos(gamma=0.4),
                       mos_model=functools.partial(Level1MOSFET, smooth=0.02))
    b.vsource("vdd", "0", 1.2, name="Vdd")
    b.vsource("in", "0", 0.55, name="Vin")
    b.resistor("vdd", "src", 2e3, name="Rs")
    b.nmos("out", "in", "src2", "0", w=2e-6, name="Mn")
    b.resistor("src2", "0", 1e3, name="Rdeg")
    b.pmos("out", "in", "vdd", "vdd", w=2e-6, name="Mp")
    c = b.build()
    out = c.node("out")

    def v_out(c2):
        return vx.dc(c2).z[out]

    for gname in ("Level1MOSFET_n", "Level1MOSFET_p"):
        el = c.elements[gname]
        for field in ("dvth", "log_w"):
            e2 = el.with_nodes(el.nodes)
            setattr(e2, field, getattr(el, field).clone().requires_grad_(True))
            v_out(c.replace(gname, e2)).backward()
            g = getattr(e2, field).grad.numpy()
            h = 1e-6
            e_p = el.with_nodes(el.nodes)
            setattr(e_p, field, getattr(el, field).clone() + h)
            e_m = el.with_nodes(el.nodes)
            setattr(e_m, field, getattr(el, field).clone() - h)
            fd = (float(v_out(c.replace(gname, e_p))) -
                  float(v_out(c.replace(gname, e_m)))) / (2 * h)
            np.testing.assert_allclose(g.sum(), fd, rtol=1e-5, atol=1e-9)


@pytest.mark.parametrize("method", ["be", "trap"])
@pytest.mark.parametrize("engine", ENGINES)
def test_mixed_devices_transient_matches_oracle(method, engine):
    """Inductor, diode (with charges) and VCCS through a pulse transient."""
    c = mixed_circuit()
    ts = np.linspace(0.0, 150e-12, 61)
    sol = vx.transient(c, ts, ic="dc", method=method, options=vx.Options(engine=engine))
    st = symbolic.structure(c)
    zr, okr, itr = oa.transient(oa.System(c, st, st.plan), ts, ic="dc", method=method)
    assert bool(sol.converged.all()) and okr.all()
    v = sol.z.cpu().numpy()
    scale = max(1.0, np.abs(zr).max())
    assert np.max(np.abs(v - zr)) < 1e-9 * scale
    assert np.array_equal(sol.iterations.cpu().numpy()[1:], itr[1:])


@pytest.mark.parametrize("engine", ENGINES)
def test_bjt_amplifier_transient_matches_oracle(engine):
    c = bjt_amplifier()
    ts = np.linspace(0.0, 6e-9, 61)
    sol = vx.transient(c, ts, ic="dc", method="trap", options=vx.Options(engine=engine))
    st = symbolic.structure(c)
    zr, okr, itr = oa.transient(oa.System(c, st, st.plan), ts, ic="dc", method="trap")
    assert bool(sol.converged.all()) and okr.all()
    v = sol.z.cpu().numpy()[:, : c.n_nodes]
    assert np.max(np.abs(v - zr[:, : c.n_nodes])) < 1e-9 * max(1.0, np.abs(zr).max())
    assert np.array_equal(sol.iterations.cpu().numpy()[1:], itr[1:])


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_controlled_sources_transient_matches_oracle(precision):
    """VCVS, CCCS, CCVS and a transformer (local blocks of 5 and 6 unknowns,
    generic engine)."""
    c = controlled_sources_circuit()
    ts = np.linspace(0.0, 8e-9, 81)
    sol = vx.transient(c, ts, ic="dc", method="trap", options=vx.Options(precision=precision))
    st = symbolic.structure(c)
    zr, okr, itr = oa.transient(oa.System(c, st, st.plan), ts, ic="dc", method="trap")
    assert bool(sol.converged.all()) and okr.all()
    scale = max(1.0, np.abs(zr).max())
    assert np.max(np.abs(sol.z.cpu().numpy() - zr)) < 1e-9 * scale
    with pytest.raises(Exception, match="not eligible"):
        vx.dc(c, options=vx.Options(engine="fused"))


@pytest.mark.parametrize("engine", ENGINES)
def test_opamp_switch_transient_matches_oracle(engine):
    """Ideal and single-pole op-amps and a smoothed switch."""
    c = opamp_switch_circuit()
    ts = np.linspace(0.0, 2e-6, 101)
    sol = vx.transient(c, ts, ic="dc", method="be", options=vx.Options(engine=engine))
    st = symbolic.structure(c)
    zr, okr, itr = oa.transient(oa.System(c, st, st.plan), ts, ic="dc", method="be")
    assert bool(sol.converged.all()) and okr.all()
    v = sol.z.cpu().numpy()[:, : c.n_nodes]
    assert np.max(np.abs(v - zr[:, : c.n_nodes])) < 1e-9 * max(1.0, np.abs(zr).max())
    assert np.array_equal(sol.iterations.cpu().numpy()[1:], itr[1:])
    # the inverting stage: a = -4 in at DC (ideal op-amp, 1k / 4k)
    assert abs(float(sol.z[0, c.node("a")]) - (-4 * -0.2)) < 1e-9


def test_controlled_sources_dc_gradient_matches_finite_differences():
    c = controlled_sources_circuit().set("Vin", v1=0.7)
    out = c.node("e")
    for gname, field in (("VCVS", "gain"), ("CCCS", "gain"), ("CCVS", "r")):
        el = c.elements[gname]
        e2 = el.with_nodes(el.nodes)
        setattr(e2, field, getattr(el, field).clone().requires_grad_(True))
        sol = vx.dc(c.replace(gname, e2))
        (sol.z[c.node("d")] + sol.z[out]).backward()
        g = getattr(e2, field).grad.numpy().sum()
        h = 1e-6 * max(1.0, float(getattr(el, field).abs().max()))
        vals = []
        for sgn in (1, -1):
            e3 = el.with_nodes(el.nodes)
            setattr(e3, field, getattr(el, field).clone() + sgn * h)
            s3 = vx.dc(c.replace(gname, e3))
            vals.append(float(s3.z[c.node("d")] + s3.z[out]))
        np.testing.assert_allclose(g, (vals[0] - vals[1]) / (2 * h), rtol=1e-6, atol=1e-12)


def test_bjt_dc_gradient_matches_finite_differences():
    c = bjt_amplifier()
    out = c.node("out")
    for gname in ("BJT_npn", "BJT_pnp"):
        el = c.elements[gname]
        for field in ("log_is", "log_bf", "inv_vaf"):
            e2 = el.with_nodes(el.nodes)
            setattr(e2, field, getattr(el, field).clone().requires_grad_(True))
            vx.dc(c.replace(gname, e2)).z[out].backward()
            g = getattr(e2, field).grad.numpy().sum()
            h = 1e-6
            vals = []
            for sgn in (1, -1):
                e3 = el.with_nodes(el.nodes)
                setattr(e3, field, getattr(el, field).clone() + sgn * h)
                vals.append(float(vx.dc(c.replace(gname, e3)).z[out]))
            np.testing.assert_allclose(g, (vals[0] - vals[1]) / (2 * h), rtol=1e-5, atol=1e-9)


def test_mixed_devices_dc_gradient_matches_finite_differences():
    """Parameter VJP of the diode, inductor and VCCS kernels (dual numbers)."""
    c = mixed_circuit().set("Vin", v1=0.8)
    out = c.node("d")
    cases = [("Diode", "log_is"), ("Diode", "n"), ("VCCS", "gm"), ("Resistor", "log_r")]
    for gname, field in cases:
        el = c.elements[gname]
        e2 = el.with_nodes(el.nodes)
        setattr(e2, field, getattr(el, field).clone().requires_grad_(True))
        vx.dc(c.replace(gname, e2)).z[out].backward()
        g = getattr(e2, field).grad.numpy().sum()
        h = 1e-6
        vals = []
        for sgn in (1, -1):
            e3 = el.with_nodes(el.nodes)
            setattr(e3, field, getattr(el, field).clone() + sgn * h)
            vals.append(float(vx.dc(c.replace(gname, e3)).z[out]))
        fd = (vals[0] - vals[1]) / (2 * h)
        np.testing.assert_allclose(g, fd, rtol=1e-5, atol=1e-9), (gname, field)


def test_rc_ladder_recorded_values_on_gpu():
    """voltax tests/test_analysis.py:33-39 through the GPU path."""
    c = rc_ladder()
    sol = vx.transient(c, np.linspace(0, 1e-5, 101), ic="zero")
    np.testing.assert_allclose(sol.z[-1].cpu().numpy(),
                               [1.0, 0.921635241, 0.766714055, -7.83647588e-05], atol=1e-8)


@pytest.mark.parametrize("engine", ENGINES)
def test_batched_mc_matches_per_instance_oracle(engine):
    c = workloads.mirror_adder_mc(6, seed=1, bits=2)
    ts = np.linspace(0, 200e-12, 21)
    sol = vx.transient(c, ts, ic="dc", method="be",
                       options=vx.Options(precision="f32", engine=engine))
    assert sol.z.shape == (6, len(ts), c.size)
    st = symbolic.structure(c)
    for b in (0, 5):
        sys_b = oa.System(c, st, st.plan, b)
        zr, okr, _ = oa.transient(sys_b, ts, ic="dc", method="be")
        assert okr.all() and bool(sol.converged[b].all())
        assert np.max(np.abs(sol.z[b].cpu().numpy() - zr)) < 1e-9


def test_spsolve_gradients_match_dense():
    c = workloads.power_grid(6, seed=2)
    st = symbolic.structure(c)
    A = ost.add_gmin(ost.jacobian(c, st, np.zeros(c.size), 0.0), st, c.n_nodes, 1e-12)
    rhs = np.random.default_rng(2).standard_normal(c.size)
    data = torch.tensor(A, device="cuda", requires_grad=True)
    b = torch.tensor(rhs, device="cuda", requires_grad=True)
    x = sparse.spsolve(st, data, b)
    torch.sin(x).sum().backward()
    dense = torch.tensor(st.to_scipy(A).toarray(), requires_grad=True)
    bd = torch.tensor(rhs, requires_grad=True)
    xd = torch.linalg.solve(dense, bd)
    torch.sin(xd).sum().backward()
    rows, cols = torch.as_tensor(st.rows), torch.as_tensor(st.indices)
    np.testing.assert_allclose(data.grad.cpu().numpy(), dense.grad[rows, cols].numpy(),
                               rtol=1e-7, atol=1e-12)
    np.testing.assert_allclose(b.grad.cpu().numpy(), bd.grad.numpy(), rtol=1e-7)


def test_dc_gradient_of_power_grid_matches_finite_differences():
    """voltax tests/test_sparse.py:336-353: d v(worst) / d log r."""
    c = workloads.power_grid(8, seed=4)
    el = c.elements["Resistor"]
    log_r = el.log_r.clone().requires_grad_(True)
    el2 = el.with_nodes(el.nodes)
    el2.log_r = log_r
    c2 = c.replace("Resistor", el2)
    sol = vx.dc(c2)
    worst = int(torch.argmin(sol.v().detach()))
    sol.z[worst].backward()
    g = log_r.grad.numpy()
    k = int(np.argmax(np.abs(g)))
    eps = 1e-5

    def v_at(delta):
        e3 = el.with_nodes(el.nodes)
        lr = el.log_r.clone()
        lr[k] += delta
        e3.log_r = lr
        return float(vx.dc(c.replace("Resistor", e3)).z[worst])

    fd = (v_at(eps) - v_at(-eps)) / (2 * eps)
    assert np.isclose(g[k], fd, rtol=1e-6)
    # and against the oracle adjoint lam = J^-T e_worst, dv/dlog_r = -lam^T dF/dlog_r
    st = symbolic.structure(c)
    sys_o = oa.System(c, st, st.plan)
    z_ref, _, _ = oa.dc(sys_o)
    e = np.zeros(c.size)
    e[worst] = 1.0
    lam = oa.dc_adjoint(sys_o, z_ref, e)
    nodes = el.node_array()
    v = np.concatenate([z_ref, [0.0]])
    lv = np.concatenate([lam, [0.0]])
    dv = v[nodes[:, 0]] - v[nodes[:, 1]]
    gref = -(lv[nodes[:, 0]] - lv[nodes[:, 1]]) * dv * (-np.exp(-el.log_r.numpy()))
    np.testing.assert_allclose(g, gref, rtol=1e-8, atol=1e-12 * np.abs(gref).max())


def test_f32_refined_matches_f64_on_power_grid():
    c = workloads.power_grid(40, seed=7)
    s64 = vx.dc(c, options=vx.Options(precision="f64"))
    s32 = vx.dc(c, options=vx.Options(precision="f32"))
    assert bool(s64.converged) and bool(s32.converged)
    assert rel(s32.z.cpu().numpy(), s64.z.cpu().numpy()) < 1e-9


def test_fused_equals_generic_on_the_4bit_adder():
    c = workloads.mirror_adder_mc(8, seed=2)
    ts = np.linspace(0, 300e-12, 31)
    a = vx.transient(c, ts, ic="dc", options=vx.Options(engine="fused"))
    b = vx.transient(c, ts, ic="dc", options=vx.Options(engine="generic"))
    assert bool(a.converged.all()) and bool(b.converged.all())
    assert float((a.z - b.z).abs().max()) < 1e-11
    assert torch.equal(a.iterations[:, 1:], b.iterations[:, 1:])


def test_fused_is_bitwise_reproducible():
    c = workloads.mirror_adder_mc(4, seed=3)
    ts = np.linspace(0, 100e-12, 11)
    o = vx.Options(engine="fused", precision="f32")
    a = vx.transient(c, ts, ic="dc", options=o)
    b = vx.transient(c, ts, ic="dc", options=o)
    assert torch.equal(a.z, b.z)


@pytest.mark.parametrize("engine", ENGINES)
def test_rc_ladder_transient_gradient_matches_recorded_values(engine):
    """voltax tests/test_analysis.py:41-49: d sum(v_out) / d log r through the
    transient (implicit adjoint over every step)."""
    c = rc_ladder()
    el = c.elements["Resistor"]
    e2 = el.with_nodes(el.nodes)
    e2.log_r = el.log_r.clone().requires_grad_(True)
    c2 = c.replace("Resistor", e2)
    ts = np.linspace(0, 1e-5, 101)
    sol = vx.transient(c2, ts, ic="zero", options=vx.Options(engine=engine))
    sol.v("out").sum().backward()
    names = c.devices("Resistor")  # R1, R2, Rload in group order
    assert names == ["R1", "R2", "Rload"]
    np.testing.assert_allclose(e2.log_r.grad.numpy(),
                               -np.array([13.35247162, 13.96802873, -11.62111701]), rtol=1e-6)


@pytest.mark.parametrize("method", ["be", "trap"])
@pytest.mark.parametrize("engine", ENGINES)
def test_ekv_transient_gradient_matches_finite_differences(method, engine):
    c = workloads.mirror_adder(1)
    ts = np.linspace(0, 120e-12, 13)
    name = "EKVMOSFET_n"
    el = c.elements[name]
    o = vx.Options(engine=engine)

    def loss(dvth):
        e2 = el.with_nodes(el.nodes)
        e2.dvth = dvth
        sol = vx.transient(c.replace(name, e2), ts, ic="dc", method=method, options=o)
        return (sol.v("s0") ** 2).sum() + sol.v("co").sum()

    dv = el.dvth.clone().requires_grad_(True)
    loss(dv).backward()
    g = dv.grad.numpy()
    k = int(np.argmax(np.abs(g)))
    eps = 1e-5
    up, dn = el.dvth.clone(), el.dvth.clone()
    up[k] += eps
    dn[k] -= eps
    fd = (float(loss(up)) - float(loss(dn))) / (2 * eps)
    assert np.isclose(g[k], fd, rtol=1e-5, atol=1e-9)


def test_fused_wide_supernode_ota_chain_matches_generic_and_oracle():
    """66-stage OTA chain: its root supernode is 66 wide, so the fused
    kernel factors and solves it with the whole CTA (k > 32 path)."""
    base = workloads.ota_chain(66)
    P = workloads.ota_params(16, seed=5)
    c = workloads.apply_ota_params(base, P)
    st = symbolic.structure(c)
    assert max(st.plan.k) == 66
    fused = vx.dc(c, options=vx.Options(engine="fused", precision="f32"))
    gen = vx.dc(c, options=vx.Options(engine="generic"))
    assert bool(fused.converged.all()) and bool(gen.converged.all())
    nv = c.layout.n_nodes
    scale = gen.z[:, :nv].abs().amax(1, keepdim=True)
    assert float(((fused.z[:, :nv] - gen.z[:, :nv]).abs() / scale).max()) <= 1e-9
    for b in (0, 7):
        zr, okr, itr = oa.dc(oa.System(c, st, st.plan, b))
        assert okr
        assert rel(fused.z[b, :nv].cpu().numpy(), zr[:nv]) <= 1e-9
        assert int(gen.iterations[b]) == itr


@pytest.mark.parametrize("engine", ENGINES)
def test_one_singular_instance_fails_alone(engine):
    """A batch where instance 1 drives 1 mA into a node cut off from every
    DC path (its only resistor set to an infinite resistance, g = 0): only
    gmin holds that node, at 1e9 V, which damped Newton with gmin stepping
    cannot reach. That instance reports converged = False; the others
    converge to their own operating points, as voltax does per instance
    under vmap."""
    b = CircuitBuilder()
    b.vsource("in", "0", 1.0, name="Vin")
    b.resistor("in", "a", 1e3, name="R1")
    b.resistor("a", "0", 2e3, name="R2")
    b.resistor("a", "f", 5e3, name="R3")
    b.capacitor("f", "0", 1e-12, name="C1")
    b.isource("0", "f", 1e-3, name="I1")
    c = b.build()
    el = c.elements["Resistor"]
    e2 = el.with_nodes(el.nodes)
    log_r = el.log_r.expand(3, el.size).clone()
    idx = c.devices("Resistor").index("R3")
    log_r[1, idx] = float("inf")
    e2.log_r = log_r
    cb = c.replace("Resistor", e2)
    sol = vx.dc(cb, options=vx.Options(engine=engine))
    conv = sol.converged.cpu().numpy()
    assert conv.tolist() == [True, False, True]
    ref = vx.dc(c, options=vx.Options(engine=engine))
    for k in (0, 2):
        assert float((sol.z[k] - ref.z).abs().max()) < 1e-12


@pytest.mark.parametrize("side,precision", [(200, "f64"), (300, "f64"), (300, "f32")])
def test_wide_supernodes_factor_and_solve(side, precision):
    """Supernodes wider than a CTA's shared memory (grid 200: k = 164, grid
    300: k = 246) factor in place in their panels; solves equal SuperLU."""
    import scipy.sparse.linalg as sla
    c = workloads.power_grid(side, seed=1)
    st = symbolic.structure(c)
    plan = st.plan
    assert plan.k.max() > (141 if precision == "f64" else 211)
    z = np.random.default_rng(0).uniform(-0.5, 1.5, c.size)
    G = ost.add_gmin(ost.jacobian(c, st, z, 0.0), st, c.n_nodes, 1e-12)
    rhs = np.random.default_rng(1).standard_normal(c.size)
    lu = sla.splu(st.to_scipy(G).tocsc())
    fac = sparse.factor(plan, torch.as_tensor(G), precision)
    for tr in (False, True):
        x = sparse.solve(plan, fac, torch.as_tensor(rhs), tr, refine=4).cpu().numpy()
        ref = lu.solve(rhs, trans="T" if tr else "N")
        np.testing.assert_allclose(x, ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max())


def test_wide_supernodes_dc_matches_oracle():
    c = workloads.power_grid(300, seed=2)
    sol = vx.dc(c, options=vx.Options(engine="generic"))
    z_ref, ok_ref, it_ref = _oracle_dc(c)
    assert bool(sol.converged) == ok_ref
    assert rel(sol.z.cpu().numpy(), z_ref) < 1e-9
    assert int(sol.iterations) == it_ref
