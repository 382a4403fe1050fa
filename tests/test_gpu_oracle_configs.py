"""The benchmarked configurations against the FP64 oracle, at their own sizes.

Each test runs one benchmark workload through the public API on the GPU and
checks every instance and every time point against the compiled oracle
(oracle/cvx.c) run on the same inputs:

* node voltages within 1e-9 relative (|v - v_ref| <= 1e-9 max(|v_ref|, 1 mV));
* the same convergence flags, and in the plain FP64 form the same Newton
  iteration counts;
* the acceptance test of the reference at the GPU's own solution: the
  oracle evaluates the FP64 residual r(z*) (the KCL residual on node rows)
  and one more Newton step dz = -J(z*)^-1 r(z*), and every unknown must pass
  voltax's convergence test |dz| <= atol + rtol |z*|
  (voltax/analysis.py:224-229, rtol 1e-6, atol 1e-9).

Workloads: the 101-stage EKV ring oscillator, trapezoidal, all 2001 points;
the 4-bit mirror-adder Monte Carlo (8 instances of the 4096-instance draw)
over all 501 backward-Euler points, both precisions, on the generic engine
and the fused kernel with one CTA or one warp per instance; the
100 x 100 power grid DC; and the first four grids of the 512-grid uneven
batch (sides 263, 209, 178, 117), solved as one segmented batch on the GPU
and each alone by the oracle.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from oracle import cbase  # noqa: E402
import voltax_gb300 as vx  # noqa: E402
from voltax_gb300 import symbolic, workloads  # noqa: E402

TOL = 1e-9      # node voltages, relative
FLOOR = 1e-3    # V: below 1 mV the bound is absolute (1e-12 V)
RTOL, ATOL = 1e-6, 1e-9


def node_rel(z, z_ref, nv):
    a, b = np.asarray(z)[..., :nv], np.asarray(z_ref)[..., :nv]
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), FLOOR)))


def accept(csys, ts, z, method, dc_first):
    """Largest KCL residual (A) and largest Newton-step ratio over a trajectory."""
    kcl, ratio = csys.check(ts, z, method=method, dc_first=dc_first, rtol=RTOL, atol=ATOL)
    return float(np.max(kcl)), float(np.max(ratio))


@pytest.mark.parametrize("block", [0, 32], ids=["auto", "fused-warp"])
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_ring101_trapezoidal_2001_points_matches_oracle(precision, block):
    ring, nodes = workloads.ring_oscillator(101)
    z0 = workloads.ring_initial_state(ring, nodes)
    ts = np.linspace(0.0, 2e-9, 2001)
    engine = "fused" if block else "auto"
    sol = vx.transient(ring, ts, ic=z0, method="trap",
                       options=vx.Options(precision=precision, engine=engine, block=block))
    z = sol.z.cpu().numpy()
    st = symbolic.structure(ring)
    cs = cbase.CSystem(ring, st, st.plan)
    zr, okr, itr = cs.run(ts, z0=z0.numpy(), method="trap", dc_first=False)
    assert okr[1:].all() and bool(sol.converged[1:].all())
    err = node_rel(z, zr, ring.n_nodes)
    assert err <= TOL, f"ring101 node voltages differ by {err:.3e} relative"
    if precision == "f64":
        assert np.array_equal(sol.iterations.cpu().numpy()[1:], itr[1:])
    kcl, ratio = accept(cs, ts, z, "trap", dc_first=False)
    assert ratio <= 1.0, f"ring101 fails the convergence test at its solution: {ratio:.3e}"
    assert kcl < 1e-9, f"ring101 KCL residual {kcl:.3e} A"


@pytest.mark.parametrize("engine,block", [("fused", 128), ("fused", 32), ("generic", 0)],
                         ids=["fused-cta", "fused-warp", "generic"])
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_mirror_adder_mc_501_points_matches_oracle(precision, engine, block):
    B = 8
    c = workloads.mirror_adder_mc(B, seed=0)
    ts = np.linspace(0.0, 1e-9, 501)
    sol = vx.transient(c, ts, ic="dc", method="be",
                       options=vx.Options(precision=precision, engine=engine, block=block))
    z = sol.z.cpu().numpy()
    its = sol.iterations.cpu().numpy().reshape(B, len(ts))
    conv = sol.converged.cpu().numpy().reshape(B, len(ts))
    st = symbolic.structure(c)
    worst_err = worst_ratio = worst_kcl = 0.0
    for b in range(B):
        cs = cbase.CSystem(c, st, st.plan, b)
        zr, okr, itr = cs.run(ts, method="be", dc_first=True)
        assert okr.all() and conv[b].all()
        worst_err = max(worst_err, node_rel(z[b], zr, c.n_nodes))
        if precision == "f64":
            assert np.array_equal(its[b], itr), f"instance {b}: iteration counts differ"
        kcl, ratio = accept(cs, ts, z[b], "be", dc_first=True)
        worst_ratio, worst_kcl = max(worst_ratio, ratio), max(worst_kcl, kcl)
    assert worst_err <= TOL, f"adder node voltages differ by {worst_err:.3e} relative"
    assert worst_ratio <= 1.0, f"adder fails the convergence test: {worst_ratio:.3e}"
    assert worst_kcl < 1e-9, f"adder KCL residual {worst_kcl:.3e} A"


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_power_grid_100_dc_matches_oracle(precision):
    c = workloads.power_grid(100, seed=0)
    sol = vx.dc(c, options=vx.Options(precision=precision))
    z = sol.z.cpu().numpy()
    st = symbolic.structure(c)
    cs = cbase.CSystem(c, st, st.plan)
    ts = np.zeros(1)
    zr, okr, itr = cs.run(ts, dc_first=True)
    assert okr.all() and bool(sol.converged)
    err = node_rel(z, zr[0], c.n_nodes)
    assert err <= TOL, f"grid100 node voltages differ by {err:.3e} relative"
    if precision == "f64":
        assert int(sol.iterations) == int(itr[0])
    kcl, ratio = accept(cs, ts, z[None], "dc", dc_first=True)
    assert ratio <= 1.0 and kcl < 1e-9, (kcl, ratio)


def test_uneven_grid_batch_matches_oracle_grid_by_grid():
    sides = workloads.grid_sides(512, 50, 300, seed=0)[:4]
    assert sides == [263, 209, 178, 117]
    cb = workloads.power_grid_batch(sides, seed=0)
    sol = vx.dc(cb, options=vx.Options(precision="f32"))
    assert bool(sol.converged.all())
    zb = sol.z.cpu().numpy()
    for k, n in enumerate(sides):
        c = workloads.power_grid(n, seed=k)
        idx = [cb.node(f"g{k}_{nm}") for nm in c.layout.node_names]
        st = symbolic.structure(c)
        cs = cbase.CSystem(c, st, st.plan)
        ts = np.zeros(1)
        zr, okr, _ = cs.run(ts, dc_first=True)
        assert okr.all()
        v = zb[idx]
        err = node_rel(v, zr[0], c.n_nodes)
        assert err <= TOL, f"grid {k} (side {n}) differs by {err:.3e} relative"
        # the oracle's acceptance test on the grid's own unknowns: node
        # voltages and pad currents taken from the batch solution
        z_k = np.empty(c.size)
        z_k[: c.n_nodes] = v
        pads = c.devices("VoltageSource")
        z_k[[c.layout.internal(p) for p in pads]] = \
            zb[[cb.layout.internal(f"g{k}_{p}") for p in pads]]
        kcl, ratio = accept(cs, ts, z_k[None], "dc", dc_first=True)
        assert ratio <= 1.0 and kcl < 1e-9, (k, kcl, ratio)
    torch.cuda.synchronize()
