"""dc_sweep (continuation) and time_grid, after voltax tests/test_analysis.py:262-308."""

import numpy as np
import pytest
import torch

import voltax_gb300 as vx
from voltax_gb300.builder import CircuitBuilder
from voltax_gb300.signals import Pulse


def _rc_pulse():
    b = CircuitBuilder()
    b.vsource("in", "0", Pulse(0, 1, delay=1e-9, rise=1e-11, fall=1e-11, width=4e-9,
                               period=10e-9), name="Vin")
    b.resistor("in", "out", 1e3, name="R1")
    b.capacitor("out", "0", 1e-13, name="C1")
    return b.build()


def test_time_grid_resolves_edges():
    """voltax tests/test_analysis.py:291-302 (the grid part)."""
    grid = vx.time_grid(_rc_pulse(), 6e-9, dt_max=0.5e-9)
    steps = np.diff(grid)
    assert grid[0] == 0 and np.isclose(grid[-1], 6e-9) and steps.max() <= 0.5e-9 * (1 + 1e-12)
    assert np.all(steps > 0)
    on_ramp = (grid >= 1e-9) & (grid <= 1.01e-9)
    assert on_ramp.sum() >= 11  # >= 10 steps across the 10 ps edge
    assert len(grid) < 200


def _crossing(t, y, level, after=-np.inf):
    for i in range(len(t) - 1):
        if t[i + 1] <= after:
            continue
        a, b = y[i] - level, y[i + 1] - level
        if a == 0 or a * b < 0:
            return t[i] + (t[i + 1] - t[i]) * (a / (a - b))
    return np.nan


@pytest.mark.gpu
def test_time_grid_transient_delay_matches_fine_grid():
    """voltax tests/test_analysis.py:303-308: the 50 % delay on the refined
    grid equals the one on a uniform 100 fs grid within 0.5 %."""
    c = _rc_pulse()
    grid = vx.time_grid(c, 6e-9, dt_max=0.5e-9)

    def delay(ts):
        sol = vx.transient(c, ts, method="trap")
        vin, vout = sol.v("in").cpu().numpy(), sol.v("out").cpu().numpy()
        t0 = _crossing(ts, vin, 0.5)
        return _crossing(ts, vout, 0.5, after=t0) - t0

    fine = np.linspace(0, 6e-9, 60001)
    assert np.isclose(delay(grid), delay(fine), rtol=5e-3)


def _rc_ladder():
    b = CircuitBuilder()
    b.vsource("in", "0", 1.0, name="Vin")
    b.resistor("in", "a", 1e3, name="R1")
    b.resistor("a", "out", 2e3, name="R2")
    b.resistor("out", "0", 1e4, name="Rload")
    return b.build()


@pytest.mark.gpu
def test_dc_sweep_with_callable_and_gradient():
    """voltax tests/test_analysis.py:276-288."""
    c = _rc_ladder()

    def out_sum(log_r):
        sweep = vx.dc_sweep(c, [1e3, 1e4],
                            lambda cc, r: cc.set("Rload", r=r * torch.exp(log_r)))
        return sweep.v("out").sum()

    expected = sum(r / (r + 3e3) for r in (1e3, 1e4))
    x = torch.zeros((), dtype=torch.float64, requires_grad=True)
    val = out_sum(x)
    assert np.isclose(val.item(), expected)
    val.backward()
    h = 1e-6
    with torch.no_grad():
        fd = (out_sum(torch.tensor(h, dtype=torch.float64)).item() -
              out_sum(torch.tensor(-h, dtype=torch.float64)).item()) / (2 * h)
    assert np.isclose(float(x.grad), fd, rtol=1e-5)


def _latch():
    """Cross-coupled CMOS inverters; the input drives node a through 600 Ohm,
    so the latch keeps its state until the input overpowers it (the oracle
    switches between 0.9 and 1.0 V going up, 0.4 and 0.3 V going down)."""
    b = CircuitBuilder()
    b.vsource("vdd", "0", 1.2, name="Vdd")
    b.vsource("in", "0", 0.0, name="Vin")
    b.resistor("in", "a", 600.0, name="Rin")
    from voltax_gb300.library import cmos
    cmos.inverter(b, "a", "q", "vdd")
    cmos.inverter(b, "q", "a", "vdd")
    return b.build()


@pytest.mark.gpu
def test_dc_sweep_follows_branches_and_shows_hysteresis():
    """voltax tests/test_analysis.py:262-273 with a CMOS latch."""
    c = _latch()
    vin = np.linspace(0.0, 1.2, 49)
    up = vx.dc_sweep(c, vin, "Vin")
    down = vx.dc_sweep(c, vin[::-1], "Vin", guess=up.z[-1])
    assert bool(up.converged.all()) and bool(down.converged.all())
    assert np.allclose(up.t.numpy(), vin)
    q_up, q_down = up.v("q").cpu().numpy(), down.v("q").cpu().numpy()[::-1]
    assert q_up[0] > 1.1 and q_up[-1] < 0.1  # the input wins at both ends
    mid = len(vin) // 2
    assert q_up[mid] > 1.0 and q_down[mid] < 0.2  # two stable states at VDD/2
    # every point is a DC operating point of its own input (no branch mixing)
    for k in (5, mid, 40):
        s = vx.dc(c.set("Vin", value=float(vin[k])), guess=up.z[k])
        assert float((s.z - up.z[k]).abs().max()) < 1e-9


@pytest.mark.gpu
def test_dc_sweep_schmitt_trigger_hysteresis():
    """voltax tests/test_analysis.py:252-273, verbatim circuit: inverting
    Schmitt trigger with thresholds at +-vmax R2/(R1+R2) = +-0.5 V."""
    b = CircuitBuilder()
    b.vsource("in", "0", 0.0, name="Vin")
    b.opamp("p", "in", "out", a0=1e3, vmin=-1.0, vmax=1.0)
    b.resistor("out", "p", 10e3)
    b.resistor("p", "0", 10e3)
    c = b.build()
    vin = np.linspace(-1, 1, 81)
    up = vx.dc_sweep(c, vin, "Vin")
    down = vx.dc_sweep(c, vin[::-1], "Vin", guess=up.z[-1])
    assert bool(up.converged.all()) and bool(down.converged.all())
    out_up, out_dn = up.v("out").cpu().numpy(), down.v("out").cpu().numpy()
    assert out_up[40] > 0.9 and out_dn[40] < -0.9  # two stable states at 0 V
    rise_thr = _crossing(vin, out_up, 0.0)
    fall_thr = -_crossing(-vin[::-1], out_dn, 0.0)
    assert 0.4 < rise_thr < 0.55 and -0.55 < fall_thr < -0.4


@pytest.mark.gpu
def test_dc_sweep_in_one_launch_matches_point_by_point():
    """A swept DC source on the fused engine runs the whole continuation in
    one persistent launch (vxg_fused_sweep); it gives the iterates of the
    point-by-point sweep bit for bit and leaves the circuit untouched."""
    from voltax_gb300 import _lib
    lib = _lib.load()
    c = _latch()
    o = vx.Options(engine="fused")
    vin = np.linspace(0.0, 1.2, 25)
    vx.dc(c, options=o)  # settle the launch-shape choice
    n0 = lib.vxg_launch_count()
    fast = vx.dc_sweep(c, vin, "Vin", options=o)
    launches = lib.vxg_launch_count() - n0
    slow = vx.dc_sweep(c, vin, lambda cc, v: cc.set("Vin", value=v), options=o)
    assert launches == 1
    assert bool(fast.converged.all()) and torch.equal(fast.converged, slow.converged)
    assert torch.equal(fast.iterations, slow.iterations)
    assert torch.equal(fast.z, slow.z)
    el, idx = c.device("Vin")
    assert float(el.value.value.reshape(-1)[idx]) == 0.0
    # down again from the top, continuing the upper branch
    down_fast = vx.dc_sweep(c, vin[::-1], "Vin", guess=fast.z[-1], options=o)
    down_slow = vx.dc_sweep(c, vin[::-1], lambda cc, v: cc.set("Vin", value=v),
                            guess=slow.z[-1], options=o)
    assert torch.equal(down_fast.z, down_slow.z)
