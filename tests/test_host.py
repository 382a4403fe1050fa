"""Host-side logic that needs no GPU: segment declarations, AC stimulus,
option validation and the device-model host tables."""

import numpy as np
import pytest
import torch

import voltax_gb300 as vx
from voltax_gb300 import workloads
from voltax_gb300.builder import CircuitBuilder


def test_power_grid_batch_segments():
    c = workloads.power_grid_batch([4, 6, 5], seed=2)
    seg = c.unknown_segments()
    counts = np.bincount(seg)
    # nodes plus the pad currents of each grid
    assert counts.tolist() == [16 + len(workloads.grid_pads(4)), 36 + len(workloads.grid_pads(6)),
                               25 + len(workloads.grid_pads(5))]
    # each grid's segment is closed: no element joins two segments
    for name, el in c.elements.items():
        nodes = el.node_array()
        for row in nodes:
            s = {int(seg[v]) for v in row if v >= 0}
            assert len(s) <= 1, name


def test_with_segments_rejects_joined_segments():
    b = CircuitBuilder()
    b.vsource("a", "0", 1.0)
    b.resistor("a", "b", 1e3)
    b.resistor("b", "0", 1e3)
    c = b.build()
    with pytest.raises(ValueError, match="joins two segments"):
        c.with_segments([0, 1])
    with pytest.raises(ValueError, match="entries"):
        c.with_segments([0])


def test_ac_stimulus_matches_oracle_restatement():
    from oracle.analysis import _ac_stimulus
    b = CircuitBuilder()
    b.vsource("in", "0", 0.0, ac=1.0, ac_phase=30.0, name="Vin")
    b.vsource("x", "0", 1.0, name="Vdc")
    b.resistor("in", "a", 1e3)
    b.resistor("x", "a", 1e3)
    b.isource("a", "0", 0.0, ac=2.0, ac_phase=-45.0, name="I1")
    b.isource("0", "x", 0.0, ac=0.5, name="I2")
    c = b.build()
    np.testing.assert_allclose(c.ac_stimulus(), _ac_stimulus(c), rtol=0, atol=0)


def test_options_validation():
    with pytest.raises(ValueError):
        vx.Options(engine="turbo")
    with pytest.raises(ValueError):
        vx.Options(block=96)
    with pytest.raises(ValueError):
        vx.Options(precision="f16")
    assert vx.Options(refine=None).native(refine=1).refine == 1


@pytest.mark.parametrize("make", [
    lambda: vx.Diode((0, 1), is_=1e-14, n=1.5, cj=1e-12, tt=1e-9),
    lambda: vx.BJT((0, 1, 2), "pnp", vaf=50.0),
    lambda: vx.OpAmp((0, 1, 2), a0=1e4, gbw=1e7),
    lambda: vx.Switch((0, 1, 2, 3), ron=2.0, roff=1e8),
    lambda: vx.Transformer((0, 1, 2, 3), 1e-6, 4e-6, k=0.5),
    lambda: vx.Level1MOSFET((0, 1, 2, 3), smooth=0.0),
])
def test_parameter_rows_are_finite_and_differentiable(make):
    el = make()
    rows = el.gpu_params()
    assert 1 <= len(rows) <= 13
    for r in rows:
        r = torch.as_tensor(r)
        assert r.shape[-1] == el.size and bool(torch.isfinite(r).all())
    # every per-device field reaches at least one row through autograd
    for f in el.fields:
        x = getattr(el, f).detach().clone().requires_grad_(True)
        e2 = el.with_nodes(el.nodes)
        setattr(e2, f, x)
        total = sum(torch.as_tensor(r).sum() for r in e2.gpu_params())
        if total.requires_grad:
            total.backward()
            assert x.grad is not None


def test_ac_solution_accessors():
    """voltax/analysis.py:142-172 on synthetic phasors: node and device
    lookups, 20 log10 |v| and the unwrapped phase in degrees."""
    import voltax_gb300 as vx
    from voltax_gb300.analysis import ACSolution
    b = CircuitBuilder()
    b.vsource("in", "0", 0.0, ac=1.0, name="Vin")
    b.resistor("in", "out", 1e3, name="R1")
    b.capacitor("out", "0", 1e-9, name="C1")
    c = b.build()
    F = 64
    f = np.logspace(1, 8, F)
    ang = np.linspace(0.0, -3.5 * np.pi, F)  # wraps past -pi twice
    mag = np.logspace(0, -3, F)
    z = np.zeros((F, c.size), complex)
    out = c.layout.node("out")
    z[:, out] = mag * np.exp(1j * ang)
    z[:, c.layout.internal("Vin")] = 2.0 - 1.0j
    s = ACSolution(torch.as_tensor(f), torch.as_tensor(z), None, c.layout)
    np.testing.assert_allclose(s.db("out").numpy(), 20 * np.log10(mag), rtol=1e-12)
    np.testing.assert_allclose(s.phase("out").numpy(), np.rad2deg(ang), atol=1e-9)
    wrapped = np.rad2deg(np.angle(np.exp(1j * ang)))
    np.testing.assert_allclose(s.phase("out", unwrap=False).numpy(), wrapped, atol=1e-9)
    assert torch.equal(s.v("0"), torch.zeros(F, dtype=torch.complex128))
    assert s.v().shape == (F, c.n_nodes)
    assert torch.all(s.i("Vin") == torch.tensor(2.0 - 1.0j))
    assert isinstance(vx.ac, type(vx.dc))


def test_solution_accessors_and_check():
    """voltax/analysis.py:92-139: lookups by node / device name, and check()
    raising voltax's RuntimeError (with the first failing time) on
    non-convergence or non-finite states."""
    from voltax_gb300.analysis import Solution
    b = CircuitBuilder()
    b.vsource("in", "0", 1.0, name="Vin")
    b.resistor("in", "out", 1e3, name="R1")
    b.resistor("out", "0", 1e3, name="R2")
    c = b.build()
    T = 4
    z = torch.arange(T * c.size, dtype=torch.float64).reshape(T, c.size)
    ok = torch.ones(T, dtype=torch.int32)
    s = Solution(torch.tensor([0.0, 1e-9, 2e-9, 3e-9], dtype=torch.float64), z, ok, c.layout)
    assert s.check() is s
    assert torch.equal(s["out"], z[:, c.layout.node("out")])
    assert torch.equal(s["Vin.i"], z[:, c.layout.internal("Vin", "i")])
    assert torch.equal(s.v("gnd"), torch.zeros(T, dtype=torch.float64))
    bad = ok.clone()
    bad[2] = 0
    with pytest.raises(RuntimeError, match=r"did not converge at t=2e-09"):
        Solution(s.t, z, bad, c.layout).check()
    z2 = z.clone()
    z2[1, 0] = float("nan")
    with pytest.raises(RuntimeError, match="did not converge"):
        Solution(s.t, z2, ok, c.layout).check()


def test_layout_state_names_and_group_internals():
    """voltax/circuit.py:92-107: labels of every state entry and the internal
    indices of a group."""
    b = CircuitBuilder()
    b.vsource("in", "0", 1.0, name="Vin")
    b.inductor("in", "mid", 1e-6, name="L1")
    b.inductor("mid", "out", 2e-6, name="L2")
    b.resistor("out", "0", 50.0, name="R1")
    c = b.build()
    names = c.layout.state_names()
    assert len(names) == c.size
    assert names[:c.n_nodes] == [f"v({n})" for n in c.layout.node_names]
    for dev in ("Vin", "L1", "L2"):
        assert names[c.layout.internal(dev)] == f"i({dev})"
    idx = c.layout.group_internals("Inductor")
    assert idx.shape == (2, 1)
    assert [int(i) for i in idx[:, 0]] == [c.layout.internal("L1"), c.layout.internal("L2")]


def test_time_grid_properties():
    """voltax/analysis.py:575-620 on the host: every waveform corner is a
    grid point, each interval holds at least `ramp_points` steps, steps never
    exceed `dt_max`, and steps grow by at most `growth` after a corner."""
    import voltax_gb300 as vx
    from voltax_gb300.signals import Pulse, Step
    b = CircuitBuilder()
    b.vsource("in", "0", Pulse(0.0, 1.0, delay=1e-9, rise=1e-10, fall=2e-10, width=2e-9,
                               period=5e-9), name="V1")
    b.isource("x", "0", Step(0.0, 1e-3, delay=2.5e-9, rise=5e-11), name="I1")
    b.resistor("in", "x", 1e3, name="R1")
    b.capacitor("x", "0", 1e-12, name="C1")
    c = b.build()
    t_stop, dt_max, ramp, growth = 12e-9, 0.5e-9, 10, 1.2
    grid = vx.time_grid(c, t_stop, dt_max=dt_max, ramp_points=ramp, growth=growth)
    corners = np.unique(np.concatenate(
        [[0.0, t_stop], c.elements["VoltageSource_Pulse"].value.breakpoints(t_stop),
         c.elements["CurrentSource_Step"].value.breakpoints(t_stop)]))
    assert grid[0] == 0.0 and grid[-1] == t_stop and np.all(np.diff(grid) > 0)
    for t in corners:
        assert np.min(np.abs(grid - t)) <= 1e-9 * 1e-12
    steps = np.diff(grid)
    assert steps.max() <= dt_max * (1 + 1e-12)
    for a, z in zip(corners[:-1], corners[1:]):
        inside = (grid > a) & (grid <= z)
        assert inside.sum() >= ramp
        s = np.diff(np.concatenate([[a], grid[inside]]))
        assert np.all(s[1:-1] <= s[:-2] * growth * (1 + 1e-12))
    # a pulse corner every period: 1, 1.1, 3.1, 3.3 ns and again 5 ns later
    for t in (1e-9, 1.1e-9, 3.1e-9, 3.3e-9, 6e-9, 6.1e-9, 8.1e-9, 8.3e-9, 2.5e-9, 2.55e-9):
        assert np.min(np.abs(grid - t)) < 1e-18


def test_builder_group_fusion_and_naming_rule():
    """Group names the state layout depends on: explicit groups keep their
    names; automatic groups take base, base_2, base_3, ... in order of their
    first device, skipping names already in use; node indices follow first
    appearance; devices of one explicit group must be fusable."""
    import pytest
    from voltax_gb300 import elements as el
    from voltax_gb300.builder import CircuitBuilder
    from voltax_gb300.signals import Step
    other = el.MOSProcess.nmos(vth=0.3)  # a second process: a second nmos group
    b = CircuitBuilder()
    b.nmos("d1", "g", "0")                          # bucket A: EKVMOSFET_n
    b.resistor("d1", "x", 1e3, group="EKVMOSFET_n_2")  # explicit, takes _2
    b.nmos("d2", "g", "0", process=other)             # bucket B: _2 taken -> _3
    b.vsource("g", "0", Step(0.0, 1.0, 1e-9, 1e-10))  # VoltageSource_Step
    b.vsource("vdd", "0", 1.2)                        # VoltageSource
    with b.scope("blk"):
        inner = b.node("mid")
        b.capacitor(inner, "0", 1e-15)
    c = b.build()
    names = sorted(c.elements)
    assert type(c.elements["EKVMOSFET_n_2"]).__name__ == "Resistor"
    assert c.layout.device("M1") == ("EKVMOSFET_n", 0)
    assert c.layout.device("M2") == ("EKVMOSFET_n_3", 0)
    assert "VoltageSource_Step" in names and "VoltageSource" in names
    assert c.layout.node_names[:3] == ("d1", "g", "x")
    assert inner == "blk.mid" and "blk.mid" in c.layout.node_names
    assert c.devices("Capacitor") == ["blk.C1"]
    with pytest.raises(ValueError, match="cannot be fused"):
        b2 = CircuitBuilder()
        b2.resistor("a", "0", 1.0, group="mix")
        b2.capacitor("a", "0", 1e-12, group="mix")
        b2.build()
    with pytest.raises(ValueError, match="duplicate device name"):
        b3 = CircuitBuilder()
        b3.resistor("a", "0", 1.0, name="R")
        b3.resistor("b", "0", 1.0, name="R")
