"""Small test circuits shared by the test modules."""

from voltax_gb300.builder import CircuitBuilder


def mixed_circuit():
    """A pulse through R and a series-RL into C, a diode (junction and
    diffusion charge) to a load, and a VCCS sensing the capacitor."""
    from voltax_gb300.signals import Pulse
    b = CircuitBuilder()
    b.vsource("in", "0", Pulse(0.0, 1.0, delay=5e-12, rise=10e-12, fall=10e-12,
                               width=60e-12, period=200e-12), name="Vin")
    b.resistor("in", "a", 50.0, name="R1")
    b.inductor("a", "b", 2e-9, rs=5.0, name="L1")
    b.capacitor("b", "0", 0.5e-12, name="C1")
    b.diode("b", "c", name="D1", is_=1e-14, n=1.2, cj=0.1e-12, tt=2e-12)
    b.resistor("c", "0", 200.0, name="R2")
    b.vccs("d", "0", "b", "0", 2e-3, name="G1")
    b.resistor("d", "0", 1e3, name="R3")
    return b.build()


def bjt_amplifier():
    """A common-emitter NPN stage (emitter degeneration, Early effect,
    junction and transit charges) with a PNP current-mirror load, driven by a
    pulse through a coupling RC."""
    from voltax_gb300.signals import Pulse
    b = CircuitBuilder()
    b.vsource("vcc", "0", 5.0, name="Vcc")
    b.vsource("in", "0", Pulse(0.0, 0.2, delay=1e-9, rise=1e-9, fall=1e-9, width=5e-9,
                               period=20e-9), name="Vin")
    b.resistor("in", "x", 1e3, name="Rs")
    b.capacitor("x", "base", 1e-9, name="Cc")
    b.resistor("vcc", "base", 100e3, name="Rb1")
    b.resistor("base", "0", 20e3, name="Rb2")
    kw = dict(is_=1e-15, bf=120.0, br=2.0, vaf=60.0, tf=0.3e-9, tr=5e-9, cje=1e-12, cjc=0.5e-12)
    b.bjt("out", "base", "emit", "npn", name="Q1", **kw)
    b.resistor("emit", "0", 500.0, name="Re")
    b.bjt("mir", "mir", "vcc", "pnp", name="Q2", **kw)
    b.bjt("out", "mir", "vcc", "pnp", name="Q3", **kw)
    b.resistor("mir", "0", 20e3, name="Rref")
    b.capacitor("out", "0", 0.2e-12, name="CL")
    return b.build()


def controlled_sources_circuit():
    """A chain through every linear controlled source and a transformer:
    RC input -> VCVS (x2) -> CCCS sensing through a zero-volt ammeter ->
    CCVS sensing another branch -> series R into a transformer primary,
    resistive secondary load."""
    from voltax_gb300.signals import Pulse
    b = CircuitBuilder()
    b.vsource("in", "0", Pulse(0.0, 1.0, delay=1e-9, rise=1e-9, fall=1e-9, width=5e-9,
                               period=20e-9), ac=1.0, name="Vin")
    b.resistor("in", "a", 1e3, name="R1")
    b.capacitor("a", "0", 1e-12, name="C1")
    b.vcvs("b", "0", "a", "0", 2.0, name="E1")
    b.cccs("c", "0", "b", "b2", 0.5, name="F1")
    b.resistor("b2", "0", 2e3, name="R2")
    b.resistor("c", "0", 1e3, name="R3")
    b.ccvs("d", "0", "c", "c2", 500.0, name="H1")
    b.resistor("c2", "0", 500.0, name="R4")
    b.resistor("d", "d2", 100.0, name="R7")
    b.transformer("d2", "0", "e", "0", 1e-6, 4e-6, k=0.9, name="K1")
    b.resistor("e", "0", 50.0, name="R6")
    b.capacitor("e", "0", 1e-12, name="C2")
    return b.build()


def opamp_switch_circuit():
    """An ideal-op-amp inverting amplifier feeding a single-pole op-amp
    integrator-follower, and a smoothed switch that a pulse opens and closes
    between the output and an RC load."""
    from voltax_gb300.signals import Pulse
    b = CircuitBuilder()
    b.vsource("in", "0", Pulse(-0.2, 0.3, delay=0.2e-6, rise=0.1e-6, fall=0.1e-6,
                               width=1e-6, period=3e-6), name="Vin")
    b.resistor("in", "m", 1e3, name="R1")
    b.resistor("m", "a", 4e3, name="R2")
    b.ideal_opamp("0", "m", "a", name="U1")
    b.opamp("a", "o", "o", name="U2", a0=1e4, gbw=5e6, rout=10.0, vmin=-1.5, vmax=1.5)
    b.vsource("ctl", "0", Pulse(0.0, 1.0, delay=0.5e-6, rise=50e-9, fall=50e-9, width=0.8e-6,
                                period=3e-6), name="Vctl")
    b.switch("o", "s", "ctl", "0", name="S1", ron=10.0, roff=1e7, vth=0.5, vwidth=0.05)
    b.resistor("s", "0", 1e3, name="R3")
    b.capacitor("s", "0", 1e-10, name="C1")
    return b.build()


def grid_via_builder(n, seed=0, prefix="", b=None, sigma=0.3, sink_max=1e-3, vpad=1.0):
    """A power grid added to a `CircuitBuilder` device by device: the
    construction `workloads.power_grid` reproduces from arrays."""
    import numpy as np

    from voltax_gb300.workloads import grid_pads
    own = b is None
    b = CircuitBuilder() if own else b
    rng = np.random.default_rng(seed)
    node = lambda i, j: f"{prefix}n{i}_{j}"  # noqa: E731
    edges = []
    for i in range(n):
        for j in range(n):
            if j + 1 < n:
                edges.append((node(i, j), node(i, j + 1)))
            if i + 1 < n:
                edges.append((node(i, j), node(i + 1, j)))
    g = np.exp(rng.normal(0.0, sigma, len(edges)))
    for k, (a, c) in enumerate(edges):
        b.resistor(a, c, 1.0 / g[k], name=f"{prefix}R{k}")
    sinks = rng.uniform(0.0, sink_max, n * n)
    for p in range(n * n):
        b.isource(node(p // n, p % n), "0", sinks[p], name=f"{prefix}I{p}")
    for k, (i, j) in enumerate(grid_pads(n)):
        b.vsource(node(i, j), "0", vpad, name=f"{prefix}Vpad{k}")
    return b.build() if own else b


def coupled_circuit(k=0.5):
    """Three inductors sharing one mutual-inductance matrix (a non-local
    group) behind a stepped source and resistors: nodes in=0, a=1, b=2, c=3
    (the circuit of voltax tests/test_sparse.py:116-123)."""
    import torch
    import voltax_gb300 as vx
    from voltax_gb300 import signals
    return vx.Circuit({
        "V": vx.VoltageSource((0, -1), signals.Step(0.0, 1.0, delay=1e-6, rise=1e-7)),
        "R": vx.Resistor([(0, 1), (2, -1), (3, -1)], torch.tensor([10.0, 100.0, 1e3])),
        "K": vx.CoupledInductors([(1, -1), (2, -1), (3, -1)], 1e-3, k=k),
    }, ["in", "a", "b", "c"])
