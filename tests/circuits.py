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
