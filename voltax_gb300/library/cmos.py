"""Static CMOS gates and arithmetic blocks (voltax/library/cmos.py).

NMOS bulks tie to `gnd`, PMOS bulks to `vdd`; a series stack of ``k``
devices is widened ``k``-fold. `mirror_full_adder` / `mirror_ripple_adder`
(the 28-transistor mirror adder) have no voltax counterpart: voltax's
`full_adder` is NAND/XOR based (50 transistors). They are written here with
the same builder calls so the batched Monte Carlo workload uses the classic
mirror topology.
"""

from __future__ import annotations

from typing import Sequence

from ..builder import CircuitBuilder

WN, WP = 1e-6, 2e-6
"""Default NMOS / PMOS widths (m) of a unit inverter."""


def inverter(b: CircuitBuilder, a, y, vdd, gnd="0", wn=WN, wp=WP) -> None:
    """``y = not a`` (cmos.py:27-31)."""
    b.pmos(y, a, vdd, vdd, w=wp)
    b.nmos(y, a, gnd, gnd, w=wn)


def nand(b: CircuitBuilder, inputs: Sequence[str], y, vdd, gnd="0", wn=WN,
         wp=WP) -> None:
    """Parallel PMOS, series NMOS (cmos.py:34-44)."""
    k = len(inputs)
    for a in inputs:
        b.pmos(y, a, vdd, vdd, w=wp)
    lower = gnd
    for i, a in enumerate(inputs):
        upper = y if i == k - 1 else b.node()
        b.nmos(upper, a, lower, gnd, w=k * wn)
        lower = upper


def nor(b: CircuitBuilder, inputs: Sequence[str], y, vdd, gnd="0", wn=WN,
        wp=WP) -> None:
    """Series PMOS, parallel NMOS (cmos.py:47-57)."""
    k = len(inputs)
    for a in inputs:
        b.nmos(y, a, gnd, gnd, w=wn)
    upper = vdd
    for i, a in enumerate(inputs):
        lower = y if i == k - 1 else b.node()
        b.pmos(lower, a, upper, vdd, w=k * wp)
        upper = lower


def and_(b, inputs, y, vdd, gnd="0", **sizes) -> None:
    mid = b.node()
    nand(b, inputs, mid, vdd, gnd, **sizes)
    inverter(b, mid, y, vdd, gnd, **sizes)


def or_(b, inputs, y, vdd, gnd="0", **sizes) -> None:
    mid = b.node()
    nor(b, inputs, mid, vdd, gnd, **sizes)
    inverter(b, mid, y, vdd, gnd, **sizes)


def xor(b, a, c, y, vdd, gnd="0", **sizes) -> None:
    """Four NAND2 gates (cmos.py:76-83)."""
    n1, n2, n3 = b.node(), b.node(), b.node()
    nand(b, [a, c], n1, vdd, gnd, **sizes)
    nand(b, [a, n1], n2, vdd, gnd, **sizes)
    nand(b, [c, n1], n3, vdd, gnd, **sizes)
    nand(b, [n2, n3], y, vdd, gnd, **sizes)


def full_adder(b, a, c, cin, s, cout, vdd, gnd="0", **sizes) -> None:
    """NAND/XOR full adder, 50 transistors (cmos.py:86-94)."""
    p, g, t = b.node(), b.node(), b.node()
    xor(b, a, c, p, vdd, gnd, **sizes)
    xor(b, p, cin, s, vdd, gnd, **sizes)
    and_(b, [a, c], g, vdd, gnd, **sizes)
    and_(b, [cin, p], t, vdd, gnd, **sizes)
    or_(b, [g, t], cout, vdd, gnd, **sizes)


def ripple_adder(b, a, c, cin, s, cout, vdd, gnd="0", **sizes) -> None:
    """``k``-bit ripple-carry adder of `full_adder` (cmos.py:97-108)."""
    if not len(a) == len(c) == len(s):
        raise ValueError("a, c and s must have the same width")
    carry = cin
    for i in range(len(a)):
        nxt = cout if i == len(a) - 1 else b.node()
        with b.scope(f"fa{i}"):
            full_adder(b, a[i], c[i], carry, s[i], nxt, vdd, gnd, **sizes)
        carry = nxt


def ring_oscillator(b, nodes: Sequence[str], vdd, gnd="0", **sizes) -> None:
    """Ring of ``len(nodes)`` inverters (odd count) (cmos.py:111-118)."""
    if len(nodes) % 2 == 0:
        raise ValueError("a ring oscillator needs an odd number of stages")
    for i, a in enumerate(nodes):
        inverter(b, a, nodes[(i + 1) % len(nodes)], vdd, gnd, **sizes)


def mirror_full_adder(b: CircuitBuilder, a, c, cin, s, cout, vdd, gnd="0",
                      wn=WN, wp=WP) -> None:
    """28-transistor mirror full adder.

    ``cob = not(a c + cin (a + c))`` with mirrored pull-up / pull-down
    networks (10 devices), ``sb = not(a c cin + cob (a + c + cin))`` (14
    devices), then output inverters ``cout = not cob`` and ``s = not sb``.
    Devices in a 2-stack are 2x wide, in a 3-stack 3x.
    """
    cob, sb = b.node(), b.node()
    x, y, xn, yn = b.node(), b.node(), b.node(), b.node()
    # carry: pull-up (a || c) -- cin, plus a -- c
    b.pmos(x, a, vdd, vdd, w=2 * wp)
    b.pmos(x, c, vdd, vdd, w=2 * wp)
    b.pmos(cob, cin, x, vdd, w=2 * wp)
    b.pmos(y, a, vdd, vdd, w=2 * wp)
    b.pmos(cob, c, y, vdd, w=2 * wp)
    # carry: mirrored pull-down
    b.nmos(xn, a, gnd, gnd, w=2 * wn)
    b.nmos(xn, c, gnd, gnd, w=2 * wn)
    b.nmos(cob, cin, xn, gnd, w=2 * wn)
    b.nmos(yn, a, gnd, gnd, w=2 * wn)
    b.nmos(cob, c, yn, gnd, w=2 * wn)
    # sum: pull-up (a || c || cin) -- cob, plus a -- c -- cin
    z, w1, w2 = b.node(), b.node(), b.node()
    for g in (a, c, cin):
        b.pmos(z, g, vdd, vdd, w=2 * wp)
    b.pmos(sb, cob, z, vdd, w=2 * wp)
    b.pmos(w1, a, vdd, vdd, w=3 * wp)
    b.pmos(w2, c, w1, vdd, w=3 * wp)
    b.pmos(sb, cin, w2, vdd, w=3 * wp)
    # sum: mirrored pull-down
    zn, v1, v2 = b.node(), b.node(), b.node()
    for g in (a, c, cin):
        b.nmos(zn, g, gnd, gnd, w=2 * wn)
    b.nmos(sb, cob, zn, gnd, w=2 * wn)
    b.nmos(v1, a, gnd, gnd, w=3 * wn)
    b.nmos(v2, c, v1, gnd, w=3 * wn)
    b.nmos(sb, cin, v2, gnd, w=3 * wn)
    inverter(b, cob, cout, vdd, gnd, wn, wp)
    inverter(b, sb, s, vdd, gnd, wn, wp)


def mirror_ripple_adder(b, a, c, cin, s, cout, vdd, gnd="0", **sizes) -> None:
    """``k``-bit ripple-carry adder of `mirror_full_adder` (LSB first)."""
    if not len(a) == len(c) == len(s):
        raise ValueError("a, c and s must have the same width")
    carry = cin
    for i in range(len(a)):
        nxt = cout if i == len(a) - 1 else b.node()
        with b.scope(f"fa{i}"):
            mirror_full_adder(b, a[i], c[i], carry, s[i], nxt, vdd, gnd, **sizes)
        carry = nxt
