"""`CircuitBuilder`: describe a circuit device by device with named nodes
(the interface of voltax/builder.py:52-256).

The circuit's state layout depends on how devices are fused into element
groups and what the groups are called (groups are laid out in sorted-name
order), so `build` follows voltax's rule exactly:

1. Node indices follow the first appearance of each non-ground node name,
   in the order devices were added (or nodes declared with `node`).
2. A device joins the group it was given explicitly, else the automatic
   group of its fusion key (element type + static configuration). Devices
   in one explicit group must share a fusion key.
3. Explicit groups keep their names. Automatic groups are named afterwards,
   in order of their first device: the base name is the class name, with
   ``_<polarity>`` for transistors or ``_<waveform class>`` for sources
   with a non-constant waveform. Each base has a cursor over the names
   ``base, base_2, base_3, ...``: a group takes the first name at or after
   the cursor that no group has yet, and the cursor moves on past the
   names it tried.
"""

from __future__ import annotations

import contextlib
import itertools
from dataclasses import dataclass

from . import elements as el
from .circuit import GROUND, Circuit
from .elements import Element, concatenate
from .signals import Constant, Signal

# SPICE letter of each element type for default device names (R1, M3, ...)
_LETTER = {
    el.Conductance: "R", el.Resistor: "R", el.Capacitor: "C", el.Inductor: "L",
    el.Transformer: "K", el.VoltageSource: "V", el.CurrentSource: "I", el.Diode: "D",
    el.BJT: "Q", el.EKVMOSFET: "M", el.Level1MOSFET: "M", el.VCVS: "E", el.VCCS: "G",
    el.CCCS: "F", el.CCVS: "H", el.IdealOpAmp: "U", el.OpAmp: "U", el.Switch: "S",
}


def group_base_name(element: Element) -> str:
    """The automatic group name of `element` before any ``_2`` suffix."""
    cls = type(element).__name__
    pol = getattr(element, "polarity", None)
    if isinstance(pol, str):
        return cls + "_" + pol
    wave = getattr(element, "value", None)
    if isinstance(wave, Signal) and not isinstance(wave, Constant):
        return cls + "_" + type(wave).__name__
    return cls


@dataclass
class _Pending:
    """A device added to the builder: its full name, the element with node
    names as terminals, and its explicit group (or None)."""
    name: str
    element: Element
    group: str | None


class _NameCursor:
    """Candidate names ``base, base_2, base_3, ...`` of one base, consumed
    in order across the groups that share the base."""

    def __init__(self, base: str):
        self._names = itertools.chain([base], (f"{base}_{i}" for i in itertools.count(2)))

    def take(self, taken) -> str:
        for cand in self._names:
            if cand not in taken:
                return cand
        raise AssertionError("unreachable")


class CircuitBuilder:
    """Incrementally assemble a `Circuit`.

    Args:
        nmos, pmos: Default `MOSProcess` for `nmos` / `pmos` devices.
        mos_model: MOSFET class used by `nmos` / `pmos` (EKVMOSFET,
            Level1MOSFET or a partial of one).
    """

    def __init__(self, nmos: el.MOSProcess | None = None,
                 pmos: el.MOSProcess | None = None, mos_model=el.EKVMOSFET):
        self.nmos_process = nmos or el.MOSProcess.nmos()
        self.pmos_process = pmos or el.MOSProcess.pmos()
        self.mos_model = mos_model
        self._pending: list[_Pending] = []
        self._taken_names: set[str] = set()
        self._node_order: dict[str, int] = {}   # node name -> index (insertion order)
        self._prefix: list[str] = []            # active scopes
        self._count: dict[str, int] = {}        # per SPICE letter / anonymous nodes

    def _bump(self, key: str) -> int:
        self._count[key] = self._count.get(key, 0) + 1
        return self._count[key]

    def _scoped(self, name: str) -> str:
        return ".".join(self._prefix + [name])

    def _touch(self, node: str) -> None:
        if node not in GROUND and node not in self._node_order:
            self._node_order[node] = len(self._node_order)

    # ---------------------------------------------------------------- nodes
    def node(self, name: str | None = None) -> str:
        """Declare a node (a fresh anonymous one when `name` is None) inside
        the current scope; returns its full name."""
        full = self._scoped(name if name is not None else f"_{self._bump('_node')}")
        self._touch(full)
        return full

    @contextlib.contextmanager
    def scope(self, prefix: str):
        """Prefix device names and `node` names with ``prefix.``."""
        self._prefix.append(prefix)
        try:
            yield
        finally:
            self._prefix.pop()

    @property
    def nodes(self) -> list[str]:
        """Non-ground node names in index order."""
        return list(self._node_order)

    # -------------------------------------------------------------- devices
    def add(self, element: Element, name: str | None = None,
            group: str | None = None) -> str:
        """Add one device whose terminals are node names; returns its full
        (scoped) name. Default names are the SPICE letter plus a counter."""
        if element.size != 1:
            raise ValueError("add() takes single-device elements")
        if name is None:
            letter = _LETTER.get(type(element), type(element).__name__)
            name = f"{letter}{self._bump(letter)}"
        full = self._scoped(name)
        if full in self._taken_names:
            raise ValueError(f"duplicate device name {full!r}")
        self._taken_names.add(full)
        terminals = tuple(map(str, element.nodes[0]))
        for t in terminals:
            self._touch(t)
        self._pending.append(_Pending(full, element.with_nodes((terminals,)), group))
        return full

    def resistor(self, p, n, r, name=None, group=None) -> str:
        return self.add(el.Resistor((p, n), r), name, group)

    def conductance(self, p, n, g, transform="log", g_min=0.0, g_max=1.0,
                    name=None, group=None) -> str:
        return self.add(el.Conductance((p, n), g, transform, g_min, g_max), name, group)

    def capacitor(self, p, n, c, name=None, group=None) -> str:
        return self.add(el.Capacitor((p, n), c), name, group)

    def inductor(self, p, n, l, rs=0.0, name=None, group=None) -> str:
        return self.add(el.Inductor((p, n), l, rs), name, group)

    def diode(self, a, k, name=None, group=None, **params) -> str:
        return self.add(el.Diode((a, k), **params), name, group)

    def bjt(self, c, b, e, polarity="npn", name=None, group=None, **params) -> str:
        return self.add(el.BJT((c, b, e), polarity, **params), name, group)

    def transformer(self, p1, n1, p2, n2, l1, l2, k=1.0, name=None, group=None) -> str:
        return self.add(el.Transformer((p1, n1, p2, n2), l1, l2, k), name, group)

    def vcvs(self, p, n, cp, cn, gain, name=None, group=None) -> str:
        return self.add(el.VCVS((p, n, cp, cn), gain), name, group)

    def cccs(self, p, n, sp, sn, gain, name=None, group=None) -> str:
        return self.add(el.CCCS((p, n, sp, sn), gain), name, group)

    def ccvs(self, p, n, sp, sn, r, name=None, group=None) -> str:
        return self.add(el.CCVS((p, n, sp, sn), r), name, group)

    def opamp(self, inp, inn, out, name=None, group=None, **params) -> str:
        return self.add(el.OpAmp((inp, inn, out), **params), name, group)

    def ideal_opamp(self, inp, inn, out, name=None, group=None) -> str:
        return self.add(el.IdealOpAmp((inp, inn, out)), name, group)

    def switch(self, p, n, cp, cn, name=None, group=None, **params) -> str:
        return self.add(el.Switch((p, n, cp, cn), **params), name, group)

    def vccs(self, p, n, cp, cn, gm, name=None, group=None) -> str:
        return self.add(el.VCCS((p, n, cp, cn), gm), name, group)

    def vsource(self, p, n, value=0.0, ac=0.0, ac_phase=0.0, name=None, group=None) -> str:
        return self.add(el.VoltageSource((p, n), value, ac, ac_phase), name, group)

    def isource(self, p, n, value=0.0, ac=0.0, ac_phase=0.0, name=None, group=None) -> str:
        return self.add(el.CurrentSource((p, n), value, ac, ac_phase), name, group)

    def _mos(self, polarity, d, g, s, b, w, l, name, group, process, dvth) -> str:
        proc = process or (self.nmos_process if polarity == "n" else self.pmos_process)
        dev = self.mos_model((d, g, s, s if b is None else b), w, l, proc, polarity, dvth)
        return self.add(dev, name, group)

    def nmos(self, d, g, s, b=None, w=1e-6, l=0.13e-6, name=None, group=None,
             process=None, dvth=0.0) -> str:
        return self._mos("n", d, g, s, b, w, l, name, group, process, dvth)

    def pmos(self, d, g, s, b=None, w=1e-6, l=0.13e-6, name=None, group=None,
             process=None, dvth=0.0) -> str:
        return self._mos("p", d, g, s, b, w, l, name, group, process, dvth)

    # ---------------------------------------------------------------- build
    def build(self) -> Circuit:
        """Resolve node names to indices, fuse devices into groups and name
        the groups by the rule in the module docstring."""
        index = self._node_order
        explicit: dict[str, list[tuple[str, Element]]] = {}
        automatic: dict[tuple, list[tuple[str, Element]]] = {}
        for p in self._pending:
            dev = p.element.with_nodes(
                (tuple(-1 if t in GROUND else index[t] for t in p.element.nodes[0]),))
            if p.group is None:
                automatic.setdefault(dev.group_key(), []).append((p.name, dev))
                continue
            members = explicit.setdefault(p.group, [])
            if members and members[0][1].group_key() != dev.group_key():
                raise ValueError(f"devices in group {p.group!r} cannot be fused")
            members.append((p.name, dev))

        named: list[tuple[str, list[tuple[str, Element]]]] = list(explicit.items())
        taken = set(explicit)
        cursors: dict[str, _NameCursor] = {}
        for members in automatic.values():
            base = group_base_name(members[0][1])
            gname = cursors.setdefault(base, _NameCursor(base)).take(taken)
            taken.add(gname)
            named.append((gname, members))

        groups = {g: concatenate([dev for _, dev in members]) for g, members in named}
        where = {dname: (g, i) for g, members in named for i, (dname, _) in enumerate(members)}
        return Circuit(groups, tuple(index), where)
