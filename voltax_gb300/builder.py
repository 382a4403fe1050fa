"""`CircuitBuilder`: describe a circuit device by device with named nodes
(voltax/builder.py:52-256).

Devices of the same type and static configuration are fused into one element
group at `build`; group names follow voltax (``EKVMOSFET_n``,
``VoltageSource_Step``, ``Resistor``, ...), so the state layout -- groups in
sorted-name order -- is the one voltax would build.
"""

from __future__ import annotations

import contextlib
from collections import defaultdict

from . import elements as el
from .circuit import GROUND, Circuit
from .elements import Element, concatenate
from .signals import Constant, Signal

_PREFIX = {
    el.Conductance: "R", el.Resistor: "R", el.Capacitor: "C",
    el.VoltageSource: "V", el.CurrentSource: "I", el.EKVMOSFET: "M", el.Level1MOSFET: "M",
    el.Inductor: "L", el.Diode: "D", el.VCCS: "G", el.BJT: "Q", el.VCVS: "E", el.CCCS: "F",
    el.CCVS: "H", el.Transformer: "K", el.IdealOpAmp: "U", el.OpAmp: "U", el.Switch: "S",
}


def _default_group_name(element: Element) -> str:
    """Class name, plus polarity for transistors or the waveform for non-DC
    sources (voltax/builder.py:39-49)."""
    name = type(element).__name__
    polarity = getattr(element, "polarity", None)
    if isinstance(polarity, str):
        return f"{name}_{polarity}"
    wave = getattr(element, "value", None)
    if isinstance(wave, Signal) and not isinstance(wave, Constant):
        return f"{name}_{type(wave).__name__}"
    return name


class CircuitBuilder:
    """Incrementally assemble a `Circuit`.

    Args:
        nmos, pmos: Default `MOSProcess` for `nmos` / `pmos` devices.
    """

    def __init__(self, nmos: el.MOSProcess | None = None,
                 pmos: el.MOSProcess | None = None, mos_model=el.EKVMOSFET):
        self.nmos_process = nmos or el.MOSProcess.nmos()
        self.pmos_process = pmos or el.MOSProcess.pmos()
        self.mos_model = mos_model  # EKVMOSFET, Level1MOSFET or a partial of one
        self._devices: list[tuple[str, Element, str | None]] = []
        self._names: set[str] = set()
        self._nodes: dict[str, None] = {}
        self._scope: list[str] = []
        self._counters: dict[str, int] = defaultdict(int)

    # ---------------------------------------------------------------- nodes
    def node(self, name: str | None = None) -> str:
        if name is None:
            self._counters["_node"] += 1
            name = f"_{self._counters['_node']}"
        full = ".".join([*self._scope, name])
        self._nodes.setdefault(full, None)
        return full

    @contextlib.contextmanager
    def scope(self, prefix: str):
        self._scope.append(prefix)
        try:
            yield
        finally:
            self._scope.pop()

    @property
    def nodes(self) -> list[str]:
        return list(self._nodes)

    # -------------------------------------------------------------- devices
    def add(self, element: Element, name: str | None = None,
            group: str | None = None) -> str:
        if element.size != 1:
            raise ValueError("add() takes single-device elements")
        if name is None:
            prefix = _PREFIX.get(type(element), type(element).__name__)
            self._counters[prefix] += 1
            name = f"{prefix}{self._counters[prefix]}"
        name = ".".join([*self._scope, name])
        if name in self._names:
            raise ValueError(f"duplicate device name {name!r}")
        self._names.add(name)
        terminals = tuple(str(n) for n in element.nodes[0])
        for n in terminals:
            if n not in GROUND:
                self._nodes.setdefault(n, None)
        self._devices.append((name, element.with_nodes((terminals,)), group))
        return name

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

    def nmos(self, d, g, s, b=None, w=1e-6, l=0.13e-6, name=None, group=None,
             process=None, dvth=0.0) -> str:
        dev = self.mos_model((d, g, s, s if b is None else b), w, l,
                             process or self.nmos_process, "n", dvth)
        return self.add(dev, name, group)

    def pmos(self, d, g, s, b=None, w=1e-6, l=0.13e-6, name=None, group=None,
             process=None, dvth=0.0) -> str:
        dev = self.mos_model((d, g, s, s if b is None else b), w, l,
                             process or self.pmos_process, "p", dvth)
        return self.add(dev, name, group)

    # ---------------------------------------------------------------- build
    def build(self) -> Circuit:
        """Resolve node names, fuse devices into groups (builder.py:224-256)."""
        index = {name: i for i, name in enumerate(self._nodes)}

        def resolve(n):
            return -1 if n in GROUND else index[n]

        buckets: dict = {}
        for name, dev, group in self._devices:
            dev = dev.with_nodes((tuple(resolve(n) for n in dev.nodes[0]),))
            key = group if group is not None else dev.group_key()
            if group is not None and buckets.get(key):
                if buckets[key][0][1].group_key() != dev.group_key():
                    raise ValueError(f"devices in group {group!r} cannot be fused")
            buckets.setdefault(key, []).append((name, dev))

        groups: dict[str, Element] = {}
        device_names: dict[str, tuple[str, int]] = {}
        used: dict[str, int] = defaultdict(int)
        order = sorted(buckets, key=lambda k: not isinstance(k, str))
        for key in order:
            members = buckets[key]
            if isinstance(key, str):
                gname = key
            else:
                base = _default_group_name(members[0][1])
                gname = base
                while gname in groups or gname in buckets:
                    used[base] += 1
                    gname = f"{base}_{used[base] + 1}"
            groups[gname] = concatenate([dev for _, dev in members])
            for i, (name, _) in enumerate(members):
                device_names[name] = (gname, i)
        return Circuit(groups, tuple(self._nodes), device_names)
