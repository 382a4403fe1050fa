"""Generate the golden symbolic-analysis fixtures from the reference itself.

voltax's structure and plan code (voltax/sparse.py:150-535) is numpy/scipy
only; jax and equinox are imported at module level but not used by it. This
script loads the reference's ``voltax/sparse.py`` from its source tree with
minimal stand-ins for those two imports, feeds it circuit topologies built
by ``voltax_gb300.builder`` (the same ``(layout, groups)`` key voltax's
`structure` hashes), and records what the reference computes:

* the CSR pattern and stamp positions (``_structure``),
* pivot groups (``_pivot_groups``),
* the plan: per bucket, each supernode's pivot unknowns and border, and the
  plan statistics (``_make_plan``).

Run from the repository root with the reference's source tree given by the
``VOLTAX_REFERENCE`` environment variable or the first argument:
``python tests/golden/make_fixtures.py <voltax source root>``.
The reference tree is only read here; the fixtures are committed.
"""

from __future__ import annotations

import hashlib
import importlib.util
import json
import sys
import types
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
import os  # noqa: E402

_REF_ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VOLTAX_REFERENCE")
REF = Path(_REF_ROOT) / "voltax" / "sparse.py" if _REF_ROOT else None
OUT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))


def load_reference_sparse():
    jax = types.ModuleType("jax")

    class _CustomVJP:
        def __init__(self, fn, nondiff_argnums=()):
            self.fn = fn

        def defvjp(self, *a):
            pass

    jax.custom_vjp = _CustomVJP
    jax.Array = object
    jnp = types.ModuleType("jax.numpy")
    jax.numpy = jnp
    pkg = types.ModuleType("voltax")
    pkg.__path__ = []
    elem = types.ModuleType("voltax.element")

    class Element:
        @staticmethod
        def charges(*a):
            return None, None

    elem.Element = Element
    sys.modules.update({"jax": jax, "jax.numpy": jnp, "voltax": pkg,
                        "voltax.element": elem})
    if REF is None:
        raise SystemExit("give the voltax source root as an argument or in VOLTAX_REFERENCE")
    spec = importlib.util.spec_from_file_location("voltax.sparse", REF)
    mod = importlib.util.module_from_spec(spec)
    sys.modules["voltax.sparse"] = mod
    spec.loader.exec_module(mod)
    return mod


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(np.asarray(a, dtype=np.int64)).tobytes())
        h.update(b"|")
    return h.hexdigest()


def circuits():
    from voltax_gb300 import workloads as wl
    from voltax_gb300.builder import CircuitBuilder
    from voltax_gb300.library import cmos

    def rc_ladder():
        b = CircuitBuilder()
        b.vsource("in", "0", 1.0, name="Vin")
        b.resistor("in", "a", 1e3, name="R1")
        b.resistor("a", "out", 2e3, name="R2")
        b.resistor("out", "0", 1e4, name="Rload")
        b.capacitor("a", "0", 1e-9, name="C1")
        b.capacitor("out", "0", 0.5e-9, name="C2")
        return b.build()

    def test_grid(n):  # topology of voltax tests/test_sparse.py:128-141
        b = CircuitBuilder()
        for i in range(n):
            for j in range(n):
                if j + 1 < n:
                    b.resistor(f"n{i}_{j}", f"n{i}_{j + 1}", 0.1)
                if i + 1 < n:
                    b.resistor(f"n{i}_{j}", f"n{i + 1}_{j}", 0.1)
                if (i * 7 + j * 3) % 5 == 0:
                    b.isource(f"n{i}_{j}", "0", 1e-3)
        for i, j in [(0, 0), (0, n - 1), (n - 1, 0), (n - 1, n - 1)]:
            b.vsource(f"n{i}_{j}", "0", 1.0)
        return b.build()

    def nand_adder(bits=2):  # voltax tests/test_sparse.py:29-37
        b = CircuitBuilder()
        b.vsource("vdd", "0", 1.2)
        a = [f"a{i}" for i in range(bits)]
        c = [f"b{i}" for i in range(bits)]
        for k, n in enumerate(a + c):
            b.vsource(n, "0", 1.2 * (k % 2))
        cmos.ripple_adder(b, a, c, "0", [f"s{i}" for i in range(bits)], "co", "vdd")
        return b.build()

    return [
        ("rc_ladder", rc_ladder, (16,)),
        ("test_grid10", lambda: test_grid(10), (1, 2, 16)),
        ("test_grid12", lambda: test_grid(12), (16,)),
        ("nand_adder2", lambda: nand_adder(2), (1, 16)),
        ("ring9", lambda: wl.ring_oscillator(9)[0], (2, 16)),
        ("ring101", lambda: wl.ring_oscillator(101)[0], (16,)),
        ("mirror_adder4", lambda: wl.mirror_adder(4), (2, 16)),
        ("grid30", lambda: wl.power_grid(30), (16,)),
        ("grid50", lambda: wl.power_grid(50), (16,)),
        ("grid100", lambda: wl.power_grid(100), (16,)),
    ]


def main():
    ref = load_reference_sparse()
    index = {}
    for name, factory, leaves in circuits():
        circuit = factory()
        key = circuit.topology_key().value  # (layout, groups): the reference's key shape
        st = ref._structure(key)
        rec = dict(size=int(st.size), n_nodes=int(st.n_nodes), nnz=int(st.nnz),
                   structure=digest(st.indptr, st.indices,
                                    *[p for _, p, _ in st.stamps]),
                   pivot_groups=digest(ref._pivot_groups(st)), plans={})
        arrays = {}
        small = st.size <= 200
        if small:
            arrays["indptr"] = st.indptr
            arrays["indices"] = st.indices
            arrays["pivot_groups"] = ref._pivot_groups(st)
        for leaf in leaves:
            plan = ref._make_plan(st, leaf)
            sets, bords = [], []
            for bk in plan.buckets:
                for j in range(bk.m):
                    sets.append(bk.piv[j][bk.valid[j]])
                    bords.append(bk.border[j][bk.border[j] < st.size])
            sizes = [len(s) for s in sets]
            bsizes = [len(b) for b in bords]
            stats = {k: (float(v) if isinstance(v, float) else int(v))
                     for k, v in plan.stats.items()}
            rec["plans"][str(leaf)] = dict(
                stats=stats, buckets=[int(bk.m) for bk in plan.buckets],
                supernodes=digest(np.concatenate(sets), sizes),
                borders=digest(np.concatenate(bords) if bords else [], bsizes))
            if small:
                arrays[f"leaf{leaf}_sets"] = np.concatenate(sets)
                arrays[f"leaf{leaf}_sizes"] = np.asarray(sizes)
                arrays[f"leaf{leaf}_borders"] = (np.concatenate(bords) if bords
                                                 else np.zeros(0, np.int64))
                arrays[f"leaf{leaf}_bsizes"] = np.asarray(bsizes)
        index[name] = rec
        if arrays:
            np.savez_compressed(OUT / f"{name}.npz",
                                **{k: np.asarray(v, np.int64) for k, v in arrays.items()})
        print(name, rec["size"], rec["nnz"],
              {k: v["stats"]["supernodes"] for k, v in rec["plans"].items()})
    (OUT / "symbolic.json").write_text(json.dumps(index, indent=1, sort_keys=True))


if __name__ == "__main__":
    main()
