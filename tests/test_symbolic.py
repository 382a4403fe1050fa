"""The symbolic analysis equals the reference's, bit for bit.

Golden fixtures come from the reference's own ``voltax/sparse.py`` run on the
same topologies (``tests/golden/make_fixtures.py``): CSR pattern and stamp
positions, pivot groups, supernodes, borders, bucket classes and plan
statistics. Both planners are pinned: the C++ one (the default) and the
numpy restatement. Also checks the GPU panel layout's invariants.
"""

import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import plan as oplan  # the numpy restatement (the C++ planner's checker)
from voltax_gb300 import symbolic

GOLDEN = Path(__file__).parent / "golden"
INDEX = json.loads((GOLDEN / "symbolic.json").read_text())


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(np.asarray(a, dtype=np.int64)).tobytes())
        h.update(b"|")
    return h.hexdigest()


def fixture_circuits(names):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_fixtures",
                                                  GOLDEN / "make_fixtures.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return {n: (f(), leaves) for n, f, leaves in mod.circuits() if n in names}


SMALL = [n for n, r in INDEX.items() if r["size"] <= 200]
LARGE = ["grid30", "grid50"]


def _check(name, circuit, leaves, native):
    rec = INDEX[name]
    st = symbolic.structure(circuit)
    assert (st.size, st.n_nodes, st.nnz) == (rec["size"], rec["n_nodes"], rec["nnz"])
    assert digest(st.indptr, st.indices, *[p for _, p, _ in st.stamps]) == rec["structure"]
    assert digest(oplan.pivot_groups(st)) == rec["pivot_groups"]
    if native:
        gid = symbolic.native_fields(st, symbolic.LEAF_SIZE)["gid"]
        assert digest(gid) == rec["pivot_groups"]
    for leaf in leaves:
        want = rec["plans"][str(leaf)]
        plan = symbolic.make_plan(st, leaf) if native else oplan.make_plan_numpy(st, leaf)
        assert [len(c) for c in plan.buckets] == want["buckets"]
        sets = [plan.supernodes[i] for c in plan.buckets for i in c]
        bords = [plan.borders[i] for c in plan.buckets for i in c]
        assert digest(np.concatenate(sets), [len(s) for s in sets]) == want["supernodes"]
        assert digest(np.concatenate(bords) if bords else [],
                      [len(b) for b in bords]) == want["borders"]
        for key, value in want["stats"].items():
            assert plan.stats[key] == value, key
        _check_layout(st, plan)


def _check_layout(st, plan):
    # every pattern entry owns a distinct panel slot inside the panel storage
    assert len(np.unique(plan.a_pos)) == st.nnz
    assert plan.a_pos.min() >= 0 and plan.a_pos.max() < plan.work
    assert plan.work == plan.stats["factor_entries"]
    # the level tables cover every supernode once, and the Schur targets of a
    # level lie in panels of later levels
    seen = np.concatenate([lv.sns for lv in plan.levels])
    assert np.array_equal(np.sort(seen), np.arange(len(plan.supernodes)))
    for li, lv in enumerate(plan.levels):
        assert lv.schur_ptr[-1] == lv.schur_len
        if len(lv.schur_tgt):
            owner = np.searchsorted(plan.panel, lv.schur_tgt, side="right") - 1
            assert np.all(plan.level[owner] > li)


@pytest.mark.parametrize("native", [True, False], ids=["cpp", "numpy"])
@pytest.mark.parametrize("name", SMALL)
def test_small_topologies_match_reference(name, native):
    circuit, leaves = fixture_circuits([name])[name]
    _check(name, circuit, leaves, native)
    arrays = np.load(GOLDEN / f"{name}.npz")
    st = symbolic.structure(circuit)
    assert np.array_equal(st.indptr, arrays["indptr"])
    assert np.array_equal(st.indices, arrays["indices"])
    assert np.array_equal(oplan.pivot_groups(st), arrays["pivot_groups"])


@pytest.mark.parametrize("native", [True, False], ids=["cpp", "numpy"])
@pytest.mark.parametrize("name", LARGE)
def test_power_grids_match_reference(name, native):
    circuit, leaves = fixture_circuits([name])[name]
    _check(name, circuit, leaves, native)


def test_voltage_sources_pair_with_their_node():
    """voltax tests/test_sparse.py:233-242: each pad current shares a pivot
    group with its node."""
    from voltax_gb300 import workloads
    c = workloads.power_grid(12)
    st = symbolic.structure(c)
    gid = oplan.pivot_groups(st)
    for name in ("Vpad0", "Vpad1", "Vpad2"):
        group, idx = c.layout.device(name)
        node = int(c.elements[group].node_array()[idx, 0])
        assert gid[c.layout.internal(name)] == gid[node]
    plan = st.plan
    assert plan.stats["supernodes"] > 1 and plan.stats["levels"] > 2


def test_structure_is_cached_per_topology():
    from voltax_gb300 import workloads
    a = workloads.power_grid(8, seed=1)
    b = workloads.power_grid(8, seed=2)
    assert symbolic.structure(a) is symbolic.structure(b)


def test_pattern_covers_device_blocks_only():
    """voltax tests/test_sparse.py:192-198: the pattern is the union of the
    device blocks plus the diagonal, nothing else."""
    from voltax_gb300.builder import CircuitBuilder
    b = CircuitBuilder()
    b.vsource("in", "0", 1.0, name="Vin")
    b.resistor("in", "a", 1e3, name="R1")
    b.resistor("a", "out", 2e3, name="R2")
    b.resistor("out", "0", 1e4, name="Rload")
    b.capacitor("a", "0", 1e-9, name="C1")
    b.capacitor("out", "0", 0.5e-9, name="C2")
    c = b.build()
    st = symbolic.structure(c)
    P = st.to_scipy(np.ones(st.nnz)).toarray()
    a, out, vin = c.layout.node("a"), c.layout.node("out"), c.layout.internal("Vin")
    assert P[a, out] and P[out, a] and P[vin, c.layout.node("in")]
    assert not P[c.layout.node("in"), out]  # no device connects in and out
    assert np.all(np.diag(P))
