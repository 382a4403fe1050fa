"""The C++ planner (libvxg_symbolic.so) equals the numpy restatement of
voltax's symbolic phase element for element, on every circuit family and
leaf size, including segmented batches whose dissection splits into many
components. The numpy restatement is itself pinned to the reference's own
output (test_symbolic.py)."""

import ctypes as C
import re
import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import plan as oplan  # the numpy restatement (the C++ planner's checker)
from voltax_gb300 import build, runtime, symbolic, workloads

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(Path(__file__).parent))
import circuits  # noqa: E402


def declared():
    text = (ROOT / "include" / "vxg_symbolic.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vxs_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(build.build_symbolic()))
    names = declared()
    assert "vxs_plan_create" in names
    for name in names:
        assert hasattr(lib, name), name


def test_field_table_matches_header():
    text = (ROOT / "include" / "vxg_symbolic.h").read_text()
    ids = {m[0].lower(): int(m[1]) for m in re.findall(r"VXS_([A-Z_]+) = (\d+),", text)
           if not m[0].startswith("ERR")}
    ids.pop("ok", None)
    ids.pop("n_fields", None)
    assert {n: i for i, n in enumerate(symbolic._FIELDS)} == ids
    assert f"VXS_N_FIELDS = {len(symbolic._FIELDS)}" in text


def assert_same_plan(a, b):
    assert (a.size, a.work) == (b.size, b.work)
    for f in ("parents", "level", "k", "r", "panel", "a_pos", "sn_of", "pos_in"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    for f in ("supernodes", "borders", "buckets"):
        x, y = getattr(a, f), getattr(b, f)
        assert len(x) == len(y), f
        assert all(np.array_equal(p, q) for p, q in zip(x, y)), f
    assert a.stats == b.stats
    assert len(a.levels) == len(b.levels)
    for la, lb in zip(a.levels, b.levels):
        for f in la.__dataclass_fields__:
            assert np.array_equal(np.asarray(getattr(la, f)), np.asarray(getattr(lb, f))), f


CASES = {
    "grid10": lambda: workloads.power_grid(10),
    "grid37": lambda: workloads.power_grid(37, seed=3),
    "grid60": lambda: workloads.power_grid(60),
    "grid_batch": lambda: workloads.power_grid_batch([12, 20, 7, 33, 5]),
    "ring101": lambda: workloads.ring_oscillator(101)[0],
    "ring_level1": lambda: workloads.ring_oscillator_level1(31)[0],
    "mirror_adder": lambda: workloads.mirror_adder(),
    "ota_chain": lambda: workloads.ota_chain(),
    "mixed": circuits.mixed_circuit,
    "bjt": circuits.bjt_amplifier,
    "controlled": circuits.controlled_sources_circuit,
    "opamp_switch": circuits.opamp_switch_circuit,
}


@pytest.mark.parametrize("leaf", [2, 4, 16, 64])
@pytest.mark.parametrize("name", sorted(CASES))
def test_native_plan_equals_restatement(name, leaf):
    st = symbolic.structure(CASES[name](), leaf)
    assert_same_plan(symbolic.make_plan(st, leaf),
                     oplan.make_plan_numpy(st, leaf))


def test_segmented_batch_plans_each_segment_apart():
    """Independent sub-circuits never share a supernode or a border."""
    c = workloads.power_grid_batch([9, 14, 6])
    seg = c.unknown_segments()
    plan = symbolic.make_plan(symbolic.structure(c))
    for s, b in zip(plan.supernodes, plan.borders):
        assert len(np.unique(seg[s])) == 1
        assert len(b) == 0 or np.all(seg[b] == seg[s[0]])


def test_invalid_input_is_rejected():
    lib = symbolic._symlib()
    indptr = np.array([0, 1, 2], np.int64)
    indices = np.array([0, 1], np.int64)
    bad = np.array([5], np.int64)
    zero = np.array([0], np.int64)
    h = C.c_void_p()
    rc = lib.vxs_plan_create(2, indptr.ctypes.data, indices.ctypes.data, 1, zero.ctypes.data,
                             bad.ctypes.data, 16, C.byref(h))
    assert rc == 1 and h.value is None
    assert b"union pair" in lib.vxs_last_error()
    rc = lib.vxs_plan_create(2, indptr.ctypes.data, indices.ctypes.data, 0, None, None, 0,
                             C.byref(h))
    assert rc == 1
    assert lib.vxs_plan_len(None, 0) == -1
    st = symbolic.structure(workloads.power_grid(4))
    with pytest.raises(ValueError):
        symbolic.native_fields(st, 0)


def test_default_planner_is_native(monkeypatch):
    st = symbolic.structure(workloads.power_grid(6))
    calls = []
    real = symbolic._make_plan_native
    monkeypatch.setattr(symbolic, "_make_plan_native",
                        lambda *a: calls.append(1) or real(*a))
    symbolic.make_plan(st)
    assert calls == [1]


@pytest.mark.parametrize("name", ["grid37", "grid_batch", "mirror_adder", "ota_chain", "mixed"])
def test_device_tables_from_native_plan_equal_restatement(name):
    """The upload tables taken straight from the C++ plan's flat arrays equal
    those assembled from the numpy plan's per-level tables."""
    c = CASES[name]()
    st = symbolic.structure(c)
    a = runtime.Tables(c, st, symbolic.make_plan(st))
    b = runtime.Tables(c, st, oplan.make_plan_numpy(st))
    keys = [k for k, v in vars(b).items() if isinstance(v, np.ndarray)]
    assert "st_src" in keys and "bt_ptr" in keys and "sn_piv" in keys
    for k in keys:
        x, y = getattr(a, k), getattr(b, k)
        assert x.dtype == y.dtype and np.array_equal(x, y), k
    assert a.work == b.work and a.n_seg == b.n_seg


def test_take_moves_fields_out_of_the_plan():
    import ctypes as C
    lib = symbolic._symlib()
    st = symbolic.structure(workloads.power_grid(5))
    indptr = np.ascontiguousarray(st.indptr, np.int64)
    indices = np.ascontiguousarray(st.indices, np.int64)
    ua, ub = symbolic.union_pairs(st)
    h = C.c_void_p()
    assert lib.vxs_plan_create(st.size, indptr.ctypes.data, indices.ctypes.data, len(ua),
                               ua.ctypes.data, ub.ctypes.data, 16, C.byref(h)) == 0
    try:
        n = lib.vxs_plan_len(h, 14)
        assert n == st.nnz
        a = np.empty(n, np.int64)
        assert lib.vxs_plan_take(h, 14, a.ctypes.data) == 0
        assert lib.vxs_plan_len(h, 14) == 0
        assert a.min() >= 0
        # a level-table field (kept in per-level pieces) moves out the same way
        for field in (23, 24):  # ST_PTR, ST_SRC
            n = lib.vxs_plan_len(h, field)
            b = np.empty(n, np.int64)
            assert lib.vxs_plan_copy(h, field, b.ctypes.data) == 0
            c = np.empty(n, np.int64)
            assert lib.vxs_plan_take(h, field, c.ctypes.data) == 0
            assert np.array_equal(b, c) and lib.vxs_plan_len(h, field) == 0
            assert lib.vxs_plan_copy(h, field, None) == 0
    finally:
        lib.vxs_plan_destroy(h)


def test_plan_is_identical_for_any_thread_count(monkeypatch):
    st = symbolic.structure(workloads.power_grid_batch([15, 22, 9, 30]), 8)
    runs = []
    for threads in ("1", "3", "16"):
        monkeypatch.setenv("VXS_THREADS", threads)
        runs.append(symbolic.native_fields(st, 8))
    for other in runs[1:]:
        assert runs[0].keys() == other.keys()
        for k in runs[0]:
            assert np.array_equal(runs[0][k], other[k]), k


@pytest.mark.parametrize("indptr,indices,why", [
    ([1, 1, 2], [0, 1], "indptr[0]"),
    ([0, 2, 1], [0, 1], "non-decreasing"),
    ([0, 1, 2], [0, 7], "column index"),
])
def test_malformed_pattern_is_rejected(indptr, indices, why):
    lib = symbolic._symlib()
    ip = np.array(indptr, np.int64)
    ix = np.array(indices, np.int64)
    h = C.c_void_p()
    rc = lib.vxs_plan_create(2, ip.ctypes.data, ix.ctypes.data, 0, None, None, 16, C.byref(h))
    assert rc == 1 and h.value is None
    assert why in lib.vxs_last_error().decode()
