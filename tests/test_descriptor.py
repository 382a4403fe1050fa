"""vxg_create checks every index of a topology descriptor on the host before
anything reaches the GPU: a malformed descriptor returns VXG_ERR_INVALID with
the violated field in vxg_last_error(), never an out-of-bounds access in a
kernel. Runs without a GPU: a valid descriptor passes the checks and then
fails at its first device allocation (a status other than VXG_ERR_INVALID).
"""

import ctypes as C
import sys
from pathlib import Path

import pytest
import torch

from voltax_gb300 import _lib as L
from voltax_gb300 import runtime, symbolic, workloads

sys.path.insert(0, str(Path(__file__).parent))
import circuits  # noqa: E402

pytestmark = pytest.mark.skipif(torch.cuda.is_available(),
                                reason="checks validation ahead of device allocation")

MAKERS = {
    "grid": lambda: workloads.power_grid(9),
    "grid_batch": lambda: workloads.power_grid_batch([5, 8, 3]),
    "ring": lambda: workloads.ring_oscillator(5)[0],
    "ring_level1": lambda: workloads.ring_oscillator_level1(5)[0],
    "adder": lambda: workloads.mirror_adder(1),
    "ota": lambda: workloads.ota_chain(6),
    "mixed": circuits.mixed_circuit,
    "bjt": circuits.bjt_amplifier,
    "controlled": circuits.controlled_sources_circuit,
    "opamp_switch": circuits.opamp_switch_circuit,
}


@pytest.fixture(scope="module")
def lib():
    from voltax_gb300 import build
    build.build()
    return L.load()


def tables(name):
    c = MAKERS[name]()
    st = symbolic.structure(c)
    return runtime.Tables(c, st, st.plan)


def create(lib, desc):
    h = C.c_void_p()
    rc = lib.vxg_create(C.byref(desc), C.byref(h))
    return rc, lib.vxg_last_error().decode()


@pytest.mark.parametrize("name", sorted(MAKERS))
def test_valid_descriptors_pass_validation(lib, name):
    t = tables(name)  # owns the arrays the descriptor points into
    rc, msg = create(lib, t.descriptor())
    assert rc != L.VXG_ERR_INVALID, msg


@pytest.mark.parametrize("leaf", [1, 2, 16])
@pytest.mark.parametrize("name", ["grid", "adder", "ring"])
def test_linear_algebra_only_descriptors_pass_validation(lib, name, leaf):
    """sparse.factor / solve on a bare plan: no device groups."""
    st = symbolic.structure(MAKERS[name]())
    t = runtime.Tables(None, st, symbolic.make_plan(st, leaf))
    rc, msg = create(lib, t.descriptor())
    assert rc != L.VXG_ERR_INVALID, msg


# (attribute of Tables, index to corrupt, value, field named in the error)
CORRUPTIONS = [
    ("indices", 3, 10_000, "indices or rows"),
    ("indptr", 2, -1, "indptr or tptr"),
    ("diag", 0, 1, "diag"),
    ("tent", 0, 10**9, "tent"),
    ("res_src", 0, 10**9, "res_src"),
    ("jac_src", -1, -3, "jac_src"),
    ("seg_of", 0, 5, "seg_idx or seg_of"),
    ("sn_k", 0, 0, "sn_k, sn_r or their offsets"),
    ("sn_panel", -1, 10**9, "sn_panel"),
    ("sn_piv", 0, -2, "sn_piv"),
    ("a_pos", 0, 10**9, "a_pos"),
    ("lv_sn", 0, 10**6, "lv_sn"),
    ("lv_schur_off", -1, 10**9, "lv_schur_off"),
    ("st_tgt", 0, 10**9, "st_tgt"),
    ("st_src", 0, 10**9, "st_src"),
    ("bt_tgt", 0, -1, "bt_tgt"),
    ("bt_src", 0, 10**9, "bt_src"),
]


@pytest.mark.parametrize("attr,idx,value,field", CORRUPTIONS,
                         ids=[c[0] for c in CORRUPTIONS])
def test_each_corrupted_index_is_rejected(lib, attr, idx, value, field):
    t = tables("grid")
    arr = getattr(t, attr).copy()
    assert arr.size, attr
    arr[idx] = value
    setattr(t, attr, arr)
    rc, msg = create(lib, t.descriptor())
    assert rc == L.VXG_ERR_INVALID
    assert msg == f"invalid topology descriptor: {field}"


def test_group_shape_and_rows_are_checked(lib):
    t = tables("adder")
    base = list(t.group_descs)
    cases = []
    for i, (kind, n, T, K, wave, n_params, off) in enumerate(base):
        cases.append((i, (kind, n, T + 1, K, wave, n_params, off),
                      "group terminals or internals for its kind"))
        cases.append((i, (kind, n, T, K, wave, n_params - 1, off), "group parameter rows"))
        cases.append((i, (99, n, T, K, wave, n_params, off), "group kind or size"))
    src = [i for i, g in enumerate(base) if g[0] in (2, 3)]
    assert src
    kind, n, T, K, wave, n_params, off = base[src[0]]
    cases.append((src[0], (kind, n, T, K, 7, n_params, off), "source waveform"))
    for i, desc, field in cases:
        t.group_descs = base[:i] + [desc] + base[i + 1:]
        rc, msg = create(lib, t.descriptor())
        assert rc == L.VXG_ERR_INVALID and msg.endswith(field), (i, desc, msg)
    t.group_descs = base
    nodes = t._nodes[0].copy()
    nodes[0] = t.nv
    t._nodes[0] = nodes
    rc, msg = create(lib, t.descriptor())
    assert rc == L.VXG_ERR_INVALID and msg.endswith("group node index")


def test_null_arrays_are_rejected(lib):
    t = tables("ring")
    d = t.descriptor()
    d.a_pos = None
    rc, msg = create(lib, d)
    assert rc == L.VXG_ERR_INVALID and msg.endswith("a required array is NULL")
    assert lib.vxg_create(None, None) == L.VXG_ERR_INVALID


def test_slot_counts_must_match_the_groups(lib):
    t = tables("mixed")
    t.n_res_slots += 1
    rc, msg = create(lib, t.descriptor())
    assert rc == L.VXG_ERR_INVALID and msg.endswith("n_res_slots or n_jac_slots")
