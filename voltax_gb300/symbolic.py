"""Sparsity structure and supernodal symbolic analysis (host side, once per
topology).

This module reproduces voltax's symbolic phase exactly -- the CSR pattern
and stamp positions (voltax/sparse.py:150-193), pivot groups
(voltax/sparse.py:257-305), nested dissection (voltax/sparse.py:308-378) and
the level schedule and statistics (voltax/sparse.py:412-535) -- so that the
GPU factorization eliminates the same supernodes in the same order as the
reference. Only the numeric layout differs: instead of voltax's padded
per-bucket batches, every supernode owns an unpadded, contiguous panel

    F11 (k x k) | F12 (k x r) | F21 (r x k)          (row-major)

and each elimination level is one launch whose CTAs take supernodes of
different sizes. The index maps the kernels need (pattern -> panel,
deterministic Schur-update and border-update gathers) are built here.

The planner is C++ (`csrc/symbolic.cpp`, `libvxg_symbolic.so`); the
bipartite matching of the pivot grouping (`union_pairs`) runs in scipy and
feeds it. Its checker, a numpy restatement of voltax's own planner, lives
with the oracle; both are pinned to plans the reference's own code produced.
"""

from __future__ import annotations

import functools
import os
from collections.abc import Sequence
from dataclasses import dataclass, field
from functools import cached_property

import numpy as np
import scipy.sparse as sp
import scipy.sparse.csgraph as csg

LEAF_SIZE = int(os.environ.get("VOLTAX_SPARSE_LEAF", 16))
"""Largest nested-dissection leaf kept as one dense supernode (sparse.py:63)."""
SPLIT_SAVING = 1e6
"""Padded flops a level must save to be split in two buckets (sparse.py:64)."""


# =============================================================================
# Pattern
# =============================================================================


@dataclass(frozen=True, eq=False)
class Structure:
    """CSR pattern of ``df/dz`` and ``dq/dz`` (sorted columns, diagonal
    always present) plus per-group stamp positions (voltax/sparse.py:73-133).

    ``stamps``: per group ``(name, positions (N, m, m), local)``, ``nnz`` =
    dropped (ground). ``devices``: per group ``(name, unknowns (N, T+K), T,
    local)`` with ``-1`` for ground.
    """

    size: int
    n_nodes: int
    indptr: np.ndarray
    indices: np.ndarray
    stamps: tuple
    devices: tuple
    leaf: int = LEAF_SIZE

    @property
    def nnz(self) -> int:
        return len(self.indices)

    @cached_property
    def rows(self) -> np.ndarray:
        return np.repeat(np.arange(self.size), np.diff(self.indptr))

    @cached_property
    def diagonal(self) -> np.ndarray:
        return positions(self, np.arange(self.size), np.arange(self.size))

    @cached_property
    def plan(self) -> "Plan":
        return make_plan(self, self.leaf)

    def to_scipy(self, data) -> sp.csr_matrix:
        return sp.csr_matrix((np.asarray(data), self.indices, self.indptr),
                             shape=(self.size, self.size))


def positions(st: Structure, rows, cols) -> np.ndarray:
    """Positions of ``(rows, cols)`` in the pattern; ``nnz`` where either is
    ground (-1). Raises if an entry is missing (voltax/sparse.py:136-147)."""
    keys = st.rows.astype(np.int64) * st.size + st.indices
    return _positions_in(keys, st.size, rows, cols)


def _positions_in(keys: np.ndarray, S: int, rows, cols) -> np.ndarray:
    """`positions` against the sorted entry keys ``row * S + col``."""
    rows, cols = np.broadcast_arrays(np.asarray(rows), np.asarray(cols))
    want = rows.astype(np.int64) * S + cols
    pos = np.searchsorted(keys, want)
    ok = (rows >= 0) & (cols >= 0)
    hit = np.where(ok, keys[np.minimum(pos, len(keys) - 1)] == want, True)
    if not hit.all():
        raise AssertionError("entry outside the sparsity pattern")
    return np.where(ok, pos, len(keys)).astype(np.int32)


# Node tables of the circuit whose structure is being built, by the identity
# of their node tuples: the topology key carries the tuples, the elements
# already hold them as arrays (`Element.node_array`).
_NODE_TABLES: dict = {}


def structure(circuit, leaf: int | None = None) -> Structure:
    """The cached `Structure` of `circuit`'s topology."""
    _NODE_TABLES.update({id(el.nodes): (el.nodes, el.node_array())
                         for el in circuit.elements.values() if el.size})
    try:
        return _structure(circuit.topology_key(), LEAF_SIZE if leaf is None else leaf)
    finally:
        _NODE_TABLES.clear()


def _node_table(nodes, n: int) -> np.ndarray:
    held = _NODE_TABLES.get(id(nodes))
    if held is not None and held[0] is nodes:
        return held[1]
    return np.asarray(nodes, dtype=np.int64).reshape(n, -1)


@functools.lru_cache(maxsize=512)
def _structure(key, leaf: int) -> Structure:
    layout, groups = key.value
    return build_structure(layout.size, layout.n_nodes,
                           {g: (n, k, off) for g, n, k, off in layout.groups},
                           groups, leaf)


def build_structure(S: int, nv: int, offsets: dict, groups, leaf: int = LEAF_SIZE
                    ) -> Structure:
    devices = []
    keys = [np.arange(S, dtype=np.int64) * (S + 1)]  # the diagonal
    for name, nodes, local in groups:
        n, k, off = offsets[name]
        if n == 0:
            continue
        idx = _node_table(nodes, n)
        allv = np.concatenate([idx, np.arange(off, off + n * k).reshape(n, k)], 1)
        devices.append((name, allv, idx.shape[1], local))
        blocks = allv if local else allv.reshape(1, -1)
        r = np.broadcast_to(blocks[:, :, None], blocks.shape + blocks.shape[1:2])
        c = np.broadcast_to(blocks[:, None, :], r.shape)
        keep = (r >= 0) & (c >= 0)
        keys.append(r[keep] * S + c[keep])
    uniq = np.concatenate(keys)
    uniq.sort()  # sorted distinct keys (a sort beats np.unique's hashing here)
    uniq = uniq[np.concatenate(([True], uniq[1:] != uniq[:-1]))]
    row_of = uniq // S
    indptr = np.zeros(S + 1, np.int64)
    np.cumsum(np.bincount(row_of, minlength=S), out=indptr[1:])
    st = Structure(S, nv, indptr, (uniq % S).astype(np.int64), (), tuple(devices),
                   leaf)
    stamps = []
    for name, allv, _, local in devices:
        blocks = allv if local else allv.reshape(1, -1)
        pos = _positions_in(uniq, S, blocks[:, :, None], blocks[:, None, :])
        stamps.append((name, pos if local else pos[0], local))
    object.__setattr__(st, "stamps", tuple(stamps))
    return st


# =============================================================================
# Pivot groups and nested dissection (the reference's exact algorithm)
# =============================================================================


def union_pairs(st: Structure) -> tuple[np.ndarray, np.ndarray]:
    """The ordered ``union(a, b)`` calls of voltax's pivot grouping
    (voltax/sparse.py:257-305): unknowns whose diagonal may vanish are glued
    to a terminal node of their device; two-terminal devices with one
    internal pick a partner by bipartite matching (matched pairs first, in
    device order), every other device glues all its unknowns."""
    pair_x, pair_cands, full = [], [], []
    for _, allv, T, local in st.devices:
        k = allv.shape[1] - T
        if k == 0:
            continue
        if not local:
            full.append([int(v) for v in np.unique(allv) if v >= 0])
            continue
        for dev in allv:
            terms = [int(v) for v in dev[:T] if v >= 0]
            internals = [int(v) for v in dev[T:]]
            if T == 2 and k == 1 and terms:
                pair_x.append(internals[0])
                pair_cands.append(terms)
            else:
                full.append(terms + internals)
    ua: list[int] = []
    ub: list[int] = []
    if pair_x:
        r = np.repeat(np.arange(len(pair_x)), [len(c) for c in pair_cands])
        c = np.concatenate(pair_cands)
        g = sp.csr_matrix((np.ones(len(r)), (r, c)), shape=(len(pair_x), st.n_nodes))
        match = csg.maximum_bipartite_matching(g, perm_type="column")
        for i, (x, cands) in enumerate(zip(pair_x, pair_cands)):
            if match[i] >= 0:
                ua.append(int(match[i]))
                ub.append(x)
            else:
                full.append(cands + [x])
    for members in full:
        ua += [members[0]] * (len(members) - 1)
        ub += members[1:]
    return np.asarray(ua, np.int64), np.asarray(ub, np.int64)


# =============================================================================
# Plan
# =============================================================================


@dataclass(frozen=True, eq=False)
class Plan:
    """Symbolic factorization of a `Structure`.

    Reference-equal parts: ``supernodes`` (sorted unknowns, postorder),
    ``parents``, ``borders``, ``level``, ``buckets`` (the reference's bucket
    classes: supernode ids per padded batch) and ``stats``.

    GPU layout (unpadded per-supernode panels): ``k``, ``r``, ``panel``
    (offset of F11; F12 follows at ``k*k``, F21 at ``k*k + k*r``), ``a_pos``
    (pattern entry -> panel slot), ``work`` (panel length), and the per-level
    launch tables in `levels`.
    """

    size: int
    supernodes: list
    parents: np.ndarray
    borders: list
    level: np.ndarray
    buckets: list
    stats: dict
    k: np.ndarray
    r: np.ndarray
    panel: np.ndarray
    work: int
    a_pos: np.ndarray
    levels: list = field(default_factory=list)
    sn_of: np.ndarray | None = None
    pos_in: np.ndarray | None = None
    structure: object = None
    flat: dict | None = None
    """The C++ planner's arrays (all levels concatenated, global CSR
    offsets: the layout `vxg_create` takes), or None for the numpy plan."""


@dataclass(frozen=True, eq=False)
class LevelTable:
    """Launch data of one elimination level.

    ``sns``: supernode ids of the level (largest first, for load balance).
    ``schur_off``: per supernode, offset of its ``r x r`` Schur block in the
    level's scratch. Deterministic Schur gather: unique panel targets
    ``schur_tgt`` with source lists ``schur_ptr``/``schur_src`` (scratch
    indices in ascending order). Border gather of the solves: unique
    unknowns ``bord_tgt`` with sources ``bord_ptr``/``bord_src`` into the
    level's concatenated border contributions (offset ``bord_off``).
    """

    sns: np.ndarray
    schur_off: np.ndarray
    schur_len: int
    schur_tgt: np.ndarray
    schur_ptr: np.ndarray
    schur_src: np.ndarray
    bord_off: np.ndarray
    bord_len: int
    bord_tgt: np.ndarray
    bord_ptr: np.ndarray
    bord_src: np.ndarray


def _stats(k, r, level, classes, G) -> dict:
    """voltax's ``plan.stats`` (voltax/sparse.py:528-535)."""
    padded = 0.0
    ref_work = 0
    for sel in classes:
        m, kp, rp = len(sel), int(k[sel].max()), int(r[sel].max())
        padded += m * (2.0 * kp**3 + 2.0 * kp * kp * rp + 2.0 * kp * rp * rp)
        ref_work += m * (kp * kp + 2 * kp * rp)
    flops = float(np.sum(2.0 * k**3 + 2.0 * k * k * r + 2.0 * k * r * r))
    return dict(supernodes=len(k), levels=int(level.max()) + 1, buckets=len(classes),
                factor_entries=int(np.sum(k * k + 2 * k * r)), work=ref_work,
                flops=flops, padded_flops=padded, largest_supernode=int(k.max()),
                pivot_groups=G)


def make_plan(st: Structure, leaf: int | None = None) -> Plan:
    """Symbolic factorization (voltax/sparse.py:412-535) plus the GPU panel
    layout and per-level gather tables, by the C++ planner
    (`voltax_gb300/csrc/symbolic.cpp`, `libvxg_symbolic.so`)."""
    return _make_plan_native(st, LEAF_SIZE if leaf is None else leaf)


# =============================================================================
# The C++ planner
# =============================================================================

_FIELDS = ("gid", "sn_ptr", "sn_idx", "parent", "bd_ptr", "bd_idx", "level", "cls_ptr",
           "cls_idx", "k", "r", "panel", "sn_of", "pos_in", "a_pos", "lv_ptr", "lv_sn",
           "lv_schur_off", "lv_bord_off", "lv_schur_len", "lv_bord_len", "lv_st_ptr",
           "st_tgt", "st_ptr", "st_src", "lv_bt_ptr", "bt_tgt", "bt_ptr", "bt_src")
"""Field ids of vxs_plan_copy, in the order of include/vxg_symbolic.h."""


@functools.lru_cache(maxsize=1)
def _symlib():
    import ctypes as C

    from . import build
    lib = C.CDLL(str(build.build_symbolic()))
    P, I64 = C.c_void_p, C.c_int64
    lib.vxs_plan_create.argtypes = [I64, P, P, I64, P, P, I64, C.POINTER(C.c_void_p)]
    lib.vxs_plan_create.restype = C.c_int
    lib.vxs_plan_len.argtypes = [P, C.c_int32]
    lib.vxs_plan_len.restype = I64
    lib.vxs_plan_copy.argtypes = [P, C.c_int32, P]
    lib.vxs_plan_copy.restype = C.c_int
    lib.vxs_plan_take.argtypes = [P, C.c_int32, P]
    lib.vxs_plan_take.restype = C.c_int
    lib.vxs_plan_destroy.argtypes = [P]
    lib.vxs_plan_destroy.restype = None
    lib.vxs_last_error.argtypes = []
    lib.vxs_last_error.restype = C.c_char_p
    return lib


def native_fields(st: Structure, leaf: int) -> dict[str, np.ndarray]:
    """Every field of the C++ plan of `st`, as int64 arrays (each moved out
    of the library's memory as it is copied)."""
    import ctypes as C

    lib = _symlib()
    indptr = np.ascontiguousarray(st.indptr, np.int64)
    indices = np.ascontiguousarray(st.indices, np.int64)
    ua, ub = union_pairs(st)
    h = C.c_void_p()
    rc = lib.vxs_plan_create(st.size, indptr.ctypes.data, indices.ctypes.data, len(ua),
                             ua.ctypes.data, ub.ctypes.data, leaf, C.byref(h))
    if rc != 0:
        msg = lib.vxs_last_error().decode()
        raise (AssertionError if rc == 2 else ValueError)(msg)
    try:
        out = {}
        for fid, name in enumerate(_FIELDS):
            a = np.empty(lib.vxs_plan_len(h, fid), np.int64)
            if lib.vxs_plan_take(h, fid, a.ctypes.data) != 0:
                raise ValueError(lib.vxs_last_error().decode())
            out[name] = a
        return out
    finally:
        lib.vxs_plan_destroy(h)


class _Split(Sequence):
    """The rows of a CSR pair (``ptr``, ``idx``) as array views, made on
    access: a plan's supernode and border lists without one small array per
    supernode (the device upload reads the flat arrays)."""

    def __init__(self, ptr: np.ndarray, idx: np.ndarray):
        self._ptr, self._idx = ptr, idx

    def __len__(self) -> int:
        return max(len(self._ptr) - 1, 0)

    def __getitem__(self, i):
        if isinstance(i, slice):
            return [self[j] for j in range(*i.indices(len(self)))]
        if i < 0:
            i += len(self)
        if not 0 <= i < len(self):
            raise IndexError(i)
        return self._idx[self._ptr[i]:self._ptr[i + 1]]


def _split(ptr: np.ndarray, idx: np.ndarray) -> _Split:
    return _Split(ptr, idx)


class _Levels(Sequence):
    """The per-level `LevelTable` views of a C++ plan, made on access (the
    flat arrays are what the library uploads)."""

    def __init__(self, f: dict):
        self._f = f

    def __len__(self) -> int:
        return len(self._f["lv_ptr"]) - 1

    def __getitem__(self, lv):
        if isinstance(lv, slice):
            return [self[i] for i in range(*lv.indices(len(self)))]
        if lv < 0:
            lv += len(self)
        if not 0 <= lv < len(self):
            raise IndexError(lv)
        f = self._f
        a, b = f["lv_ptr"][lv], f["lv_ptr"][lv + 1]
        ta, tb = f["lv_st_ptr"][lv], f["lv_st_ptr"][lv + 1]
        sptr = f["st_ptr"][ta:tb + 1]
        ba, bb = f["lv_bt_ptr"][lv], f["lv_bt_ptr"][lv + 1]
        bptr = f["bt_ptr"][ba:bb + 1]
        return LevelTable(
            f["lv_sn"][a:b], f["lv_schur_off"][a:b], int(f["lv_schur_len"][lv]),
            f["st_tgt"][ta:tb], sptr - sptr[0], f["st_src"][sptr[0]:sptr[-1]],
            f["lv_bord_off"][a:b], int(f["lv_bord_len"][lv]),
            f["bt_tgt"][ba:bb], bptr - bptr[0], f["bt_src"][bptr[0]:bptr[-1]])


def _make_plan_native(st: Structure, leaf: int) -> Plan:
    f = native_fields(st, leaf)
    k, r, level = f["k"], f["r"], f["level"]
    classes = _split(f["cls_ptr"], f["cls_idx"])
    G = int(f["gid"].max()) + 1 if st.size else 0
    return Plan(st.size, _split(f["sn_ptr"], f["sn_idx"]), f["parent"],
                _split(f["bd_ptr"], f["bd_idx"]), level, classes,
                _stats(k, r, level, classes, G), k, r, f["panel"],
                int(np.sum(k * k + 2 * k * r)), f["a_pos"], _Levels(f), f["sn_of"],
                f["pos_in"], st, f)
