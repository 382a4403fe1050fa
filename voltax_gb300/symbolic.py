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

Two planners give identical plans: the C++ one (`csrc/symbolic.cpp`, the
default; ~50x faster on large grids) and the numpy restatement
(`make_plan_numpy`), which is pinned to the reference's own output. The
bipartite matching of the pivot grouping runs in scipy for both.
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
NATIVE = os.environ.get("VOLTAX_SYMBOLIC", "native") != "numpy"
"""Plan with the C++ planner (`libvxg_symbolic.so`) unless VOLTAX_SYMBOLIC=numpy."""


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
    rows, cols = np.broadcast_arrays(np.asarray(rows), np.asarray(cols))
    keys = st.rows.astype(np.int64) * st.size + st.indices
    want = rows.astype(np.int64) * st.size + cols
    pos = np.searchsorted(keys, want)
    ok = (rows >= 0) & (cols >= 0)
    hit = np.where(ok, keys[np.minimum(pos, len(keys) - 1)] == want, True)
    if not hit.all():
        raise AssertionError("entry outside the sparsity pattern")
    return np.where(ok, pos, len(keys)).astype(np.int32)


def structure(circuit, leaf: int | None = None) -> Structure:
    """The cached `Structure` of `circuit`'s topology."""
    return _structure(circuit.topology_key(), LEAF_SIZE if leaf is None else leaf)


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
        idx = np.asarray(nodes, dtype=np.int64).reshape(n, -1)
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
        pos = positions(st, blocks[:, :, None], blocks[:, None, :])
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


def pivot_groups(st: Structure) -> np.ndarray:
    """Group id of every unknown (voltax/sparse.py:257-305): union-find over
    `union_pairs`, groups numbered by their root."""
    S = st.size
    parent = np.arange(S)

    def find(a):
        root = a
        while parent[root] != root:
            root = parent[root]
        while parent[a] != root:  # path compression
            parent[a], a = root, parent[a]
        return root

    for a, b in zip(*union_pairs(st)):
        ra, rb = find(int(a)), find(int(b))
        if ra != rb:
            parent[rb] = ra
    roots = np.array([find(a) for a in range(S)])
    return np.unique(roots, return_inverse=True)[1]


def _bfs_levels(sub: sp.csr_matrix, start: int) -> np.ndarray:
    return csg.shortest_path(sub, unweighted=True, indices=start)


def nested_dissection(adj: sp.csr_matrix, w: np.ndarray, leaf: int, last: np.ndarray):
    """Supernodes (vertex sets) in postorder and their parents
    (voltax/sparse.py:308-378): BFS level-structure separators from a
    pseudo-peripheral vertex, the lightest 1/3-balanced level."""
    nodes: list[tuple[np.ndarray, int]] = []
    top = -1
    if last.any():
        nodes.append((np.flatnonzero(last), -1))
        top = 0
    stack = [(np.flatnonzero(~last), top)]
    while stack:
        verts, par = stack.pop()
        if len(verts) == 0:
            continue
        sub = adj[verts][:, verts]
        ncomp, lab = csg.connected_components(sub, directed=False)
        if ncomp > 1:
            stack += [(verts[lab == c], par) for c in range(ncomp)]
            continue
        if w[verts].sum() <= leaf:
            nodes.append((verts, par))
            continue
        start = 0
        for _ in range(4):
            d = _bfs_levels(sub, start)
            far = int(np.argmax(d))
            if d[far] <= d[start] or far == start:
                break
            start = far
        d = _bfs_levels(sub, start).astype(int)
        depth = d.max()
        if depth < 2:
            nodes.append((verts, par))
            continue
        lw = np.bincount(d, weights=w[verts], minlength=depth + 1)
        cum = np.cumsum(lw)
        total = cum[-1]
        cands = [lv for lv in range(1, depth)
                 if cum[lv - 1] >= total / 3 and total - cum[lv] >= total / 3]
        if not cands:
            mid = int(np.searchsorted(cum, total / 2))
            cands = [min(max(mid, 1), depth - 1)]
        lv = min(cands, key=lambda c: lw[c])
        touches = (sub @ (d == lv + 1).astype(float)) > 0
        sep = (d == lv) & touches
        me = len(nodes)
        nodes.append((verts[sep], par))
        stack.append((verts[(d < lv) | ((d == lv) & ~touches)], me))
        stack.append((verts[d > lv], me))
    children: list[list[int]] = [[] for _ in nodes]
    roots = []
    for i, (_, p) in enumerate(nodes):
        (children[p] if p >= 0 else roots).append(i)
    order: list[int] = []
    todo = [(r, False) for r in reversed(roots)]
    while todo:
        i, done = todo.pop()
        if done:
            order.append(i)
        else:
            todo.append((i, True))
            todo += [(c, False) for c in reversed(children[i])]
    new = {old: i for i, old in enumerate(order)}
    sets = [nodes[old][0] for old in order]
    parents = np.array([new[nodes[old][1]] if nodes[old][1] >= 0 else -1
                        for old in order], dtype=np.int64)
    return sets, parents


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


def _gather_csr(targets: np.ndarray):
    """Group source indices ``0..len(targets)-1`` by target: unique targets,
    CSR pointers and sources (ascending within each target)."""
    order = np.argsort(targets, kind="stable")
    tsorted = targets[order]
    uniq, starts = np.unique(tsorted, return_index=True)
    ptr = np.append(starts, len(tsorted)).astype(np.int64)
    return uniq.astype(np.int64), ptr, order.astype(np.int64)


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


def make_plan(st: Structure, leaf: int | None = None, native: bool | None = None) -> Plan:
    """Symbolic factorization (voltax/sparse.py:412-535) plus the GPU panel
    layout and per-level gather tables.

    ``native`` (default: on unless ``VOLTAX_SYMBOLIC=numpy``) runs the C++
    planner (`voltax_gb300/csrc/symbolic.cpp`); otherwise the numpy
    restatement below. Both give identical plans."""
    leaf = LEAF_SIZE if leaf is None else leaf
    if native is None:
        native = NATIVE
    return _make_plan_native(st, leaf) if native else make_plan_numpy(st, leaf)


def make_plan_numpy(st: Structure, leaf: int | None = None) -> Plan:
    """The numpy restatement of the symbolic factorization."""
    leaf = LEAF_SIZE if leaf is None else leaf
    S = st.size
    gid = pivot_groups(st)
    G = int(gid.max()) + 1
    E = sp.csr_matrix((np.ones(S), (np.arange(S), gid)), shape=(S, G))
    P = sp.csr_matrix((np.ones(st.nnz), st.indices, st.indptr), shape=(S, S))
    Ps = (P + P.T).tocsr()
    Q = (E.T @ Ps @ E).tocsr()
    Q.setdiag(0)
    Q.eliminate_zeros()
    w = np.bincount(gid, minlength=G).astype(float)
    deg = np.diff(Q.indptr)
    if S <= 2 * leaf:
        last = np.ones(G, bool)
    else:
        last = deg > max(32.0, 8.0 * np.sqrt(G))
    qsets, parents = nested_dissection(Q, w, leaf, last)
    order = np.argsort(gid, kind="stable")
    starts = np.searchsorted(gid[order], np.arange(G + 1))
    sns = [np.sort(np.concatenate([order[starts[g]:starts[g + 1]] for g in qs]))
           for qs in qsets]
    nsn = len(sns)
    sn_of = np.empty(S, np.int64)
    pos_in = np.empty(S, np.int64)
    for i, s in enumerate(sns):
        sn_of[s] = i
        pos_in[s] = np.arange(len(s))
    children: list[list[int]] = [[] for _ in range(nsn)]
    for i, p in enumerate(parents):
        if p >= 0:
            children[p].append(i)
    borders: list[np.ndarray] = []
    level = np.zeros(nsn, np.int64)
    for i, s in enumerate(sns):
        adj = Ps.indices[np.concatenate([np.arange(Ps.indptr[v], Ps.indptr[v + 1])
                                         for v in s])]
        cand = np.unique(np.concatenate([adj] + [borders[c] for c in children[i]]))
        borders.append(cand[sn_of[cand] > i])
        if children[i]:
            level[i] = 1 + max(level[c] for c in children[i])
    k = np.array([len(s) for s in sns], np.int64)
    r = np.array([len(b) for b in borders], np.int64)

    def cost(sel):
        if len(sel) == 0:
            return 0.0
        K, R = k[sel].max(), r[sel].max()
        return len(sel) * (2.0 * K**3 + 2.0 * K * K * R + 2.0 * K * R * R + 64.0)

    classes: list[np.ndarray] = []
    for lv in range(int(level.max()) + 1):
        sel = np.flatnonzero(level == lv)
        sel = sel[np.argsort(k[sel] ** 3 + k[sel] ** 2 * r[sel] + k[sel] * r[sel] ** 2,
                             kind="stable")]
        cut = min(range(len(sel)), key=lambda c: cost(sel[:c]) + cost(sel[c:]))
        if cost(sel) - cost(sel[:cut]) - cost(sel[cut:]) < SPLIT_SAVING:
            cut = 0
        classes += [part for part in (sel[:cut], sel[cut:]) if len(part)]
    stats = _stats(k, r, level, classes, G)

    # ---- GPU layout: unpadded panels in supernode order
    sizes = k * k + 2 * k * r
    panel = np.zeros(nsn, np.int64)
    if nsn > 1:
        panel[1:] = np.cumsum(sizes)[:-1]
    work = int(sizes.sum())
    # border position lookup: (supernode, unknown) -> index in its border
    bkeys = np.concatenate([np.int64(i) * S + np.asarray(b, np.int64)
                            for i, b in enumerate(borders)]) \
        if nsn else np.zeros(0, np.int64)
    bidx = np.concatenate([np.arange(len(b)) for b in borders]) \
        if nsn else np.zeros(0, np.int64)
    border_order = np.argsort(bkeys)
    bkeys, bidx = bkeys[border_order], bidx[border_order]

    def bpos(o, v):
        key = np.asarray(o, np.int64) * S + np.asarray(v, np.int64)
        q = np.searchsorted(bkeys, key)
        qc = np.minimum(q, max(len(bkeys) - 1, 0))
        if len(bkeys) == 0 or not np.all(bkeys[qc] == key):
            raise AssertionError("entry outside the supernodal factor structure")
        return bidx[qc]

    def position(u, v):
        u, v = np.broadcast_arrays(np.asarray(u, np.int64), np.asarray(v, np.int64))
        su, sv = sn_of[u], sn_of[v]
        out = np.empty(u.shape, np.int64)
        same = su == sv
        out[same] = panel[su[same]] + pos_in[u[same]] * k[su[same]] + pos_in[v[same]]
        up = su < sv
        if up.any():
            o = su[up]
            out[up] = panel[o] + k[o] * k[o] + pos_in[u[up]] * r[o] + bpos(o, v[up])
        lo = su > sv
        if lo.any():
            o = sv[lo]
            out[lo] = (panel[o] + k[o] * k[o] + k[o] * r[o]
                       + bpos(o, u[lo]) * k[o] + pos_in[v[lo]])
        return out

    a_pos = position(st.rows, st.indices)

    # ---- per-level launch tables
    levels = []
    for lv in range(int(level.max()) + 1):
        ids = np.flatnonzero(level == lv)
        ids = ids[np.argsort(-(k[ids] ** 3 + k[ids] ** 2 * r[ids] + k[ids] * r[ids] ** 2),
                             kind="stable")]
        rr = r[ids]
        schur_off = np.zeros(len(ids), np.int64)
        if len(ids) > 1:
            schur_off[1:] = np.cumsum(rr * rr)[:-1]
        bord_off = np.zeros(len(ids), np.int64)
        if len(ids) > 1:
            bord_off[1:] = np.cumsum(rr)[:-1]
        tg, bt = [], []
        for j in ids:
            b = borders[j]
            if len(b):
                tg.append(position(b[:, None], b[None, :]).ravel())
                bt.append(b)
        if tg:
            s_t, s_p, s_s = _gather_csr(np.concatenate(tg))
            b_t, b_p, b_s = _gather_csr(np.concatenate(bt))
        else:
            s_t = b_t = np.zeros(0, np.int64)
            s_p = b_p = np.zeros(1, np.int64)
            s_s = b_s = np.zeros(0, np.int64)
        levels.append(LevelTable(ids, schur_off, int((rr * rr).sum()), s_t, s_p, s_s,
                                 bord_off, int(rr.sum()), b_t, b_p, b_s))

    return Plan(S, sns, parents, borders, level, classes, stats, k, r, panel, work,
                a_pos, levels, sn_of, pos_in, st)


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
