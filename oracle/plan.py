"""numpy restatement of voltax's symbolic planner (TEST INFRASTRUCTURE:
the checker of the product's C++ planner, `voltax_gb300/csrc/symbolic.cpp`;
only tests/ use it).

It follows the reference step for step, so that its plans can be compared
field by field with the C++ planner's and with the fixtures the reference's
own code produced (tests/golden):

* pivot groups: union-find over the ordered unions of
  `voltax_gb300.symbolic.union_pairs` (voltax/sparse.py:257-305);
* nested dissection: BFS level-structure separators from a
  pseudo-peripheral vertex (4 sweeps), the lightest 1/3-balanced level,
  leaves of at most `leaf` unknowns, high-degree groups into the root
  (voltax/sparse.py:308-378, 412-433);
* borders, levels and the bucket split (voltax/sparse.py:434-473) and the
  statistics (voltax/sparse.py:528-535);
* the GPU panel layout and per-level gathers of the product
  (`voltax_gb300.symbolic.Plan` / `LevelTable`).
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.csgraph as csg

from voltax_gb300.symbolic import (LEAF_SIZE, SPLIT_SAVING, LevelTable, Plan, Structure,
                                   _stats, union_pairs)


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


def _gather_csr(targets: np.ndarray):
    """Group source indices ``0..len(targets)-1`` by target: unique targets,
    CSR pointers and sources (ascending within each target)."""
    order = np.argsort(targets, kind="stable")
    tsorted = targets[order]
    uniq, starts = np.unique(tsorted, return_index=True)
    ptr = np.append(starts, len(tsorted)).astype(np.int64)
    return uniq.astype(np.int64), ptr, order.astype(np.int64)


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
