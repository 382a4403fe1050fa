"""Block-LDU factorization and solves exactly as voltax lays them out (oracle).

`padded_plan` rebuilds voltax's padded per-bucket panel storage from a
symbolic plan (supernode sets, borders, bucket classes; the symbolic part is
pinned to the reference's own output by tests/golden/symbolic.json):
``F11 (m, kp, kp) | F12 (m, kp, rp) | F21 (m, rp, kp)`` per bucket, the
pattern-to-panel map ``a_pos`` and the Schur target positions
(voltax/sparse.py:474-527).

`factor` / `solve` / `spsolve_vjp` restate voltax/sparse.py:543-621: per
bucket ``W = inv(F11)`` (LAPACK LU with partial pivoting inside the block;
padded pivots get a unit diagonal), ``Ub = W F12``, ``Lb = F21 W``, Schur
update ``work[schur] -= F21 Ub``; forward ``y = x[piv]``,
``x[border] -= Lb y``, ``x[piv] = W y``; backward ``x[piv] -= Ub x[border]``;
transposed variants for the adjoint.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Bucket:
    m: int
    kp: int
    rp: int
    off: int
    piv: np.ndarray
    border: np.ndarray
    valid: np.ndarray
    schur: np.ndarray


@dataclass
class PaddedPlan:
    size: int
    work: int
    buckets: list
    a_pos: np.ndarray


def padded_plan(size, supernodes, borders, classes, rows, indices) -> PaddedPlan:
    S = size
    nsn = len(supernodes)
    k = np.array([len(s) for s in supernodes])
    r = np.array([len(b) for b in borders])
    sn_of = np.empty(S, np.int64)
    pos_in = np.empty(S, np.int64)
    for i, s in enumerate(supernodes):
        sn_of[s] = i
        pos_in[s] = np.arange(len(s))
    off = 0
    base11 = np.zeros(nsn, np.int64)
    base12 = np.zeros(nsn, np.int64)
    base21 = np.zeros(nsn, np.int64)
    KP = np.zeros(nsn, np.int64)
    RP = np.zeros(nsn, np.int64)
    layout = []
    for sel in classes:
        sel = np.asarray(sel)
        m, kp, rp = len(sel), int(k[sel].max()), int(r[sel].max())
        j = np.arange(m)
        base11[sel] = off + j * kp * kp
        base12[sel] = off + m * kp * kp + j * kp * rp
        base21[sel] = off + m * kp * kp + m * kp * rp + j * rp * kp
        KP[sel], RP[sel] = kp, rp
        layout.append((sel, m, kp, rp, off))
        off += m * (kp * kp + 2 * kp * rp)
    work = off
    bsn = np.repeat(np.arange(nsn), r)
    bvar = np.concatenate(borders) if nsn else np.zeros(0, np.int64)
    bkeys = np.asarray(bsn, np.int64) * S + np.asarray(bvar, np.int64)
    order = np.argsort(bkeys)
    bkeys = bkeys[order]
    bidx = np.concatenate([np.arange(x) for x in r])[order]

    def bpos(o, v):
        if len(bidx) == 0:
            return np.zeros(np.shape(o), np.int64)
        qq = np.searchsorted(bkeys, np.asarray(o, np.int64) * S + np.asarray(v, np.int64))
        return bidx[np.minimum(qq, len(bidx) - 1)]

    def position(u, v):
        su, sv = sn_of[u], sn_of[v]
        o = np.minimum(su, sv)
        same = base11[o] + pos_in[u] * KP[o] + pos_in[v]
        upper = base12[o] + pos_in[u] * RP[o] + bpos(o, v)
        lower = base21[o] + bpos(o, u) * KP[o] + pos_in[v]
        return np.where(su == sv, same, np.where(su < sv, upper, lower))

    a_pos = position(rows, indices)
    buckets = []
    for sel, m, kp, rp, boff in layout:
        piv = np.full((m, kp), S, np.int64)
        brd = np.full((m, rp), S, np.int64)
        schur = np.full((m, rp, rp), work, np.int64)
        for j, i in enumerate(sel):
            piv[j, : k[i]] = supernodes[i]
            brd[j, : r[i]] = borders[i]
            if r[i]:
                b = borders[i]
                schur[j, : r[i], : r[i]] = position(b[:, None], b[None, :])
        valid = np.arange(kp)[None, :] < k[sel][:, None]
        buckets.append(Bucket(m, kp, rp, boff, piv, brd, valid, schur))
    return PaddedPlan(S, work, buckets, a_pos)


def from_plan(plan, st) -> PaddedPlan:
    """`padded_plan` of a product `Plan` (its reference-equal fields)."""
    return padded_plan(st.size, plan.supernodes, plan.borders, plan.buckets,
                       st.rows, st.indices)


def _inverse(A):
    """Batched inverse; a singular block yields non-finite values (as
    ``jnp.linalg.inv`` does) instead of raising."""
    if A.shape[-1] == 1:
        with np.errstate(divide="ignore", invalid="ignore"):
            return 1.0 / A
    try:
        return np.linalg.inv(A)
    except np.linalg.LinAlgError:
        out = np.empty_like(A)
        for i, blk in enumerate(A):
            try:
                out[i] = np.linalg.inv(blk)
            except np.linalg.LinAlgError:
                out[i] = np.nan
        return out


def factor(pp: PaddedPlan, data):
    """Per bucket ``(W, Ub, Lb)`` (voltax/sparse.py:549-572)."""
    data = np.asarray(data)
    work = np.zeros(pp.work + 1, data.dtype)
    np.add.at(work, pp.a_pos, data)
    out = []
    for bk in pp.buckets:
        m, kp, rp, o = bk.m, bk.kp, bk.rp, bk.off
        F11 = work[o: o + m * kp * kp].reshape(m, kp, kp)
        F11 = F11 + np.where(bk.valid, 0.0, 1.0)[:, :, None] * np.eye(kp)
        W = _inverse(F11)
        if rp:
            o2 = o + m * kp * kp
            F12 = work[o2: o2 + m * kp * rp].reshape(m, kp, rp)
            o3 = o2 + m * kp * rp
            F21 = work[o3: o3 + m * rp * kp].reshape(m, rp, kp)
            Ub, Lb = W @ F12, F21 @ W
            np.add.at(work, bk.schur.ravel(), -(F21 @ Ub).ravel())
            work[pp.work] = 0
        else:
            Ub = Lb = None
        out.append((W, Ub, Lb))
    return out


def solve(pp: PaddedPlan, factors, b, transpose=False):
    """``A x = b`` or ``A^T x = b`` (voltax/sparse.py:575-595)."""
    b = np.asarray(b)
    x = np.concatenate([b, np.zeros(1, b.dtype)])  # index S = padding

    def get(idx):
        return np.where(idx < pp.size, x[np.minimum(idx, pp.size)], 0)

    pairs = list(zip(pp.buckets, factors))
    for bk, (W, Ub, Lb) in pairs:
        y = get(bk.piv)
        if bk.rp:
            off = Ub if transpose else np.swapaxes(Lb, 1, 2)
            np.add.at(x, bk.border.ravel(), -np.einsum("mkr,mk->mr", off, y).ravel())
        Wop = np.swapaxes(W, 1, 2) if transpose else W
        x[bk.piv.ravel()] = np.einsum("mjk,mk->mj", Wop, y).ravel()
        x[pp.size] = 0
    for bk, (W, Ub, Lb) in reversed(pairs):
        if bk.rp:
            off = np.swapaxes(Lb, 1, 2) if transpose else Ub
            np.add.at(x, bk.piv.ravel(), -np.einsum("mkr,mr->mk", off, get(bk.border)).ravel())
            x[pp.size] = 0
    return x[: pp.size]


def spsolve(pp: PaddedPlan, data, b):
    return solve(pp, factor(pp, data), b)


def spsolve_vjp(pp: PaddedPlan, st, data, b, g):
    """Cotangents ``(gdata, gb)`` of ``x = A^-1 b`` (voltax/sparse.py:608-618)."""
    factors = factor(pp, data)
    x = solve(pp, factors, b)
    gb = solve(pp, factors, g, transpose=True)
    gdata = -gb[st.rows] * x[st.indices]
    return gdata, gb
