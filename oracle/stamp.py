"""Residual and Jacobian assembly in the canonical order (oracle).

Residual (voltax/circuit.py:209-226): per group in layout order, terminal
contributions are added into node rows and internal contributions into
internal rows, device by device, terminal by terminal; ground is dropped.

Jacobian (voltax/sparse.py:220-249): per group in layout order, device by
device, each local block is added row-major into the CSR values at its stamp
positions; entries touching ground are dropped. ``np.add.at`` applies the
additions strictly in index order, which fixes the summation order -- the
canonical order the GPU's segmented reduction reproduces bit for bit.

The residual recipes of the analyses (voltax/analysis.py:325-378) are here
too: DC ``f + gmin v``, backward Euler ``(q - q_prev)/h + f + gmin v`` and
trapezoidal ``(q - q_prev)/h + (f + f_prev)/2 + gmin v``; their Jacobians use
``(cf, cq) = (1, 0), (1, 1/h), (0.5, 1/h)`` plus gmin on node diagonals.
"""

from __future__ import annotations

import numpy as np
import torch

from .devices import F64, GroupModel


def groups_of(circuit, b: int = 0):
    """``(name, model, nodes (N, T), internal offset, k)`` in layout order."""
    out = []
    for name, n, k, off in circuit.layout.groups:
        if n == 0:
            continue
        el = circuit.elements[name]
        out.append((name, GroupModel(el, b), np.asarray(el.nodes, np.int64).reshape(n, -1),
                    off, k))
    return out


def assemble(circuit, z, fn, b: int = 0) -> np.ndarray:
    """``f`` or ``q`` of the DAE; `fn(model, v, x) -> (I, F)``."""
    z = np.asarray(z, np.float64)
    nv, S = circuit.layout.n_nodes, circuit.layout.size
    v_ext = np.concatenate([z[:nv], [0.0]])
    nodes_out = np.zeros(nv + 1)
    internal_out = np.zeros(S - nv)
    for _, model, idx, off, k in groups_of(circuit, b):
        n = idx.shape[0]
        internal_idx = np.arange(off - nv, off - nv + n * k).reshape(n, k)
        v = torch.as_tensor(v_ext[idx], dtype=F64)
        x = torch.as_tensor(z[nv + internal_idx], dtype=F64)
        I, F = fn(model, v, x)
        if I is not None:
            np.add.at(nodes_out, idx.ravel(),
                      np.broadcast_to(I.numpy(), idx.shape).ravel())
        if F is not None and k:
            np.add.at(internal_out, internal_idx.ravel(), F.numpy().ravel())
    return np.concatenate([nodes_out[:nv], internal_out])


def f(circuit, z, t, b: int = 0) -> np.ndarray:
    return assemble(circuit, z, lambda m, v, x: m.currents(v, x, t), b)


def q(circuit, z, b: int = 0) -> np.ndarray:
    return assemble(circuit, z, lambda m, v, x: m.charges(v, x), b)


def local_blocks(circuit, st, z, t, cf, cq, b: int = 0):
    """Per group ``(positions, values)`` in layout order: ``(N, m, m)`` local
    blocks, or one ``(N m, N m)`` block for a non-local group."""
    z = np.asarray(z, np.float64)
    z_ext = np.concatenate([z, [0.0]])
    out = []
    for (name, allv, T, local), (_, pos, _) in zip(st.devices, st.stamps):
        model = GroupModel(circuit.elements[name], b)
        cq_g = cq if model.has_charges else 0.0
        if cf == 0 and cq_g == 0:
            continue
        u0 = torch.as_tensor(z_ext[np.where(allv < 0, len(z_ext) - 1, allv)], dtype=F64)
        vals = (model.local_jacobian(u0, t, cf, cq_g) if local
                else model.group_jacobian(u0, t, cf, cq_g)).numpy()
        out.append((pos, vals))
    return out


def assemble_jacobian(nnz: int, blocks) -> np.ndarray:
    """Canonical-order sum of local blocks into the CSR values."""
    data = np.zeros(nnz + 1)
    for pos, vals in blocks:
        np.add.at(data, pos.ravel(), vals.ravel())
    return data[:nnz]


def jacobian(circuit, st, z, t=0.0, cf=1.0, cq=0.0, b: int = 0) -> np.ndarray:
    """Stamped values of ``cf df/dz + cq dq/dz`` (voltax/sparse.py:220-249)."""
    return assemble_jacobian(st.nnz, local_blocks(circuit, st, z, t, cf, cq, b))


def add_gmin(data, st, n_nodes, gmin):
    out = np.array(data, copy=True)
    out[st.diagonal[:n_nodes]] += gmin
    return out


# ------------------------------------------------------- analysis residuals
def with_gmin(circuit, z, gmin):
    nv = circuit.layout.n_nodes
    out = np.zeros_like(z)
    out[:nv] = gmin * z[:nv]
    return out


def dc_residual(circuit, z, t, gmin, b=0):
    return f(circuit, z, t, b) + with_gmin(circuit, z, gmin)


def be_residual(circuit, z, z_prev, t_prev, t, gmin, b=0):
    h = t - t_prev
    dq = q(circuit, z, b) - q(circuit, z_prev, b)
    return dq / h + f(circuit, z, t, b) + with_gmin(circuit, z, gmin)


def trap_residual(circuit, z, z_prev, t_prev, t, gmin, b=0):
    h = t - t_prev
    dq = q(circuit, z, b) - q(circuit, z_prev, b)
    f_mid = 0.5 * (f(circuit, z, t, b) + f(circuit, z_prev, t_prev, b))
    return dq / h + f_mid + with_gmin(circuit, z, gmin)
