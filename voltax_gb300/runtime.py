"""Host runtime around the C ABI: topology upload, parameter packing, buffers.

`Engine` owns one ``vxg_handle`` (a topology + symbolic plan resident on the
GPU) and the index tables that define the deterministic stamping order:

* residual slots: each row sums its contributions in canonical order --
  group-major, device-major, local unknown order (voltax/circuit.py:209-226);
* Jacobian slots: each CSR entry sums its contributions in canonical order --
  group-major, device-major, row-major local blocks (voltax/sparse.py:233-248).

The gathers hold storage slot ids: within a group the device contributions
are stored SoA (residual slot (i, d) at i*n + d, Jacobian slot (i, j, d) at
(i*m + j)*n + d), so the ids of one row are not ascending.

Engines are cached per topology (the analogue of voltax's cached
`structure` / `plan`, voltax/sparse.py:114-117, 150-161).
"""

from __future__ import annotations

import ctypes as C
import numpy as np
import torch

from . import _lib as L
from .symbolic import Plan, Structure


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def cuda_device() -> torch.device:
    if not torch.cuda.is_available():
        raise L.VxgError("voltax_gb300 needs a CUDA GPU (there is no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream


def tptr(t: torch.Tensor | None):
    return None if t is None else t.data_ptr()


class Tables:
    """All host index arrays of one topology (numpy, kept alive for ctypes)."""

    def __init__(self, circuit, st: Structure, plan: Plan):
        self.st, self.plan = st, plan
        S, nnz = st.size, st.nnz
        self.S, self.nnz, self.nv = S, nnz, st.n_nodes
        i64 = lambda x: np.ascontiguousarray(x, dtype=np.int64)  # noqa: E731
        i32 = lambda x: np.ascontiguousarray(x, dtype=np.int32)  # noqa: E731
        self.indptr = i64(st.indptr)
        self.indices = i32(st.indices)
        self.rows = i32(st.rows)
        col_order = np.argsort(st.indices, kind="stable")
        self.tent = i64(col_order)
        self.tptr = i64(np.concatenate([[0], np.cumsum(np.bincount(st.indices, minlength=S))]))
        self.diag = i64(st.diagonal)

        # ---- groups and stamping gathers
        offsets = ({g: (n, k, off) for g, n, k, off in circuit.layout.groups}
                   if circuit is not None else {})
        self.group_names, self.group_descs, self._nodes = [], [], []
        res_tgt, jac_tgt, res_id, jac_id = [], [], [], []
        res_base = jac_base = 0
        devices = list(zip(st.devices, st.stamps)) if circuit is not None else []
        for (name, allv, T, local), (_, pos, _) in devices:
            el = circuit.elements[name]
            n, K, off = offsets[name]
            m = T + K
            nodes = i32(allv[:, :T])
            self._nodes.append(nodes)
            wave = getattr(el, "wave_kind", -1) if hasattr(el, "value") else -1
            n_params = len(el.gpu_params())
            self.group_names.append(name)
            self.group_descs.append((el.kind, n, T, K, wave, n_params, off))
            # canonical (AoS) order: device-major, then local row (and column);
            # storage (SoA): slot (i, d) at i*n + d, slot (i, j, d) at (i*m + j)*n + d
            tg = allv.copy()  # terminal nodes then internals: the row of each slot
            tg[tg < 0] = -1
            res_tgt.append(tg.ravel())
            dd, ii = np.meshgrid(np.arange(n), np.arange(m), indexing="ij")
            res_id.append((res_base + ii * n + dd).ravel())
            # a non-local group's block covers all n*m group unknowns: device d
            # owns rows d*m .. d*m+m-1 of it, each with n*m columns
            w = m if local else n * m
            pj = pos.reshape(n, m * w).astype(np.int64)
            jac_tgt.append(np.where(pj >= nnz, -1, pj).ravel())
            dd, ee = np.meshgrid(np.arange(n), np.arange(m * w), indexing="ij")
            jac_id.append((jac_base + ee * n + dd).ravel())
            res_base += n * m
            jac_base += n * m * w
        self.n_res_slots, self.n_jac_slots = res_base, jac_base
        cat = lambda xs: np.concatenate(xs) if xs else np.zeros(0, np.int64)  # noqa: E731
        self.res_ptr, self.res_src = self._pull(cat(res_tgt), cat(res_id), S)
        self.jac_ptr, self.jac_src = self._pull(cat(jac_tgt), cat(jac_id), nnz)

        # ---- segments (independent sub-circuits, Circuit.with_segments)
        seg_of = None if circuit is None else circuit.unknown_segments()
        if seg_of is None:
            seg_of = np.zeros(S, dtype=np.int32)
        self.seg_of = i32(seg_of)
        self.n_seg = int(self.seg_of.max()) + 1 if S else 1
        counts = np.bincount(self.seg_of, minlength=self.n_seg)
        self.seg_ptr = i32(np.concatenate([[0], np.cumsum(counts)]))
        self.seg_idx = i32(np.argsort(self.seg_of, kind="stable"))

        # ---- plan
        self.sn_k = i32(plan.k)
        self.sn_r = i32(plan.r)
        self.sn_panel = i64(plan.panel)
        self.sn_piv_ptr = i64(np.concatenate([[0], np.cumsum(plan.k)]))
        self.sn_bord_ptr = i64(np.concatenate([[0], np.cumsum(plan.r)]))
        self.a_pos = i64(plan.a_pos)
        self.work = int(plan.work)
        if plan.flat is not None:  # the C++ planner's arrays already have this layout
            f = plan.flat
            self.sn_piv, self.sn_bord = i32(f["sn_idx"]), i32(f["bd_idx"])
            self.lv_ptr, self.lv_sn = i64(f["lv_ptr"]), i32(f["lv_sn"])
            self.lv_schur_off, self.lv_bord_off = i64(f["lv_schur_off"]), i64(f["lv_bord_off"])
            self.lv_schur_len, self.lv_bord_len = i64(f["lv_schur_len"]), i64(f["lv_bord_len"])
            self.lv_st_ptr, self.st_tgt = i64(f["lv_st_ptr"]), i64(f["st_tgt"])
            self.st_ptr, self.st_src = i64(f["st_ptr"]), i64(f["st_src"])
            self.lv_bt_ptr, self.bt_tgt = i64(f["lv_bt_ptr"]), i32(f["bt_tgt"])
            self.bt_ptr, self.bt_src = i64(f["bt_ptr"]), i64(f["bt_src"])
            return
        self.sn_piv = i32(np.concatenate(plan.supernodes))
        self.sn_bord = i32(np.concatenate(plan.borders) if len(plan.borders) else [])
        lv = plan.levels
        self.lv_ptr = i64(np.concatenate([[0], np.cumsum([len(x.sns) for x in lv])]))
        self.lv_sn = i32(np.concatenate([x.sns for x in lv]))
        self.lv_schur_off = i64(np.concatenate([x.schur_off for x in lv]))
        self.lv_bord_off = i64(np.concatenate([x.bord_off for x in lv]))
        self.lv_schur_len = i64([x.schur_len for x in lv])
        self.lv_bord_len = i64([x.bord_len for x in lv])
        self.lv_st_ptr = i64(np.concatenate([[0], np.cumsum([len(x.schur_tgt) for x in lv])]))
        self.st_tgt = i64(np.concatenate([x.schur_tgt for x in lv]))
        self.st_src = i64(np.concatenate([x.schur_src for x in lv]))
        src_off = np.concatenate([[0], np.cumsum([len(x.schur_src) for x in lv])])
        self.st_ptr = i64(np.concatenate([x.schur_ptr[:-1] + o for x, o in zip(lv, src_off)]
                                         + [[src_off[-1]]]))
        self.lv_bt_ptr = i64(np.concatenate([[0], np.cumsum([len(x.bord_tgt) for x in lv])]))
        self.bt_tgt = i32(np.concatenate([x.bord_tgt for x in lv]))
        self.bt_src = i64(np.concatenate([x.bord_src for x in lv]))
        bsrc_off = np.concatenate([[0], np.cumsum([len(x.bord_src) for x in lv])])
        self.bt_ptr = i64(np.concatenate([x.bord_ptr[:-1] + o for x, o in zip(lv, bsrc_off)]
                                         + [[bsrc_off[-1]]]))

    @staticmethod
    def _pull(targets: np.ndarray, slot_ids: np.ndarray, n_out: int):
        """Slots grouped by target; within a target in canonical order (the
        position in `targets`), stored as their storage ids. CSR over
        0..n_out-1."""
        keep = np.flatnonzero(targets >= 0)
        order = np.argsort(targets[keep], kind="stable")
        src = slot_ids[keep[order]].astype(np.int64)
        counts = np.bincount(targets[keep], minlength=n_out)
        ptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        return ptr, np.ascontiguousarray(src)

    def descriptor(self) -> L.TopologyDesc:
        groups = (L.GroupDesc * max(len(self.group_descs), 1))()
        for i, (kind, n, T, K, wave, n_params, off) in enumerate(self.group_descs):
            groups[i] = L.GroupDesc(kind, n, T, K, wave, n_params, off,
                                    _ptr(self._nodes[i], L.I32))
        self._groups = groups
        d = L.TopologyDesc()
        d.size, d.n_nodes, d.nnz = self.S, self.nv, self.nnz
        d.indptr, d.indices, d.rows = (_ptr(self.indptr, L.I64), _ptr(self.indices, L.I32),
                                       _ptr(self.rows, L.I32))
        d.tptr, d.tent, d.diag = (_ptr(self.tptr, L.I64), _ptr(self.tent, L.I64),
                                  _ptr(self.diag, L.I64))
        d.n_groups, d.groups = len(self.group_descs), groups
        d.n_res_slots, d.res_ptr, d.res_src = (self.n_res_slots, _ptr(self.res_ptr, L.I64),
                                               _ptr(self.res_src, L.I64))
        d.n_jac_slots, d.jac_ptr, d.jac_src = (self.n_jac_slots, _ptr(self.jac_ptr, L.I64),
                                               _ptr(self.jac_src, L.I64))
        d.n_seg, d.seg_ptr, d.seg_of = (self.n_seg, _ptr(self.seg_ptr, L.I32),
                                        _ptr(self.seg_of, L.I32))
        d.seg_idx = _ptr(self.seg_idx, L.I32)
        d.n_sn = len(self.sn_k)
        d.sn_k, d.sn_r, d.sn_panel = (_ptr(self.sn_k, L.I32), _ptr(self.sn_r, L.I32),
                                      _ptr(self.sn_panel, L.I64))
        d.sn_piv_ptr, d.sn_piv = _ptr(self.sn_piv_ptr, L.I64), _ptr(self.sn_piv, L.I32)
        d.sn_bord_ptr, d.sn_bord = _ptr(self.sn_bord_ptr, L.I64), _ptr(self.sn_bord, L.I32)
        d.work, d.a_pos = self.work, _ptr(self.a_pos, L.I64)
        d.n_levels = len(self.lv_schur_len)
        d.lv_ptr, d.lv_sn = _ptr(self.lv_ptr, L.I64), _ptr(self.lv_sn, L.I32)
        d.lv_schur_off, d.lv_bord_off = (_ptr(self.lv_schur_off, L.I64),
                                         _ptr(self.lv_bord_off, L.I64))
        d.lv_schur_len, d.lv_bord_len = (_ptr(self.lv_schur_len, L.I64),
                                         _ptr(self.lv_bord_len, L.I64))
        d.lv_st_ptr, d.st_tgt = _ptr(self.lv_st_ptr, L.I64), _ptr(self.st_tgt, L.I64)
        d.st_ptr, d.st_src = _ptr(self.st_ptr, L.I64), _ptr(self.st_src, L.I64)
        d.lv_bt_ptr, d.bt_tgt = _ptr(self.lv_bt_ptr, L.I64), _ptr(self.bt_tgt, L.I32)
        d.bt_ptr, d.bt_src = _ptr(self.bt_ptr, L.I64), _ptr(self.bt_src, L.I64)
        return d


class Engine:
    """A topology resident on the GPU (one ``vxg_handle``)."""

    def __init__(self, circuit, st: Structure, plan: Plan):
        self.device = cuda_device()
        self.lib = L.load()
        self.tables = Tables(circuit, st, plan)
        self.st, self.plan = st, plan
        self.S, self.nnz, self.nv = st.size, st.nnz, st.n_nodes
        self.n_seg = self.tables.n_seg
        h = C.c_void_p()
        L.check(self.lib.vxg_create(C.byref(self.tables.descriptor()), C.byref(h)), "vxg_create")
        self.handle = h
        self._ws: dict = {}

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.lib.vxg_destroy(h)
            except Exception:  # interpreter shutdown
                pass

    # ------------------------------------------------------------ buffers
    def workspace(self, batch: int, precision: int) -> torch.Tensor:
        key = (batch, precision)
        ws = self._ws.get(key)
        if ws is None:
            n = C.c_size_t()
            L.check(self.lib.vxg_workspace_size(self.handle, batch, precision, C.byref(n)),
                    "vxg_workspace_size")
            ws = torch.empty(max(n.value, 1), dtype=torch.uint8, device=self.device)
            self._ws = {key: ws}  # keep one workspace alive
        return ws

    def factor_buffer(self, batch: int, precision: int) -> torch.Tensor:
        n = C.c_size_t()
        L.check(self.lib.vxg_factor_size(self.handle, batch, precision, C.byref(n)),
                "vxg_factor_size")
        return torch.empty(max(n.value, 1), dtype=torch.uint8, device=self.device)

    # ------------------------------------------------------------ parameters
    def pack_params(self, circuit, batch: int | None = None):
        """``(GroupParams array, tensors kept alive, per-group row tensors)``."""
        rows_per_group, packed = [], []
        B = batch if batch is not None else circuit.batch
        arr = (L.GroupParams * L.MAX_GROUPS)()
        for i, name in enumerate(self.tables.group_names):
            rows = circuit.elements[name].gpu_params()
            rows_per_group.append(rows)
            n = circuit.elements[name].size
            batched = any(r.ndim == 2 for r in rows)
            dev_rows = [r.detach().to(self.device, torch.float64) for r in rows]
            if batched:
                t = torch.stack([r.expand(B, n) for r in dev_rows])
            else:
                t = torch.stack([r.reshape(n) for r in dev_rows])[:, None, :]
            t = t.contiguous()
            packed.append(t)
            Bp = t.shape[1]
            arr[i] = L.GroupParams(t.data_ptr(), Bp * n, n if Bp > 1 else 0)
        return arr, packed, rows_per_group


_ENGINES: dict = {}


def _kinds(circuit) -> tuple:
    if circuit is None:
        return ()
    return tuple((name, el.kind, getattr(el, "wave_kind", -1) if hasattr(el, "value") else -1)
                 for name, el in sorted(circuit.elements.items()))


def engine_for(st: Structure, circuit=None, plan: Plan | None = None) -> Engine:
    """The cached `Engine` of a structure and plan (default ``st.plan``),
    with the device tables of `circuit` when stamping is needed."""
    plan = st.plan if plan is None else plan
    key = (id(st), id(plan), _kinds(circuit), None if circuit is None else circuit.segment_hash())
    eng = _ENGINES.get(key)
    if eng is None or eng.st is not st or eng.plan is not plan:
        if circuit is None:  # linear algebra only: reuse any engine of this plan
            for (sid, pid, _, _), e in list(_ENGINES.items()):
                if sid == id(st) and pid == id(plan) and e.st is st and e.plan is plan:
                    return e
        eng = Engine(circuit, st, plan)
        _ENGINES[key] = eng
    return eng
