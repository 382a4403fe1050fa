/* vxg_symbolic.h -- host-side symbolic analysis for the supernodal LU.
 *
 * Once per topology, on the host (no GPU): pivot groups, nested dissection,
 * supernode borders and elimination levels, the reference's bucket classes,
 * and the unpadded GPU panel layout with its deterministic Schur and border
 * gathers. The result is the plan `vxg_create` (vxg.h) takes.
 *
 * Replaces voltax's symbolic phase (voltax/sparse.py:257-535): the union-find
 * of `_pivot_groups` (sparse.py:257-305; the bipartite matching that picks
 * the unions stays with the caller, scipy.sparse.csgraph), `_nested_dissection`
 * (sparse.py:308-378) and `_make_plan` (sparse.py:412-535). It computes the
 * same supernodes, borders, levels and buckets as voltax_gb300.symbolic's
 * numpy restatement, element for element.
 *
 * Thread safety: independent plans may be built concurrently; the error
 * string is per thread. All arrays are int64.
 */
#ifndef VXG_SYMBOLIC_H
#define VXG_SYMBOLIC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  VXS_OK = 0,
  VXS_ERR_INVALID = 1,   /* bad sizes or indices */
  VXS_ERR_STRUCTURE = 2, /* a pattern entry lies outside the factor structure */
  VXS_ERR_NOMEM = 3
};

/* Result fields (vxs_plan_len / vxs_plan_copy). "ptr" arrays are CSR offsets
 * (length count+1) into the matching "idx"/"src" array. */
enum {
  VXS_GID = 0,          /* S: pivot group of each unknown, numbered by root */
  VXS_SN_PTR = 1,       /* nsn+1 */
  VXS_SN_IDX = 2,       /* the unknowns of each supernode, ascending; postorder */
  VXS_PARENT = 3,       /* nsn: parent supernode, -1 for roots */
  VXS_BD_PTR = 4,       /* nsn+1 */
  VXS_BD_IDX = 5,       /* border of each supernode, ascending */
  VXS_LEVEL = 6,        /* nsn: elimination level (leaves 0) */
  VXS_CLS_PTR = 7,      /* buckets+1 */
  VXS_CLS_IDX = 8,      /* supernode ids of each bucket (voltax's padded batches) */
  VXS_K = 9,            /* nsn: supernode width */
  VXS_R = 10,           /* nsn: border length */
  VXS_PANEL = 11,       /* nsn: panel offset (F11 k*k | F12 k*r | F21 r*k) */
  VXS_SN_OF = 12,       /* S: supernode of each unknown */
  VXS_POS_IN = 13,      /* S: position of each unknown in its supernode */
  VXS_A_POS = 14,       /* nnz: panel slot of each pattern entry */
  VXS_LV_PTR = 15,      /* levels+1 into LV_SN */
  VXS_LV_SN = 16,       /* supernodes of each level, by descending k^3+k^2r+kr^2 */
  VXS_LV_SCHUR_OFF = 17,/* per LV_SN entry: offset of its r*r Schur block */
  VXS_LV_BORD_OFF = 18, /* per LV_SN entry: offset of its border block */
  VXS_LV_SCHUR_LEN = 19,/* levels */
  VXS_LV_BORD_LEN = 20, /* levels */
  VXS_LV_ST_PTR = 21,   /* levels+1 into ST_TGT */
  VXS_ST_TGT = 22,      /* unique panel targets of the Schur updates, per level */
  VXS_ST_PTR = 23,      /* len(ST_TGT)+1 into ST_SRC */
  VXS_ST_SRC = 24,      /* level-scratch indices, ascending within a target */
  VXS_LV_BT_PTR = 25,   /* levels+1 into BT_TGT */
  VXS_BT_TGT = 26,      /* unique unknowns the solves' border updates hit */
  VXS_BT_PTR = 27,      /* len(BT_TGT)+1 into BT_SRC */
  VXS_BT_SRC = 28,      /* level border-scratch indices, ascending */
  VXS_N_FIELDS = 29
};

typedef struct vxs_plan vxs_plan;

/* Builds the plan of the S x S pattern (indptr, indices: CSR, sorted columns,
 * diagonal present). Pivot groups come from the n_unions pairs
 * (union_a[i], union_b[i]), applied in order as union(a, b): the root of b's
 * set is attached under the root of a's. `leaf`: the largest nested-
 * dissection leaf kept whole (voltax/sparse.py:63). */
int vxs_plan_create(int64_t S, const int64_t* indptr, const int64_t* indices,
                    int64_t n_unions, const int64_t* union_a, const int64_t* union_b,
                    int64_t leaf, vxs_plan** out);

/* Length (elements) of a field; -1 for an unknown field. */
int64_t vxs_plan_len(const vxs_plan* p, int32_t field);

/* Copies a field into dst (vxs_plan_len elements). */
int vxs_plan_copy(const vxs_plan* p, int32_t field, int64_t* dst);

/* Copies a field into dst and frees the plan's copy of it (its length is 0
 * afterwards): the caller never holds two copies of the large gathers. */
int vxs_plan_take(vxs_plan* p, int32_t field, int64_t* dst);

void vxs_plan_destroy(vxs_plan* p);

/* Text of the calling thread's last error. */
const char* vxs_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* VXG_SYMBOLIC_H */
