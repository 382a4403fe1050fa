/*
 * vxg.h -- C ABI of the GB300 (sm_103a) Newton inner loop for voltax circuits.
 *
 * Plain C types only: host descriptors hold host pointers, every array an
 * entry point reads or writes at call time is a caller-owned DEVICE buffer,
 * `stream` is a cudaStream_t passed as void*. Every call returns an int
 * status (VXG_OK = 0); no C++ exception crosses this boundary. A handle may
 * be used from several threads at once when each thread passes its own
 * stream and its own workspace.
 *
 * Batches: `batch` instances share one topology. Per-instance arrays are
 * instance-major with the strides given in each comment (S = state size,
 * nnz = pattern entries, work = panel length of the handle). A topology may
 * itself hold `n_seg` independent sub-circuits (an uneven batch concatenated
 * into one block-diagonal system); Newton convergence, damping and gmin are
 * then per segment. Instance index of (b, s) = b * n_seg + s.
 */
#ifndef VXG_H
#define VXG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes ------------------------------------------------------ */
enum {
  VXG_OK = 0,
  VXG_ERR_INVALID = 1,   /* bad argument or descriptor                      */
  VXG_ERR_CUDA = 2,      /* a CUDA runtime call failed (see vxg_last_error) */
  VXG_ERR_TOO_LARGE = 3, /* a supernode exceeds the shared-memory kernels   */
  VXG_ERR_ALLOC = 4      /* vxg_create could not allocate its tables        */
};

/* ---- per-instance Newton status bits (written to `status`) ------------- */
enum {
  VXG_ST_CONVERGED = 1, /* |dz| <= atol + rtol |z|, undamped, finite    */
  VXG_ST_NONFINITE = 2, /* the iterate or the factorization went non-finite */
  VXG_ST_MAXITER = 4    /* the iteration limit was reached              */
};

/* ---- numeric formats of the factorization ------------------------------ */
enum {
  VXG_F64 = 0, /* plain form: FP64 panels, FP64 solves                       */
  VXG_F32 = 1, /* chosen form: FP32 panels and solves + FP64 refinement     */
  VXG_C128 = 2 /* complex FP64 panels (AC small-signal; sizes only)         */
};

/* ---- device kinds (kernel parameter rows in brackets) ------------------ */
enum {
  VXG_KIND_CONDUCTANCE = 0, /* Resistor / Conductance    [g]                    */
  VXG_KIND_CAPACITOR = 1,   /* Capacitor                 [c]                    */
  VXG_KIND_VSOURCE = 2,     /* VoltageSource             [waveform rows]        */
  VXG_KIND_ISOURCE = 3,     /* CurrentSource             [waveform rows]        */
  VXG_KIND_EKV = 4,         /* EKVMOSFET [sign, i_spec, vth, dvth, n, vt, lam, c_ox, cov_w,
                                     1/n, 1/(2 vt), c_ox n vt, -(n-1)/n] */
  VXG_KIND_L1 = 5,          /* Level1MOSFET [sign, kp W/L, vth, dvth, lam, gamma, phi,
                                     smooth, cov_w, sqrt(phi), 1/(2 sqrt(phi)),
                                     1/smooth or 0] */
  VXG_KIND_DIODE = 6,       /* Diode        [is, 1/(n vt), tt, cj]                  */
  VXG_KIND_INDUCTOR = 7,    /* Inductor     [l, rs], one internal (the current)     */
  VXG_KIND_VCCS = 8,        /* VCCS         [gm], terminals (p, n, cp, cn)          */
  VXG_KIND_BJT = 9,         /* BJT          [sign, is, 1/vt, 1/bf, 1/br, 1/vaf, tf, tr,
                                             cje, cjc], terminals (c, b, e)     */
  VXG_KIND_VCVS = 10,       /* VCVS         [gain], (p, n, cp, cn) + current i      */
  VXG_KIND_CCCS = 11,       /* CCCS         [gain], (p, n, cp, cn) + sense current  */
  VXG_KIND_CCVS = 12,       /* CCVS         [r], (p, n, cp, cn) + i, sense current  */
  VXG_KIND_XFMR = 13,       /* Transformer  [l1, l2, k sqrt(l1 l2)], (p1, n1, p2, n2)
                                             + winding currents i1, i2          */
  VXG_KIND_IDEAL_OPAMP = 14,/* IdealOpAmp   [unused], (inp, inn, out) + output current */
  VXG_KIND_OPAMP = 15,      /* OpAmp        [a0, 1/rout, tau, mid, half, 1/half],
                                             (inp, inn, out) + state x          */
  VXG_KIND_SWITCH = 16,     /* Switch       [log roff, log(roff/ron), vth, 1/vwidth],
                                             (p, n, cp, cn)                     */
  VXG_KIND_COUPLED_L = 17   /* CoupledInductors [l, sqrt l, k], (p, n) + current i.
                               A non-local group (voltax/element.py:30-34,
                               sparse.py:245-247): the flux of device d is
                               sum_e M_de i_e, M_de = k sqrt(l_d l_e) for e != d
                               and l_d for e = d, so device d's three rows take
                               all 3 n unknowns of the group as columns.       */
};
enum { VXG_WAVE_CONSTANT = 0, VXG_WAVE_STEP = 1, VXG_WAVE_PULSE = 2 };

/* ---- Newton residual forms --------------------------------------------- */
enum {
  VXG_MODE_DC = 0,   /* f(z,t) + gmin v                                   */
  VXG_MODE_BE = 1,   /* (q(z) - q(z_prev))/h + f(z,t) + gmin v            */
  VXG_MODE_TRAP = 2  /* (q(z) - q(z_prev))/h + (f(z,t) + f(z_prev,t_prev))/2 + gmin v */
};

#define VXG_MAX_GROUPS 32
#define VXG_MAX_PARAM_ROWS 13 /* parameter rows of one group */

/* One element group (voltax/circuit.py:30-159 layout, voltax/element.py:66-131). */
typedef struct {
  int32_t kind, n, T, K; /* device kind, devices, terminals, internals per device */
  int32_t wave;          /* VXG_WAVE_* for sources, else -1                       */
  int32_t n_params;      /* parameter rows the kernel reads                        */
  int32_t int_offset;    /* state index of device 0's first internal unknown       */
  const int32_t* nodes;  /* host (n*T) node indices, -1 = ground                   */
} vxg_group_desc;

/* Topology + symbolic plan, all host arrays (copied by vxg_create).
 * Replaces the Structure/Plan objects of voltax/sparse.py:73-133, 381-535. */
typedef struct {
  int32_t size, n_nodes; /* S, number of node voltages (first entries of z) */
  int64_t nnz;
  const int64_t* indptr;  /* S+1 */
  const int32_t* indices; /* nnz, sorted within rows */
  const int32_t* rows;    /* nnz, row of each entry */
  const int64_t* tptr;    /* S+1, column-major view of the pattern ... */
  const int64_t* tent;    /* nnz, ... entry ids per column (ascending) */
  const int64_t* diag;    /* S, entry id of each diagonal */
  int32_t n_groups;
  const vxg_group_desc* groups;
  /* stamping: canonical-order gathers of device contributions */
  int64_t n_res_slots;    /* sum over groups of n*(T+K) */
  const int64_t* res_ptr; /* S+1 */
  const int64_t* res_src; /* storage slot ids per row, in summation order */
  int64_t n_jac_slots;    /* sum over groups of n*(T+K)^2; (n*(T+K))^2 for a
                             non-local group (VXG_KIND_COUPLED_L) */
  const int64_t* jac_ptr; /* nnz+1 */
  const int64_t* jac_src; /* storage slot ids per entry, in summation order */
  /* independent sub-circuits (segments) inside the topology */
  int32_t n_seg;
  const int32_t* seg_ptr;  /* n_seg+1 offsets into seg_idx */
  const int32_t* seg_of;   /* S: segment of each unknown */
  const int32_t* seg_idx;  /* S: the unknowns of segment s, ascending, are
                              seg_idx[seg_ptr[s] .. seg_ptr[s+1]); NULL means
                              the identity (segment s = unknowns seg_ptr[s] ..) */
  /* supernodes: unpadded panels F11 (k*k) | F12 (k*r) | F21 (r*k) */
  int32_t n_sn;
  const int32_t* sn_k;
  const int32_t* sn_r;
  const int64_t* sn_panel;    /* panel offset of F11 */
  const int64_t* sn_piv_ptr;  /* n_sn+1 into sn_piv */
  const int32_t* sn_piv;      /* pivot unknowns of each supernode (sorted) */
  const int64_t* sn_bord_ptr; /* n_sn+1 into sn_bord */
  const int32_t* sn_bord;     /* border unknowns of each supernode (sorted) */
  int64_t work;               /* panel length */
  const int64_t* a_pos;       /* nnz: panel slot of each pattern entry */
  /* elimination levels */
  int32_t n_levels;
  const int64_t* lv_ptr;     /* n_levels+1 into lv_sn */
  const int32_t* lv_sn;      /* supernodes of each level */
  const int64_t* lv_schur_off; /* per lv_sn entry: offset of its r*r block */
  const int64_t* lv_bord_off;  /* per lv_sn entry: offset of its r contributions */
  const int64_t* lv_schur_len; /* n_levels */
  const int64_t* lv_bord_len;  /* n_levels */
  const int64_t* lv_st_ptr;  /* n_levels+1 into schur targets */
  const int64_t* st_tgt;     /* panel slots receiving Schur updates */
  const int64_t* st_ptr;     /* (#targets + 1) into st_src */
  const int64_t* st_src;     /* level-scratch indices, ascending */
  const int64_t* lv_bt_ptr;  /* n_levels+1 into border targets */
  const int32_t* bt_tgt;     /* unknowns receiving border updates */
  const int64_t* bt_ptr;     /* (#targets + 1) into bt_src */
  const int64_t* bt_src;     /* level border-contribution indices, ascending */
} vxg_topology_desc;

/* Parameter rows of one group for one call (device memory). Row p of
 * instance b, device d is params[p*row_stride + b*batch_stride + d]. */
typedef struct {
  const double* params;
  int64_t row_stride;
  int64_t batch_stride; /* 0: shared by all instances */
} vxg_group_params;

typedef struct {
  int32_t max_steps;  /* Newton iterations (voltax Options.max_steps)   */
  double rtol, atol;  /* convergence test                                */
  double max_dv;      /* damping: largest node-voltage update            */
  int32_t precision;  /* VXG_F64 or VXG_F32                              */
  int32_t refine;     /* FP64 refinement sweeps per solve (VXG_F32)     */
  int32_t block;      /* vxg_fused_run threads per instance: 64, 128, 256
                         or 512 (one CTA per instance), 32 (one warp per
                         instance, several per CTA; supernodes <= 32 wide),
                         or 0 for the library's choice (no counterpart) */
} vxg_newton_opts;

typedef struct vxg_handle vxg_handle;

/* Last CUDA error text of this thread (static storage). */
const char* vxg_last_error(void);

/* Upload a topology + plan. Replaces voltax's host-side Structure/Plan
 * caching (voltax/sparse.py:150-193, 412-535); the symbolic analysis itself
 * runs on the host before this call. Every index array is checked against
 * the buffer it addresses (and each group's terminals, internals and
 * parameter rows against its kind) before anything is copied:
 * VXG_ERR_INVALID names the first violated field in vxg_last_error(). */
int vxg_create(const vxg_topology_desc* desc, vxg_handle** out);
int vxg_destroy(vxg_handle* h);

/* Bytes of caller-owned scratch for `batch` instances at `precision`. */
int vxg_workspace_size(const vxg_handle* h, int32_t batch, int32_t precision, size_t* bytes);
/* Bytes of a factor buffer (panels of all instances) at `precision`. */
int vxg_factor_size(const vxg_handle* h, int32_t batch, int32_t precision, size_t* bytes);

/* Device evaluation and stamping at state z (B x S) and time t:
 *   f_out (B x S) = f(z, t), q_out (B x S) = q(z)        (either may be NULL)
 *   data_out (B x nnz) = cf df/dz + cq dq/dz + gmin on node diagonals (or NULL)
 * gmin: device array (B*n_seg) or NULL for the scalar gmin_scalar.
 * Replaces Circuit.f/q (voltax/circuit.py:196-226), sparse.jacobian
 * (voltax/sparse.py:220-249) and _add_gmin (voltax/analysis.py:359-360). */
int vxg_eval(const vxg_handle* h, int32_t batch, const vxg_group_params* params,
             const double* z, double t, double cf, double cq, const double* gmin,
             double gmin_scalar, double* f_out, double* q_out, double* data_out,
             void* workspace, void* stream);

/* Numeric refactorization of data (B x nnz, FP64) under the plan into
 * factors (vxg_factor_size bytes): per supernode W = F11^-1 (Gauss-Jordan
 * with partial pivoting inside the block), Ub = W F12, Lb = F21 W, Schur
 * updates of ancestors in a fixed order. Replaces sparse.factor
 * (voltax/sparse.py:543-572). */
int vxg_factor(const vxg_handle* h, int32_t batch, int32_t precision, const double* data,
               void* factors, void* workspace, void* stream);

/* Launch-shape autotuning of the factorization (no voltax counterpart:
 * voltax's XLA program has no launch shapes). Each elimination level whose
 * F11 fits in shared memory and whose Schur product stays on the CUDA
 * cores runs its factor kernel at a CTA width of 128, 256 or 512 threads;
 * the size rule picks one from the widest supernode. vxg_tune_factor times
 * each such level at all three widths (best of three launches, in plan
 * order, on the panels of `data`, B x nnz) and keeps the fastest for later
 * factorizations of this handle in this precision (VXG_F64 or VXG_F32).
 * factors and workspace are scratch of vxg_factor_size / vxg_workspace_size
 * bytes whose contents are left undefined; widths (optional, n_levels
 * entries, vxg_level_count) receives the choice, 0 for a level of fixed
 * shape. The width changes no arithmetic: every sum keeps its order, so the
 * factors are bitwise those of the size rule. vxg_set_factor_shapes sets the
 * widths directly (0 = size rule; NULL resets every level). Both drop the
 * handle's cached Newton graphs and synchronize nothing but the tuning
 * stream; neither may run while another thread factors with the handle. */
int vxg_level_count(const vxg_handle* h, int32_t* n_levels);
int vxg_tune_factor(vxg_handle* h, int32_t batch, int32_t precision, const double* data,
                    void* factors, void* workspace, int32_t* widths, void* stream);
int vxg_set_factor_shapes(vxg_handle* h, int32_t precision, const int32_t* widths);

/* x = A^-1 b (or A^-T b) with factors from vxg_factor; b, x are B x S FP64
 * (may alias). With VXG_F32 and data != NULL, `refine` FP64 refinement sweeps
 * r = b - A x follow the first solve. Replaces sparse.solve
 * (voltax/sparse.py:575-595). */
int vxg_solve(const vxg_handle* h, int32_t batch, int32_t precision, const void* factors,
              const double* data, const double* b, double* x, int32_t transpose,
              int32_t refine, void* workspace, void* stream);

/* y = A x (transpose: A^T x), FP64, B x S. Structure.matvec (voltax/sparse.py:130-133). */
int vxg_spmv(const vxg_handle* h, int32_t batch, const double* data, const double* x,
             double* y, int32_t transpose, void* stream);

/* gdata = -g[rows] * x[indices] (B x nnz): the data cotangent of spsolve
 * (voltax/sparse.py:614-618). */
int vxg_spsolve_gdata(const vxg_handle* h, int32_t batch, const double* g, const double* x,
                      double* gdata, void* stream);

/* One damped Newton solve per instance (voltax/analysis.py:208-233) with the
 * residual of `mode` (voltax/analysis.py:333-378). z (B x S) holds the guess
 * and receives the result; z_prev (B x S) and t_prev are read for BE/TRAP.
 * converged, iters (B*n_seg int32) are written. Instances that converge are
 * frozen while others iterate (vmap semantics). If factors != NULL the
 * factors of the final Jacobian, at the returned z, are left there (for the
 * adjoint). The loop runs on the device: the call enqueues one CUDA graph
 * (a conditional WHILE node over one Newton iteration) on `stream` and
 * returns without waiting; its counters live in `workspace`, so calls from
 * several threads on one handle need their own streams and workspaces.
 * The graph is instantiated on the first call with a given set of
 * arguments and cached on the handle. A stream that is being captured is
 * refused (VXG_ERR_INVALID): a graph with a conditional node cannot be
 * nested in the caller's graph. */
int vxg_newton(const vxg_handle* h, int32_t batch, const vxg_group_params* params,
               int32_t mode, double t, double t_prev, const double* z_prev,
               const double* gmin, double gmin_scalar, const vxg_newton_opts* opts,
               double* z, int32_t* converged, int32_t* iters, void* factors,
               void* workspace, void* stream);

/* vxg_newton restricted to the instances with mask[i] != 0 (B*n_seg int32,
 * device); the others keep z, converged and iters untouched. Used for gmin
 * stepping of a batch, where only the instances that failed the direct
 * attempt continue (voltax/analysis.py:236-266 under jax.vmap). */
int vxg_newton_masked(const vxg_handle* h, int32_t batch, const vxg_group_params* params,
                      int32_t mode, double t, double t_prev, const double* z_prev,
                      const double* gmin, double gmin_scalar, const vxg_newton_opts* opts,
                      double* z, int32_t* converged, int32_t* iters, const int32_t* mask,
                      void* workspace, void* stream);

/* Transient: for n_t time points ts (host), starting from z0 (B x S),
 * one vxg_newton per step with guess z_prev (voltax/analysis.py:434-480),
 * all enqueued on `stream` without host synchronisation (one uncached
 * Newton graph per step).
 * z_out: n_t x B x S (row 0 = z0); converged, iters: n_t x B*n_seg. */
int vxg_transient(const vxg_handle* h, int32_t batch, const vxg_group_params* params,
                  int32_t mode, int32_t n_t, const double* ts, const double* z0,
                  double gmin_scalar, const vxg_newton_opts* opts, double* z_out,
                  int32_t* converged, int32_t* iters, void* workspace, void* stream);

/* Parameter VJP of the residual: for each group g and parameter row p,
 * grads[g][p*row_stride + b*batch_stride + d] += -sum_i lam[i] d r_i/d param
 * with r = cf f(z,t) + cq q(z) (voltax/analysis.py:282-288, the
 * eqx.filter_vjp of the residual). grads has the layout of params. */
int vxg_param_vjp(const vxg_handle* h, int32_t batch, const vxg_group_params* params,
                  const double* z, double t, double cf, double cq, const double* lam,
                  double* const* grads, void* stream);

/* Shared memory one instance needs in the fused persistent kernel
 * (vxg_fused_run); VXG_ERR_TOO_LARGE when the topology is not eligible
 * (a supernode wider than 128, several segments, or more shared memory than
 * one CTA may have). */
int vxg_fused_smem(const vxg_handle* h, int32_t precision, size_t* bytes);

/* The whole analysis of every instance in ONE persistent launch: one CTA
 * per instance keeps the state, the stamps, the panels and the solves in
 * shared memory. With dc_first, the DC operating point at ts[0] is solved
 * first from the guess z0 (direct attempt of direct_steps iterations, then
 * gmin stepping over gmins[1..gmin_steps] restarting from z0,
 * voltax/analysis.py:236-266); otherwise z0 is the initial state. Then one
 * Newton solve of `mode` per time point ts[1..n_t-1] (device array),
 * warm-started from the previous state (voltax/analysis.py:434-480).
 * z_out: n_t x B x S; converged, iters: n_t x B (row 0: the DC solve). */
int vxg_fused_run(const vxg_handle* h, int32_t batch, const vxg_group_params* params,
                  int32_t mode, int32_t n_t, const double* ts, const double* z0,
                  int32_t dc_first, const double* gmins, int32_t gmin_steps,
                  int32_t direct_steps, double gmin, const vxg_newton_opts* opts,
                  double* z_out, int32_t* converged, int32_t* iters, void* stream);

/* DC sweep with continuation in ONE persistent launch (dc_sweep,
 * voltax/analysis.py:530-568): for point k = 0 .. n_points-1, parameter row
 * `row` of device `device` of group `group` takes values[k] (device array)
 * in every instance, and the DC operating point at time t is solved as in
 * vxg_fused_run's dc_first (direct attempt, then the gmin stages) starting
 * from point k-1's solution (point 0: from z0). The kernel writes the value
 * into each instance's own copy of the parameter, so that group's rows must
 * be per instance (batch_stride > 0) in writable device memory; they hold
 * the last value afterwards. z_out: n_points x B x S; converged, iters:
 * n_points x B. */
int vxg_fused_sweep(const vxg_handle* h, int32_t batch, const vxg_group_params* params,
                    int32_t group, int32_t row, int32_t device, int32_t n_points,
                    const double* values, double t, const double* z0, const double* gmins,
                    int32_t gmin_steps, int32_t direct_steps, double gmin,
                    const vxg_newton_opts* opts, double* z_out, int32_t* converged,
                    int32_t* iters, void* stream);

/* Phase timing of the fused kernel (a diagnostic; no counterpart in the
 * reference). With `cycles` != NULL (device, 8 int64, zeroed by the
 * caller), every later vxg_fused_run of the calling thread adds, summed
 * over its CTAs, the SM clock cycles spent in device evaluation [0],
 * assembly of the CSR values, panels and right-hand side [1],
 * factorization [2], solves and refinement [3], the damped update and
 * convergence test [4], and the whole kernel [5] (the rest: state
 * writes, trapezoidal f(z_prev), instance changes). NULL switches it off. */
int vxg_fused_set_profile(int64_t* cycles);

/* vxg_factor for callers that cannot allocate device memory when they
 * refactor (allocation-free plugin or custom-call hooks, real-time loops,
 * hosts whose allocator is owned by another runtime). No counterpart in
 * the reference. The per-level Schur scratch that vxg_factor takes from the
 * caller's workspace lives instead in an 8 MiB array inside this library;
 * the call allocates nothing, and data and factors are still the caller's.
 * Returns VXG_ERR_TOO_LARGE when batch * (largest level Schur scratch) *
 * element size exceeds 8 MiB. Every GPU that loads the library holds the
 * 8 MiB until exit. All calls share the array: calls that overlap on a GPU
 * race, so serialise them. The first call on a device looks up the array's
 * address; make it before any stream capture. The address is kept per
 * device and context: after a cudaDeviceReset the next call looks it up
 * again, so it too must precede any capture. */
int vxg_factor_static(const vxg_handle* h, int32_t batch, int32_t precision,
                      const double* data, void* factors, void* stream);

/* ---- Learned Newton warm start ------------------------------------------
 * No counterpart in the reference: voltax's DC Newton starts from the
 * caller's guess or zeros (voltax/analysis.py:410-431). These are the
 * kernels of an MLP that predicts a DC operating point from an instance's
 * parameter vector; the analysis then runs the ordinary Newton from the
 * prediction, and from the default guess where that fails. Layers are
 * y = act(x W^T + b): W is [out, in] BF16, b FP32, activations BF16, every
 * product accumulated in FP32. All buffers are the caller's; every kernel
 * reduces in a fixed order (bitwise reproducible). */
enum { VXG_ACT_NONE = 0, VXG_ACT_GELU = 1 /* exact erf form */ };

/* x_bf16[m, k] = bf16((x[rows[m] * ldx + k] - mean[k]) * inv_std[k]) for
 * m < M, k < K (rows NULL: identity). */
int vxg_mlp_normalize(int64_t M, int32_t K, const double* x, int64_t ldx, const int64_t* rows,
                      const float* mean, const float* inv_std, void* x_bf16, void* stream);

/* Forward layer: v = x[M, K] W[N, K]^T + bias. Optional outputs: pre[M, N] = v
 * (FP32, kept for the backward pass), y_bf16[M, N] = act(v), y_f32[M, N] =
 * act(v), and z[m * ldz + n] = act(v) * scale[n] + shift[n] in FP64 (the
 * de-normalised prediction written straight into a Newton state). */
int vxg_mlp_linear(int64_t M, int32_t N, int32_t K, const void* x_bf16, const void* w_bf16,
                   const float* bias, int32_t act, float* pre, void* y_bf16, float* y_f32,
                   const float* scale, const float* shift, double* z, int64_t ldz,
                   void* stream);

/* Data gradient of a layer: dx[M, K] = (dy[M, N] W[N, K]) * gelu'(pre[M, K]),
 * pre being the pre-activation of the layer's input (NULL: no activation). */
int vxg_mlp_linear_dx(int64_t M, int32_t N, int32_t K, const void* dy_bf16, const void* w_bf16,
                      const float* pre, void* dx_bf16, void* stream);

/* Weight gradients of a layer: dw[N, K] = dy[M, N]^T x[M, K] (FP32,
 * overwritten), db[N] = column sums of dy (NULL: skipped). */
int vxg_mlp_linear_dw(int64_t M, int32_t N, int32_t K, const void* dy_bf16, const void* x_bf16,
                      float* dw, float* db, void* stream);

/* Mean squared error of y[M, N] against target rows (target[rows[m]], rows
 * NULL: identity): *loss = sum (y - t)^2 / (M N), dy = 2 (y - t) / (M N) in
 * BF16. scratch holds 256 floats. */
int vxg_mlp_mse(int64_t M, int32_t N, const float* y, const float* target, const int64_t* rows,
                void* dy_bf16, float* loss, float* scratch, void* stream);

/* Adam step `step` (>= 1) on n FP32 master weights, with bias correction;
 * w_bf16 (if not NULL) receives the rounded weights. step == 0 only
 * rewrites w_bf16 from w. */
int vxg_mlp_adam(int64_t n, float* w, void* w_bf16, const float* grad, float* m, float* v,
                 float lr, float beta1, float beta2, float eps, int32_t step, void* stream);

/* ---- AC small-signal analysis (voltax/analysis.py:483-524) ---------------
 * A(w) = G + j w C on the topology's pattern, one instance per angular
 * frequency w = omega[f]; G, C: the FP64 CSR values of df/dz and dq/dz at
 * the operating point (vxg_eval with (cf, cq) = (1, 0) and (0, 1)), shared by
 * all frequencies. Factors are complex FP64 (interleaved re, im; size from
 * vxg_factor_size with VXG_C128), factored under the same plan and pivoting
 * rule (largest |re| + |im| in the block column). Workspace: vxg_workspace_size
 * with VXG_C128. */
int vxg_ac_factor(const vxg_handle* h, int32_t n_freq, const double* G, const double* C,
                  const double* omega, void* factors, void* workspace, void* stream);

/* x[f] = A(w_f)^-1 b[f] for every frequency; b and x complex (interleaved),
 * b[f] at b + 2 * f * b_stride (b_stride 0: one right-hand side for all). */
int vxg_ac_solve(const vxg_handle* h, int32_t n_freq, const void* factors, const double* b,
                 int64_t b_stride, double* x, void* workspace, void* stream);

/* C[M x N] = A[M x K] B[K x N] (row-major FP32, leading dimensions lda,
 * ldb, ldc) on the fifth-generation tensor cores with three TF32 products
 * per term (a_hi b_hi + a_hi b_lo + a_lo b_hi, x = x_hi + x_lo each rounded
 * to TF32) accumulated in FP32: the panel-update product of wide supernodes
 * (voltax/sparse.py:566-568 computes these products as einsums), exposed
 * on its own. *status (device int32) is set to 1 if a wait on the tensor
 * cores gave up (the result is then invalid); it is not cleared. */
int vxg_gemm_tf32x3(int32_t M, int32_t N, int32_t K, const float* A, int32_t lda, const float* B,
                    int32_t ldb, float* C, int32_t ldc, int32_t* status, void* stream);

/* Kernels this library has launched since it was loaded (a diagnostic
 * counter; no counterpart in the reference). */
uint64_t vxg_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* VXG_H */
