/*
 * wavetorch_gb300 -- C ABI of the GB300 (sm_103a) time-stepping kernels for the
 * damped 2-D scalar wave equation of fancompute/wavetorch v0.2.1.
 *
 * Conventions
 *   - Every pointer argument is a DEVICE pointer (float32, C-contiguous) unless
 *     the parameter name ends in "_host".  The caller owns all memory; the only
 *     device memory the library uses beyond the caller's buffers is the
 *     workspace the caller passes in (size from the *_workspace_bytes queries).
 *   - Fields are row-major [batch][nx][ny]: x is the row index, y the column
 *     index, exactly the reference's tensor layout (wavetorch/rnn.py:39-41).
 *   - Every call is asynchronous on the given stream and returns a status code
 *     (WT_OK on success).  No exception crosses this boundary.
 *   - Arithmetic is IEEE float32 in the reference's own association order, so
 *     the per-step entry points reproduce the reference's CPU results bit for
 *     bit (see each entry point for the remaining differences).
 */
#ifndef WAVETORCH_GB300_H
#define WAVETORCH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* wt_stream_t; /* == cudaStream_t */

/* ---- status codes ------------------------------------------------------- */
#define WT_OK               0
#define WT_ERR_INVALID      1  /* bad argument (shape, index, null pointer)  */
#define WT_ERR_CUDA         2  /* a CUDA runtime call failed                 */
#define WT_ERR_TIMEOUT      3  /* a bounded device-side wait gave up         */
#define WT_ERR_UNSUPPORTED  4  /* valid request this build cannot serve      */

/* ---- Laplacian association order ---------------------------------------
 * The reference computes the 5-point Laplacian with torch conv2d
 * (wavetorch/operators.py:5-11).  On CPU torch picks oneDNN when the batch is
 * above 1 or the grid has more than 20480 cells, else an im2col+GEMM path; the
 * two sum the five taps in different orders:
 *   WT_LAP_SEQ    : ((((w*u + w*l) - 4w*c) + w*r) + w*d)   (fused multiply-adds)
 *   WT_LAP_PAIRED : (u + l) + (-4c + (r + d))              (h == 1 only)
 * u/d are the x-1/x+1 neighbours, l/r the y-1/y+1 neighbours; taps outside the
 * grid are zero (Dirichlet, conv2d padding=1).  WT_LAP_PAIRED with an h whose
 * h**-2 is not exactly 1 is refused with WT_ERR_INVALID.                    */
#define WT_LAP_SEQ     0
#define WT_LAP_PAIRED  1

/* Physics scalars shared by every entry point.  dt and h are the float32
 * values of the reference's `dt` buffer (wavetorch/cell.py:60) and the
 * geometry's `h` buffer (wavetorch/geom.py:20).                             */
typedef struct wt_scalars {
    float dt;
    float h;
    int32_t lap_order;   /* WT_LAP_SEQ or WT_LAP_PAIRED */
} wt_scalars;

/* Library version / build identification ("wavetorch_gb300 <ver> sm_103a"). */
const char* wt_version(void);
/* Human-readable text for a status code. */
const char* wt_status_string(int status);
/* Text of the last CUDA error seen by this library in the calling thread. */
const char* wt_last_error(void);
/* Number of kernels this library has launched since it was loaded (all
 * threads); a diagnostic for counting the launches of a timed region.  No
 * counterpart in the reference, which has no kernels of its own.          */
uint64_t wt_kernel_launches(void);

/* ======================================================================== *
 * 1. One leapfrog step: drop-in for TimeStep (wavetorch/cell.py:20-44).     *
 * ======================================================================== */

/* Forward, wavetorch/cell.py:12-17:
 *   y = (dt^-2 + b dt^-1)^-1 * ((2/dt^2) y1 - (dt^-2 - b dt^-1) y2 + c^2 Lap(y1))
 * b, c: [nx,ny] (coef_batched == 0) or [batch,nx,ny] (coef_batched == 1).
 * y1, y2, y: [batch,nx,ny].  Bit-exact with the reference's float32 CPU path. */
int wt_step_fwd(const wt_scalars* s, int32_t batch, int32_t nx, int32_t ny,
                int32_t coef_batched, const float* b, const float* c,
                const float* y1, const float* y2, float* y, wt_stream_t stream);

/* Backward, wavetorch/cell.py:26-44.  Each output pointer may be NULL (that
 * input needs no gradient).  When coef_batched == 0, grad_b and grad_c are
 * [nx,ny]: the [batch,nx,ny] per-instance terms are summed over the batch in
 * torch's CPU order (sequential within blocks of 16, blocks added in order),
 * which is what autograd's sum-to-shape does in the reference.  When
 * coef_batched == 1 they are [batch,nx,ny].                                 */
int wt_step_bwd(const wt_scalars* s, int32_t batch, int32_t nx, int32_t ny,
                int32_t coef_batched, const float* b, const float* c,
                const float* y1, const float* y2, const float* grad_y,
                float* grad_b, float* grad_c, float* grad_y1, float* grad_y2,
                wt_stream_t stream);

/* ======================================================================== *
 * 2. A whole sequence: drop-in for the time loop of WaveRNN.forward         *
 *    (wavetorch/rnn.py:50-70) and its backward through T TimeStep nodes.    *
 * ======================================================================== */

/* One injection: field[b, cell] += x[in_row(b), t] every step, applied after
 * the update in table order (wavetorch/source.py:15-22, rnn.py:56-57).
 * in_row == -1 means "the instance's own row b"; in_row >= 0 means that fixed
 * row of x for every instance (the reference's broadcast of a [batch] input
 * over a line of `batch` cells, source.py:19-20).                           */
typedef struct wt_source_entry {
    int32_t cell;      /* x*ny + y */
    int32_t in_row;
} wt_source_entry;

/* One probe output column q: out[b, t, q] = field[b, cell] (kind 0, WaveProbe,
 * probe.py:14-15) or its square (kind 1, WaveIntensityProbe, probe.py:26-27),
 * read after the injection.  `order` is the reference's probe index, which
 * fixes the order in which backward seeds are added (descending order).     */
typedef struct wt_probe_entry {
    int32_t cell;
    int32_t kind;
    int32_t order;
} wt_probe_entry;

#define WT_FORM_PLAIN  0   /* per-step kernels, every field kept (exact)     */
#define WT_FORM_FUSED  1   /* persistent kernels (cluster or band layout)    */

typedef struct wt_seq_desc {
    int32_t batch, nx, ny, steps;
    int32_t n_sources;
    const wt_source_entry* sources_host;   /* host array, n_sources entries  */
    int32_t n_probes;
    const wt_probe_entry* probes_host;     /* host array, n_probes entries   */
    int32_t form;                          /* WT_FORM_PLAIN / WT_FORM_FUSED  */
    int32_t segment;                       /* fused adjoint mode, see below  */
    int32_t cluster;                       /* CTAs per instance, 0 = auto,
                                              -1 = the band layout            */
    int32_t output_fields;                 /* 1: also write every field      */
    int32_t coef_batched;                  /* 1: one geometry per instance   */
    int32_t sm_count;                      /* SMs for the band layout, 0 = the
                                              current device's                */
} wt_seq_desc;

/* The fused form has two layouts.  Instances that fit on one thread-block
 * cluster (up to 256 columns; up to 256 rows with 16-CTA clusters) run one
 * cluster per instance with the band boundaries exchanged over distributed
 * shared memory.  Larger grids (up to 1024 columns) run in bands of rows, one
 * CTA per band and SM in a cooperative launch, the band boundaries exchanged
 * through global memory (a batch whose bands outnumber sm_count runs its
 * instances in rounds); that layout needs no output_fields.  From
 * checkpoints (segment > 0 or -2, or automatically past a 64 GiB tape) its
 * adjoint runs one segment at a time, last first: a launch recomputes the
 * segment's Laplacians into a one-segment stash and the next runs the
 * segment's adjoint steps from it.
 * `cluster` > 0 fixes the cluster size; -1 asks for the band layout even
 * where a cluster would hold the instance (its CTAs need not share a GPC,
 * as a cluster's must).                                                     */

/* `segment` chooses how the fused form's adjoint gets the forward's fields:
 *   -1  tape: the forward stores Lap(h_{t-1}) of every cell and step
 *       (about steps x batch x nx x ny floats of workspace, plus the padding
 *       of the kernels' strips) and the adjoint streams it back; no
 *       recompute.
 *   >0  checkpoints every `segment` steps; the adjoint recomputes each
 *       segment's forward (workspace ~ 2 fields per segment).  Where the
 *       cluster layout runs 10-cell strips (120 x 120 grids among them) one
 *       group of threads per CTA recomputes the next segment while a second
 *       runs the adjoint steps of the current one, and two segments'
 *       Laplacians (2 x segment x batch x nx x ny floats, plus strip
 *       padding) are staged in the workspace; elsewhere each segment is
 *       recomputed in shared memory or a one-segment stash before its
 *       adjoint steps.
 *    0  automatic: the tape when it takes at most 16 GiB and output_fields
 *       is 0, else checkpoints: every ceil(sqrt(steps)) steps where the
 *       two-group recompute applies, else at the largest interval whose
 *       recompute stash fits in shared memory.
 *   -2  checkpoints at that automatic interval (never the tape).
 * Both modes give identical results.  The plain form ignores it.            */

/* Bytes of workspace that wt_seq_fwd must be given and that must be handed,
 * unchanged, to wt_seq_bwd (checkpoints or the full field history, plus the
 * per-step probe amplitudes).                                               */
int wt_seq_workspace_bytes(const wt_seq_desc* d, size_t* bytes);

/* `coef_batched` = 1 gives every instance its own geometry: b and c are
 * [batch,nx,ny] and wt_seq_bwd's grad_c is [batch,nx,ny] (dLoss/dc of each
 * instance, not summed).  The reference has one geometry per WaveRNN; this
 * serves batches of different models of the same grid size (ragged batches).
 * Fused form only: the plain form returns WT_ERR_UNSUPPORTED for it.        */

/* Forward.  b, c: [nx,ny]; x: [batch,steps]; out: [batch,steps,n_probes];
 * fields (only if output_fields): [batch,steps,nx,ny]; probe_sum (nullable):
 * [batch,n_probes] Kahan-compensated time sums of out.                      */
int wt_seq_fwd(const wt_scalars* s, const wt_seq_desc* d,
               const float* b, const float* c, const float* x,
               float* out, float* fields, float* probe_sum,
               void* workspace, size_t workspace_bytes, wt_stream_t stream);

/* Backward.  grad_out: [batch,steps,n_probes] (dLoss/d out).  grad_c: [nx,ny],
 * overwritten with dLoss/dc.  grad_x (nullable): [batch,steps], overwritten
 * with dLoss/dx.  The plain form is bit-exact with the reference; the fused
 * form sums the per-instance terms over time first and then over the batch. */
int wt_seq_bwd(const wt_scalars* s, const wt_seq_desc* d,
               const float* b, const float* c, const float* x,
               const float* grad_out, float* grad_c, float* grad_x,
               void* workspace, size_t workspace_bytes, wt_stream_t stream);

/* Waits for `stream`, then reads the device-side status word that the last
 * wt_seq_fwd / wt_seq_bwd on this workspace left (bounds checks inside the
 * kernels record instead of trapping).  Returns WT_OK, WT_ERR_INVALID
 * (a device-side bounds check fired) or WT_ERR_TIMEOUT.                      */
int wt_seq_device_status(const wt_seq_desc* d, const void* workspace, size_t workspace_bytes,
                         wt_stream_t stream);

/* ---- the training loss, fused ---------------------------------------------
 * The reference trains on CrossEntropy(normalize_power(sum_t out), label)
 * (wavetorch/train.py:61-62, utils.py:35-36): the loss depends on the probe
 * series only through its time sums.  wt_loss_ce_normalize_power takes those
 * sums ([batch,n_probes], e.g. wt_seq_fwd's Kahan probe_sum) and int64 labels
 * [batch], and writes the batch-mean loss (one float) and dLoss/dsum
 * [batch,n_probes].  wt_seq_bwd_sum is wt_seq_bwd for such a loss: it takes
 * grad_sum instead of a [batch,steps,n_probes] grad_out (fused form only).
 * No counterpart in the reference, which runs the loss as torch ops.       */
int wt_loss_ce_normalize_power(int32_t batch, int32_t n_probes, const float* probe_sum,
                               const int64_t* labels, float* loss, float* grad_sum,
                               wt_stream_t stream);
int wt_seq_bwd_sum(const wt_scalars* s, const wt_seq_desc* d, const float* b, const float* c,
                   const float* x, const float* grad_sum, float* grad_c, void* workspace,
                   size_t workspace_bytes, wt_stream_t stream);

/* ---- the nonlinear cell ----------------------------------------------------
 * WaveCell with satdamp_b0 > 0 and/or c_nl != 0 (wavetorch/cell.py:8-9,
 * :93-101): every step, at every cell,
 *   b = b_pml + rho * satdamp_b0 / (1 + |h1 / satdamp_uth|^2)   (if b0 > 0)
 *   c = c_lin + (rho * c_nl) * h1^2                              (if c_nl != 0)
 * with h1 the field one step ago, then the leapfrog step with these b and c.
 * Fused form only, with the adjoint reading a two-part tape (Lap(h1), h1:
 * twice the linear tape); `segment` must be 0 or -1 and output_fields 0.
 * b: b_pml, c_lin: the linear speed, rho: the density the nonlinear terms
 * are weighted with (the geometry's raw rho), each [nx,ny] (or
 * [batch,nx,ny] with coef_batched).  The backward returns dLoss/dc_lin in
 * grad_c and the direct dLoss/drho through b and c in grad_rho (both
 * [nx,ny] summed over the batch, or per instance with coef_batched).      */
typedef struct wt_nonlinear {
    float satdamp_b0, satdamp_uth, c_nl;   /* float32 values of the buffers */
} wt_nonlinear;

int wt_seq_workspace_bytes_nl(const wt_seq_desc* d, size_t* bytes);
int wt_seq_fwd_nl(const wt_scalars* s, const wt_seq_desc* d, const wt_nonlinear* nl,
                  const float* b, const float* c_lin, const float* rho, const float* x,
                  float* out, float* probe_sum, void* workspace, size_t workspace_bytes,
                  wt_stream_t stream);
int wt_seq_bwd_nl(const wt_scalars* s, const wt_seq_desc* d, const wt_nonlinear* nl,
                  const float* b, const float* c_lin, const float* rho, const float* x,
                  const float* grad_out, float* grad_c, float* grad_rho, float* grad_x,
                  void* workspace, size_t workspace_bytes, wt_stream_t stream);

/* ======================================================================== *
 * 3. Free-form geometry: rho -> c (wavetorch/geom.py:207-233).              *
 * ======================================================================== */

typedef struct wt_geom_desc {
    int32_t nx, ny;
    int32_t blur_radius;      /* kernel is (2r+1)^2, weights from blur_kernel */
    int32_t blur_n;           /* blur passes                                  */
    float eta, beta;          /* projection parameters                        */
    float c0, c1;             /* float32 values of the c0/c1 buffers          */
} wt_geom_desc;

/* c = c0 + (c1-c0) * P(blur^n(rho)),  P(r) = (tanh(beta eta) + tanh(beta (r-eta)))
 *                                           / (tanh(beta eta) + tanh(beta (1-eta))).
 * blur_kernel: [(2r+1),(2r+1)] device weights.  work: 2*nx*ny floats scratch
 * (caller-owned) that wt_rho_to_c_bwd reads back: it holds the last blurred
 * density and the tanh values.                                              */
int wt_rho_to_c_fwd(const wt_geom_desc* g, const float* rho, const float* blur_kernel,
                    float* c, float* work, wt_stream_t stream);

/* grad_rho = (d c / d rho)^T grad_c, using `work` from the matching forward
 * (it reads the stored tanh values and reuses the rest as scratch).         */
int wt_rho_to_c_bwd(const wt_geom_desc* g, const float* rho, const float* blur_kernel,
                    const float* grad_c, float* grad_rho, float* work, wt_stream_t stream);

/* Bytes of `work` the two calls above need (2 * nx * ny floats). */
int wt_rho_to_c_work_bytes(const wt_geom_desc* g, size_t* bytes);

/* The forward above for callers that cannot hand the library a work buffer:
 * code that runs where no allocator is at hand (a C or ctypes caller without
 * torch or a memory pool) or where allocating is not allowed (a loop whose
 * device memory was budgeted up front, where a cudaMalloc would also
 * synchronise the device).  It writes the same c as wt_rho_to_c_fwd and
 * allocates nothing: its scratch is one array of WT_RHO_TO_C_NOALLOC_MAX_CELLS
 * x 2 floats (8 MiB) in the library's own static device memory.
 *   - Grids of more than WT_RHO_TO_C_NOALLOC_MAX_CELLS cells are refused with
 *     WT_ERR_UNSUPPORTED before anything runs; use wt_rho_to_c_fwd for them.
 *   - Each call looks up the current device's copy of the array (with that
 *     device current; the lookup allocates nothing), so a device reset
 *     between calls leaves no stale address behind.  The first call on a
 *     device also loads the library's device code there: make it before
 *     any stream capture begins.
 *   - Every call on a device shares that one array.  No part of it has to
 *     start at zero (each call writes every element it reads), but calls
 *     whose executions overlap (different streams, or host threads, without
 *     ordering between them) race on it and may return wrong c.
 *   - It keeps no state for wt_rho_to_c_bwd: a backward needs the forward
 *     with a caller-owned `work`.
 * No counterpart in the reference, whose rho -> c runs in torch ops that
 * allocate their intermediates.                                             */
#define WT_RHO_TO_C_NOALLOC_MAX_CELLS 1048576   /* 1024 x 1024 */
int wt_rho_to_c_fwd_noalloc(const wt_geom_desc* g, const float* rho, const float* blur_kernel,
                            float* c, wt_stream_t stream);

/* ======================================================================== *
 * 4. Hole geometry (WaveGeometryHoley, wavetorch/geom.py:88-132).           *
 * ======================================================================== */

typedef struct wt_holey_desc {
    int32_t nx, ny;
    int32_t n_holes;          /* holes used: the shortest of x, y, r         */
    float eta, beta;          /* projection parameters                       */
    float c0, c1;             /* float32 values of the c0/c1 buffers         */
} wt_holey_desc;

/* rho = P(s), s[i][j] = sum_k exp(-sqrt((i - x_k)^2 + (j - y_k)^2) / r_k)
 * (holes summed in index order), c = c0 + (c1 - c0) * rho, P as for the
 * free-form geometry.  Replaces WaveGeometryHoley._rho / .rho / .c
 * (wavetorch/geom.py:109-132).  x, y, r: n_holes device floats.  rho and c
 * ([nx, ny]) may each be NULL.  work: wt_holey_work_bytes bytes, caller-
 * owned; the forward writes the tanh values the backward reads.            */
int wt_holey_fwd(const wt_holey_desc* d, const float* x, const float* y, const float* r,
                 float* rho, float* c, float* work, wt_stream_t stream);

/* grad_x/y/r[k] = sum over cells of d(rho, c)/d(x_k, y_k, r_k) applied to
 * grad_rho and grad_c (either may be NULL), using `work` from the matching
 * forward.  Cell contributions are formed in float32 in the order of the
 * reference's autograd chain and summed in double, in a fixed order.  A hole
 * centred exactly on a cell gives NaN gradients, as in the reference (the
 * derivative of the distance at 0).                                        */
int wt_holey_bwd(const wt_holey_desc* d, const float* x, const float* y, const float* r,
                 const float* grad_rho, const float* grad_c, float* grad_x, float* grad_y,
                 float* grad_r, float* work, wt_stream_t stream);

/* Bytes of `work` the two calls above need. */
int wt_holey_work_bytes(const wt_holey_desc* d, size_t* bytes);

/* ======================================================================== *
 * 5. Ragged batches: the layout of each group of a batch of models.         *
 *    No counterpart in the reference, which trains one model at a time.     *
 * ======================================================================== */

/* One layout option of a group, with its measured time.                    */
typedef struct wt_ragged_option {
    int32_t cluster;    /* wt_seq_desc.cluster of the option (> 0, or -1: bands) */
    int32_t ctas;       /* SMs one instance occupies (the cluster size, or the
                           band layout's limit per instance)                 */
    double seconds;     /* the group's measured run with this option         */
} wt_ragged_option;

/* One group of a ragged batch: `instances` models of one grid, run side by
 * side in one launch.                                                       */
typedef struct wt_ragged_group {
    int32_t instances;
    double scale;                       /* measured run -> full step count  */
    int32_t n_options;
    const wt_ragged_option* options;    /* host array                       */
} wt_ragged_group;

/* Pick one option per group (choice[g]: an index into group g's options).
 * The groups run concurrently and share the GPU's n_sm SMs, so the choice
 * minimises SM-time (instances x ctas x seconds x scale; ties: fewer CTAs,
 * then the earlier option); the step then takes at least max(total SM-time /
 * n_sm, the longest group's time).  While the longest group's time is above
 * that SM-time bound, it moves to a faster option (of those, the least
 * SM-time; ties: the slower).  Host only; deterministic.                   */
int wt_ragged_plan(const wt_ragged_group* groups, int32_t n_groups, int32_t n_sm,
                   int32_t* choice);

/* ---- a ragged batch in one launch ------------------------------------
 * Many single-instance models of different grids and step counts advance in
 * ONE persistent, cooperative forward launch and ONE adjoint launch: one CTA
 * per SM walks a list of work items, each item a band of rows of one model
 * run for all of that model's steps (the band layout's kernels: fields in
 * registers, boundary rows exchanged through L2 with bounded waits).  A
 * model's bands run at once on different CTAs; every CTA takes its items in
 * one global order (by start time in the host's schedule), so no CTA waits
 * on a band that waits on it.  Linear cells, free-form geometries, every
 * source driven by the model's own input.  Laplacian order per model: a
 * batch of one (WT_LAP_PAIRED below 20,481 cells when h == 1, WT_LAP_SEQ
 * otherwise).                                                              */
typedef struct wt_ragged_model {
    int32_t nx, ny, steps;
    int32_t n_sources;
    const wt_source_entry* sources_host;   /* host; in_row must be -1       */
    int32_t n_probes;
    const wt_probe_entry* probes_host;     /* host                          */
    const float* b;                        /* device [nx][ny]               */
    const float* c;                        /* device [nx][ny]               */
    const float* x;                        /* device [steps]                */
    float* out;                            /* device [steps][n_probes]      */
    const float* grad_out;                 /* device [steps][n_probes]      */
    float* grad_c;                         /* device [nx][ny] (dL/dc)       */
} wt_ragged_model;

/* The host-side plan of one ragged batch (filled by wt_ragged_prepare; plain
 * data, kept by the caller and passed to the launches).                    */
typedef struct wt_ragged_plan_t {
    int32_t n_models, ctas, strip, n_items;
    size_t smem_fwd, smem_bwd;
    size_t workspace_bytes;
    size_t off_params, off_first, off_items, off_halo, halo_bytes, off_err;
    double est_steps_per_cta;              /* schedule length, band-steps    */
} wt_ragged_plan_t;

/* Device bytes of the workspace of a ragged batch on `sm_count` SMs (0: the
 * current device's) with strips of `strip` cells per thread (4 or 8; 0: the
 * tallest that every model's shared memory allows).                        */
int wt_ragged_workspace_bytes(const wt_scalars* s, const wt_ragged_model* models,
                              int32_t n_models, int32_t sm_count, int32_t strip, size_t* bytes);
/* Plan the batch (band geometry per model, the schedule), and write the
 * models' tables and launch parameters into the workspace (synchronous:
 * do it before any stream capture; the pointers of `models` are bound
 * here).  WT_ERR_UNSUPPORTED for a model the band layout cannot serve.     */
int wt_ragged_prepare(const wt_scalars* s, const wt_ragged_model* models, int32_t n_models,
                      int32_t sm_count, int32_t strip, void* workspace, size_t workspace_bytes,
                      wt_ragged_plan_t* plan);
/* The forward of every model (out), then the adjoint (grad_c; after the
 * forward on the same workspace).  Launches only: capturable.              */
int wt_ragged_fwd(const wt_ragged_plan_t* plan, void* workspace, wt_stream_t stream);
int wt_ragged_bwd(const wt_ragged_plan_t* plan, void* workspace, wt_stream_t stream);
/* WT_OK, or WT_ERR_TIMEOUT when a bounded wait of the last launch gave up
 * (synchronises the stream).                                              */
int wt_ragged_status(const wt_ragged_plan_t* plan, const void* workspace, wt_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* WAVETORCH_GB300_H */
