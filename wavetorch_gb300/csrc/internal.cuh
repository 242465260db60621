// Structures and launchers shared between the translation units.
#pragma once
#include "common.cuh"

namespace wt {

// Per-step epilogue of the plain sequence forward: sources and probes.
// srcmap/probemap are per-cell heads of singly linked entry lists (-1: none).
struct SeqEpilogue {
    const int* srcmap;        // [nx*ny] first source entry index or -1
    const int* src_next;      // [n_src] next entry at the same cell or -1
    const int* src_row;       // [n_src] input row (-1 = own instance)
    const float* x;           // [batch][steps]
    int steps;
    int t;
    const int* probemap;      // [nx*ny] first probe entry or -1
    const int* probe_next;    // [n_probe]
    const int* probe_kind;    // [n_probe]
    float* out;               // [batch][steps][n_probe]
    float* amp;               // [batch][steps][n_probe] raw amplitudes (adjoint seeds)
    int n_probe;
    // per tile of the vector kernels (STEP4_TX x STEP4_TY cells): nonzero when
    // a source or probe lies in it; null = look up the maps at every cell
    const int* tileflag;
    int tiles_y;
};

// Tile of the vector (float4) per-step kernels: rows x columns.
constexpr int STEP4_TX = 8;
constexpr int STEP4_TY = 128;

// Per-step epilogue of the plain sequence adjoint.
struct AdjEpilogue {
    const int* probemap;
    const int* probe_next;         // per-cell chain in descending reference order
    const int* probe_kind;
    const float* grad_out;         // [batch][steps][n_probe]
    const float* amp;              // [batch][steps][n_probe]
    int n_probe, steps, t;
    const int* srcmap;
    const int* src_next;
    const int* src_row;
    float* grad_x;                 // [batch][steps] or null
    const int* tileflag;           // as SeqEpilogue::tileflag
    int tiles_y;
    // batch of one: accumulate dL/dc here directly (the batch reduction's
    // arithmetic for one instance) instead of writing the step's term
    float* G;
    int first;
};

// Parameters of the fused persistent kernels.
struct FusedParams {
    StepScalars k;
    int batch, nx, ny, steps;
    int C;          // CTAs per instance (cluster size)
    int R;          // rows per CTA (multiple of M)
    int NCP;        // threads per strip row (ny rounded up to 32)
    int LD;         // tile column stride (floats)
    int seg;        // checkpoint interval
    int PB;         // probe chunk length (steps staged in shared memory per flush/load)
    const float* b;         // [nx,ny], or [batch][nx][ny] when coef_stride != 0
    const float* c;         // likewise
    size_t coef_stride;     // floats between instances' b / c (0: shared by the batch)
    const float* x;         // [batch][steps]
    // sources in table order, probes in descending reference order
    int n_src;
    const int* src_cell;
    const int* src_row;
    int n_prb;
    const int* prb_cell;
    const int* prb_kind;
    const int* prb_col;
    const int* prb_kind_col;    // kind of output column q
    // forward outputs
    float* out;             // [batch][steps][n_prb]
    float* amp;             // [batch][steps][n_prb]
    float* fields;          // [batch][steps][nx][ny] or null
    float* psum;            // [batch][n_prb] Kahan time sums of out, or null
    float* ckpt;            // [nseg][2][batch][nx][ny]
    // adjoint
    const float* grad_out;  // [batch][steps][n_prb]
    const float* grad_w;    // [batch][n_prb] dLoss/d(sum_t out), used instead of grad_out if set
    float* gc_part;         // [batch][nx][ny] per-instance dL/dc
    float* grad_x;          // [batch][steps] or null
    float* stash;           // global stash [batch][C][seg][M][nthreads] (unless in smem)
    int stash_smem;         // 1: the stash lives in shared memory after the tiles
    // tape mode: the forward stores Lap(h_{t-1}) of every cell and step, the
    // adjoint streams it back instead of recomputing segments
    float* lap;             // [steps][batch][C][M/V][threads][V] or null (checkpoint mode)
    int nbuf;               // tape slices in the adjoint's shared-memory ring
    // nonlinear cell (wavetorch/cell.py:8-9, :93-101): b and c formed every
    // step from the field; the tape then holds Lap(h_{t-1}) and h_{t-1}
    const float* rho;       // density (as b, c: shared or per instance)
    float b0, uth, cnl;     // satdamp_b0, satdamp_uth, c_nl (float32 values)
    float* grho_part;       // [batch][nx][ny] per-instance direct dL/drho
    int* err;
    // band form (grids too large for one cluster): C is the number of bands
    // per instance; the bands' boundary rows travel through global memory
    unsigned long long* halo;   // [batch][band][from above | from below][2][NCP] tagged words
    int* abort_g;               // launch-wide abort word (a wait gave up)
    int mute_band1;             // test hook: band index + 1 whose forward never sends; 0: none
    int mute_cta1;              // test hook: cluster forward, CTA index + 1 of instance 0
                                // that never sends its boundary rows; 0: none
    int skip_slice1;            // test hook: cluster tape adjoint, step + 1 whose tape
                                // slice is never issued; 0: none
    // band layout from checkpoints: a launch runs the steps [t_lo, t_hi) only
    // (t_hi 0: the whole sequence), its tape is the segment's stash (step t
    // at t - t_lo), `recompute` 1 in the forward launches that rebuild a
    // segment (no outputs), and the adjoint keeps its per-cell state between
    // its segment launches in bstate [batch][band][3][M][threads]
    int t_lo, t_hi;
    int recompute;
    float* bstate;
};

// Up to INT_SCATTER_CAP int writes base[idx[i]] = val[i], passed by value as
// kernel parameters (24 KB, within the 32 KB parameter limit).
constexpr int INT_SCATTER_CAP = 3000;
struct IntScatter {
    int n;
    int idx[INT_SCATTER_CAP];
    int val[INT_SCATTER_CAP];
};

}  // namespace wt

// Launch shape of the fused kernels for one grid size.
struct WtFusedLaunch {
    int C, NCP;
    int M, R, S, LD, threads;          // adjoint kernel strips
    int fM, fR, fS, fLD, fthreads;     // forward kernel strips (fewer registers: more threads)
    int PB;                 // probe chunk length
    size_t smem_fwd;        // tiles + probe ring buffers
    size_t smem_bwd;        // tiles + seed ring buffers (+ the stash when stash_smem)
    int seg;                // checkpoint interval
    int stash_smem;
    // tape mode (see FusedParams::lap): possible when `nbuf` >= 2 slices fit;
    // the forward then runs on the adjoint's strips (M, R, LD, threads)
    int nbuf;
    size_t smem_tape;       // adjoint shared memory in tape mode
    size_t smem_fwd_tape;   // forward shared memory in tape mode
    size_t smem_bwd_base;   // adjoint shared memory before the tape ring
    int nbuf_nl;            // ring slices of the nonlinear adjoint (two-part slices)
    size_t smem_nl_coef;    // the nonlinear adjoint's per-thread coefficient words
    int nl_cache;           // ... with the step's X1, q, sat kept between its halves
    // checkpoint mode with the segment recompute beside the adjoint
    // (seq_bwd_ws_kernel: 2 x threads, a stash of two segments in global
    // memory): ring slices, shared memory, and whether the plan uses it
    int nbuf_ws;
    size_t smem_ws;
    int ws;
};

namespace wt {
// seq_bwd_ws_kernel (checkpoint adjoint with the segment recompute beside
// it): per-thread coefficient words (3 per cell, stride rounded up to odd),
// threads (two groups of the adjoint's strips), and its shared-memory layout
// in float offsets: both groups' tile slots, their halo words [4][NCP],
// their coefficients, the adjoint seeds of two segments [2][seg][n_prb],
// dL/dx of two segments [2][seg], the ring of stash slices (16-byte
// aligned) and its mbarriers (byte offset).
__host__ __device__ constexpr int ws_coef_stride(int M) { return (3 * M) | 1; }
__host__ __device__ constexpr int ws_max_threads(int M) { return M >= 10 ? 768 : 1024; }
struct WsLayout {
    int tile, haloR, haloA, coefR, coefA, seeds, gx, ring, mbar;
    __host__ __device__ WsLayout(int ny, int LD, int NCP, int NG, int M, int n_prb, int seg,
                                 int nbuf) {
        tile = (ny + 2) * LD;
        haloR = 4 * tile;
        haloA = haloR + 8 * NCP;
        coefR = haloA + 8 * NCP;
        coefA = coefR + NG * ws_coef_stride(M);
        seeds = coefA + NG * ws_coef_stride(M);
        gx = seeds + ((2 * seg * n_prb + 3) & ~3);
        ring = gx + ((2 * seg + 3) & ~3);
        mbar = 4 * (ring + nbuf * NG * M);
    }
    __host__ __device__ size_t bytes(int nbuf) const { return (size_t)mbar + 8 * (size_t)nbuf; }
};
}  // namespace wt

// Size the ring of seq_bwd_ws_kernel for a fused plan whose checkpoint
// interval L->seg is set (2 to 4 slices in shared memory): sets L->nbuf_ws
// and L->smem_ws; WT_ERR_UNSUPPORTED where the kernel does not apply.
int wt_ws_plan(int batch, int ny, int n_prb, WtFusedLaunch* L);

// Launch shape of the band kernels (see seq_band.cu).
struct WtBandLaunch {
    int PR;                 // bands per instance (CTAs per instance)
    int M, S, R;            // cells per thread, strips per band, rows per band (S * M)
    int NCP;                // threads per strip row (ny rounded up to 32)
    int LD;                 // tile column stride (floats)
    int threads;            // S * NCP
    int PB;                 // probe chunk length
    size_t smem_fwd, smem_bwd;
};

int wt_band_plan(int batch, int nx, int ny, int n_prb, int n_sm, WtBandLaunch* L);

// Work list of a ragged batch's packed launch (seq_band.cu band_list_kernel):
// one parameter block per model (batch 1, the model's pointers and band
// plan), and per CTA a range of (model, band) items in the global order.
struct WtBandList {
    const wt::FusedParams* params;
    const int* first;            // [ctas + 1]
    const int2* items;           // (model, band)
    int* abort_g;
};
int wt_launch_band_list(bool fwd, const WtBandList& L, int ctas, int M, size_t smem,
                        cudaStream_t st);
// Bytes of the band form's halo area (words and the abort word) for a plan.
size_t wt_band_halo_bytes(int batch, const WtBandLaunch& L);
int wt_launch_band(bool fwd, const wt::FusedParams& P, const WtBandLaunch& L, cudaStream_t st);
// The band layout in rounds (more bands than SMs for the batch): `ctas` CTAs,
// CTA c running items first[c] .. first[c+1]-1 of `items` ((instance, band)
// int pairs, in instance order).
int wt_launch_band_rounds(bool fwd, const wt::FusedParams& P, const WtBandLaunch& L, int ctas,
                          const int* first, const int* items, cudaStream_t st);

// fco (nullable): the forward's coefficient planes [A | Bc | c^2] of b, c
// (wt_launch_fwd_coef), read instead of forming them per cell and step.
int wt_launch_step_fwd(const StepScalars& k, int batch, int nx, int ny, int coef_batched,
                       const float* b, const float* c, const float* y1, size_t bs1,
                       const float* y2, size_t bs2, float* y, size_t bs,
                       const wt::SeqEpilogue* epi, cudaStream_t st, const float* fco = nullptr);
int wt_launch_fwd_coef(const StepScalars& k, size_t plane, const float* b, const float* c,
                       float* fco, cudaStream_t st);
int wt_launch_step_bwd(const StepScalars& k, int batch, int nx, int ny, int coef_batched,
                       const float* b, const float* c, const float* y1, const float* y2,
                       const float* g, float* gb, float* gcp, float* gy1, float* gy2,
                       cudaStream_t st);
// The adjoint's coefficient planes [X1 | Kc | Kg | Ky2] of b and c (4 x plane).
int wt_launch_adj_coef(const StepScalars& k, size_t plane, const float* b, const float* c,
                       float* kco, cudaStream_t st);
int wt_launch_seq_adj_step(const StepScalars& k, int batch, int nx, int ny, const float* b,
                           const float* c, const float* kco, const float* lam1, const float* lam2,
                           const float* hprev, size_t hbs, float* lam_out, float* gc, float* G,
                           int first, const wt::AdjEpilogue& epi, cudaStream_t st);
int wt_launch_seq_adj_reduce(int batch, size_t plane, const float* gc, float* G, int first,
                             cudaStream_t st);
int wt_launch_fill_zero(float* p, size_t n, cudaStream_t st);
int wt_launch_fill_int(int* p, size_t n, int v, cudaStream_t st);
int wt_launch_scatter_ints(int* base, const wt::IntScatter& s, cudaStream_t st);
int wt_fused_plan(int nx, int ny, int steps, int n_prb, int cluster_req, int seg_req,
                  WtFusedLaunch* L);
int wt_launch_probe_sum(int batch, int steps, int n_prb, const float* out, float* sum,
                        cudaStream_t st);
int wt_launch_loss_ce_np(int batch, int n_prb, const float* sum, const int64_t* labels,
                         float* loss, float* grad_sum, cudaStream_t st);
int wt_launch_fused(bool fwd, const wt::FusedParams& P, const WtFusedLaunch& L, cudaStream_t st);
// The same for one Laplacian order each (seq_fused.cu, parts 1 to 3).
#define WT_FUSED_ORDER_DECL(name)                                                                 \
    int wt_launch_fused_##name(bool fwd, const wt::FusedParams& P, const WtFusedLaunch& L,        \
                               cudaStream_t st);                                                  \
    int wt_launch_fused_nl_##name(bool fwd, const wt::FusedParams& P, const WtFusedLaunch& L,     \
                                  cudaStream_t st);
WT_FUSED_ORDER_DECL(seq)
WT_FUSED_ORDER_DECL(seq_unit)
WT_FUSED_ORDER_DECL(paired_unit)
// Nonlinear cell, tape mode: nbuf ring slices of two parts (Lap, field).
int wt_launch_fused_nl(bool fwd, const wt::FusedParams& P, const WtFusedLaunch& L, cudaStream_t st);
