// Per-step ("plain") kernels: one launch advances every instance of the batch
// by one leapfrog step, or runs one step of the adjoint.  These are the
// drop-in for TimeStep (wavetorch/cell.py:20-44) and, with the fused source
// and probe epilogues, the plain per-step form of the sequence.
//
// Layout: fields [batch][nx][ny] float32.  A CTA of 32x8 threads covers an
// 8-row x 32-column tile; the tile plus a one-cell halo is staged in shared
// memory with coalesced loads, so each input cell is read from L2/HBM once.
#include <initializer_list>

#include "internal.cuh"

namespace wt {

constexpr int TX = 8;    // tile rows    (x)
constexpr int TY = 32;   // tile columns (y)

// Stage rows [x0-1, x0+TX] x cols [y0-1, y0+TY] of field f (one instance) into
// s[TX+2][TY+2], zero outside the grid.
WT_DEV void stage_tile(float (*s)[TY + 2], const float* __restrict__ f, int nx, int ny,
                       int x0, int y0) {
    const int tid = threadIdx.y * TY + threadIdx.x;
    constexpr int NT = TX * TY;
    constexpr int NS = (TX + 2) * (TY + 2);
    for (int i = tid; i < NS; i += NT) {
        int r = i / (TY + 2), q = i % (TY + 2);
        int gx = x0 - 1 + r, gy = y0 - 1 + q;
        float v = 0.0f;
        if (gx >= 0 && gx < nx && gy >= 0 && gy < ny) v = __ldg(f + (size_t)gx * ny + gy);
        s[r][q] = v;
    }
}

template <int ORDER>
WT_DEV float tile_lap(float (*s)[TY + 2], int r, int q, const StepScalars& k) {
    return lap5<ORDER>(s[r - 1][q], s[r][q - 1], s[r][q], s[r][q + 1], s[r + 1][q], k.lap_w,
                       k.lap_w4);
}

// ---------------------------------------------------------------------------
// Forward step, optionally with the sequence epilogue:
//   y = leapfrog(b, c, y1, y2); y[src] += x[.., t]; out[b, t, q] = probe(y)
template <int ORDER, bool EPI>
__global__ void __launch_bounds__(TX* TY)
step_fwd_kernel(StepScalars k, int nx, int ny, int coef_batched, const float* __restrict__ b,
                const float* __restrict__ c, const float* __restrict__ y1, size_t bs1,
                const float* __restrict__ y2, size_t bs2, float* __restrict__ y, size_t bs,
                SeqEpilogue e) {
    __shared__ float s[TX + 2][TY + 2];
    const int inst = blockIdx.z;
    const int x0 = blockIdx.y * TX, y0 = blockIdx.x * TY;
    const size_t plane = (size_t)nx * ny;
    stage_tile(s, y1 + inst * bs1, nx, ny, x0, y0);
    __syncthreads();
    const int gx = x0 + threadIdx.y, gy = y0 + threadIdx.x;
    if (gx >= nx || gy >= ny) return;
    const size_t cell = (size_t)gx * ny + gy;
    const size_t ci = coef_batched ? inst * plane + cell : cell;
    FwdCoef f = fwd_coef(__ldg(b + ci), __ldg(c + ci), k);
    const int r = threadIdx.y + 1, q = threadIdx.x + 1;
    float L = tile_lap<ORDER>(s, r, q, k);
    float v = leapfrog(f.A, f.Bc, f.c2, k.two_over, s[r][q], __ldg(y2 + inst * bs2 + cell), L);
    if (EPI) {
        // Sources, in table order (wavetorch/rnn.py:56-57, source.py:15-22).
        for (int en = __ldg(e.srcmap + cell); en >= 0; en = __ldg(e.src_next + en)) {
            int row = __ldg(e.src_row + en);
            row = row < 0 ? inst : row;
            v = fadd(v, __ldg(e.x + (size_t)row * e.steps + e.t));
        }
        // Probes (wavetorch/probe.py:14-15, :26-27).
        for (int en = __ldg(e.probemap + cell); en >= 0; en = __ldg(e.probe_next + en)) {
            size_t o = ((size_t)inst * e.steps + e.t) * e.n_probe + en;
            e.out[o] = __ldg(e.probe_kind + en) ? fmul(v, v) : v;
            if (e.amp) e.amp[o] = v;
        }
    }
    y[inst * bs + cell] = v;
}

// ---------------------------------------------------------------------------
// TimeStep.backward drop-in (wavetorch/cell.py:26-44).  One thread per cell;
// the batch is walked in order so that the [nx,ny] reductions of grad_b and
// grad_c use torch's CPU summation order (blocks of 16 summed sequentially,
// block sums added in order).
template <int ORDER>
__global__ void __launch_bounds__(TX* TY)
step_bwd_kernel(StepScalars k, int batch, int nx, int ny, int coef_batched,
                const float* __restrict__ b, const float* __restrict__ c,
                const float* __restrict__ y1, const float* __restrict__ y2,
                const float* __restrict__ g, float* __restrict__ grad_b,
                float* __restrict__ grad_c, float* __restrict__ grad_y1,
                float* __restrict__ grad_y2) {
    __shared__ float sy[TX + 2][TY + 2];
    __shared__ float sg[TX + 2][TY + 2];
    const int x0 = blockIdx.y * TX, y0 = blockIdx.x * TY;
    const size_t plane = (size_t)nx * ny;
    const int gx = x0 + threadIdx.y, gy = y0 + threadIdx.x;
    const bool live = gx < nx && gy < ny;
    const size_t cell = live ? (size_t)gx * ny + gy : 0;
    const int r = threadIdx.y + 1, q = threadIdx.x + 1;
    const bool need_lap_y = grad_b || grad_c;
    float acc_b = 0.f, blk_b = 0.f, acc_c = 0.f, blk_c = 0.f;
    // With [nx,ny] coefficients the per-cell constants are loop invariant.
    float bb = 0.f, cc = 0.f;
    if (live && !coef_batched) { bb = __ldg(b + cell); cc = __ldg(c + cell); }
    for (int inst = 0; inst < batch; ++inst) {
        __syncthreads();
        if (need_lap_y) stage_tile(sy, y1 + inst * plane, nx, ny, x0, y0);
        if (grad_y1) {
            // c2_grad = (X1 * c^2) * g must be staged with its halo: it is the
            // field the Laplacian of grad_y1 acts on.
            const int tid = threadIdx.y * TY + threadIdx.x;
            for (int i = tid; i < (TX + 2) * (TY + 2); i += TX * TY) {
                int rr = i / (TY + 2), qq = i % (TY + 2);
                int hx = x0 - 1 + rr, hy = y0 - 1 + qq;
                float v = 0.f;
                if (hx >= 0 && hx < nx && hy >= 0 && hy < ny) {
                    size_t hc = (size_t)hx * ny + hy;
                    size_t hi = coef_batched ? inst * plane + hc : hc;
                    BwdCoef kb = bwd_coef(__ldg(b + hi), __ldg(c + hi), k);
                    v = fmul(kb.Kg, __ldg(g + inst * plane + hc));
                }
                sg[rr][qq] = v;
            }
        }
        __syncthreads();
        if (!live) continue;
        const size_t ic = inst * plane + cell;
        if (coef_batched) { bb = __ldg(b + ic); cc = __ldg(c + ic); }
        BwdCoef kb = bwd_coef(bb, cc, k);
        const float gv = __ldg(g + ic);
        float L = 0.f;
        if (need_lap_y) L = tile_lap<ORDER>(sy, r, q, k);
        if (grad_c) {
            float t = fmul(fmul(kb.X1, fmul(kb.Kc, L)), gv);
            if (coef_batched) grad_c[ic] = t;
            else {
                blk_c = fadd(blk_c, t);
                if ((inst & 15) == 15 || inst == batch - 1) {
                    acc_c = inst < 16 ? blk_c : fadd(acc_c, blk_c);
                    blk_c = 0.f;
                }
            }
        }
        if (grad_b) {
            // -(dt*b+1).pow(-2) * dt * (c^2 dt^2 Lap + 2 y1 - 2 y2) * g
            float v = fadd(fmul(bb, k.dt), 1.0f);
            float kb1 = fmul(-fdiv(1.0f, fmul(v, v)), k.dt);
            float inner = fadd(fmul(fmul(fmul(cc, cc), k.dt2), L), fmul(2.0f, sy[r][q]));
            inner = fsub(inner, fmul(2.0f, __ldg(y2 + ic)));
            float t = fmul(fmul(kb1, inner), gv);
            if (coef_batched) grad_b[ic] = t;
            else {
                blk_b = fadd(blk_b, t);
                if ((inst & 15) == 15 || inst == batch - 1) {
                    acc_b = inst < 16 ? blk_b : fadd(acc_b, blk_b);
                    blk_b = 0.f;
                }
            }
        }
        if (grad_y1) {
            float lg = lap5<ORDER>(sg[r - 1][q], sg[r][q - 1], sg[r][q], sg[r][q + 1], sg[r + 1][q],
                                   k.lap_w, k.lap_w4);
            grad_y1[ic] = fadd(fmul(k.dt2, lg), fmul(fmul(2.0f, gv), kb.X1));
        }
        if (grad_y2) grad_y2[ic] = fmul(kb.Ky2, gv);
    }
    if (live && !coef_batched) {
        if (grad_c) grad_c[cell] = acc_c;
        if (grad_b) grad_b[cell] = acc_b;
    }
}

// ---------------------------------------------------------------------------
// Plain sequence adjoint, phase 1 (one launch per step t, t = T-1 .. 0):
//   lam_t = (gy2_{t+2} + gy1_{t+1}) then probe seeds in descending probe order
// with gy1_{t+1} = dt^2 Lap(Kg lam_{t+1}) + (2 lam_{t+1}) X1 and
// gy2_{t+2} = Ky2 lam_{t+2}.  Also writes the per-instance grad_c term
//   gc[b] = (X1 * (Kc * Lap(h_{t-1}))) * lam_t
// and, at source cells, dL/dx.  lam_{t+1}, lam_{t+2} may be null (t >= T-1,
// t >= T-2), h_{t-1} is null at t == 0.
template <int ORDER>
__global__ void __launch_bounds__(TX* TY)
seq_adj_step_kernel(StepScalars k, int nx, int ny, const float* __restrict__ b,
                    const float* __restrict__ c, const float* __restrict__ lam1,
                    const float* __restrict__ lam2, const float* __restrict__ hprev, size_t hbs,
                    float* __restrict__ lam_out, float* __restrict__ gc, AdjEpilogue e) {
    __shared__ float sg[TX + 2][TY + 2];
    __shared__ float sy[TX + 2][TY + 2];
    const int inst = blockIdx.z;
    const int x0 = blockIdx.y * TX, y0 = blockIdx.x * TY;
    const size_t plane = (size_t)nx * ny;
    const int tid = threadIdx.y * TY + threadIdx.x;
    for (int i = tid; i < (TX + 2) * (TY + 2); i += TX * TY) {
        int rr = i / (TY + 2), qq = i % (TY + 2);
        int hx = x0 - 1 + rr, hy = y0 - 1 + qq;
        float v = 0.f, w = 0.f;
        if (hx >= 0 && hx < nx && hy >= 0 && hy < ny) {
            size_t hc = (size_t)hx * ny + hy;
            if (lam1) {
                BwdCoef kb = bwd_coef(__ldg(b + hc), __ldg(c + hc), k);
                v = fmul(kb.Kg, __ldg(lam1 + inst * plane + hc));
            }
            if (hprev) w = __ldg(hprev + inst * hbs + hc);
        }
        sg[rr][qq] = v;
        sy[rr][qq] = w;
    }
    __syncthreads();
    const int gx = x0 + threadIdx.y, gy = y0 + threadIdx.x;
    if (gx >= nx || gy >= ny) return;
    const size_t cell = (size_t)gx * ny + gy;
    const size_t ic = inst * plane + cell;
    const int r = threadIdx.y + 1, q = threadIdx.x + 1;
    BwdCoef kb = bwd_coef(__ldg(b + cell), __ldg(c + cell), k);
    // gradient arriving at h_t: first gy2 from step t+2, then gy1 from t+1
    float lam = 0.f;
    if (lam2) lam = fmul(kb.Ky2, __ldg(lam2 + ic));
    if (lam1) {
        float l1 = __ldg(lam1 + ic);
        float lg = lap5<ORDER>(sg[r - 1][q], sg[r][q - 1], sg[r][q], sg[r][q + 1], sg[r + 1][q],
                               k.lap_w, k.lap_w4);
        float gy1 = fadd(fmul(k.dt2, lg), fmul(fmul(2.0f, l1), kb.X1));
        lam = lam2 ? fadd(lam, gy1) : gy1;
    }
    // probe seeds, highest probe index first (autograd runs the later-created
    // IndexBackward nodes first); intensity: g * (2 y), amplitude: g.
    int head = __ldg(e.probemap + cell);
    if (head >= 0) {
        // entries of one cell are linked in descending probe order on the host
        for (int en = head; en >= 0; en = __ldg(e.probe_next + en)) {
            size_t o = ((size_t)inst * e.steps + e.t) * e.n_probe + en;
            float gv = __ldg(e.grad_out + o);
            float s = __ldg(e.probe_kind + en) ? fmul(gv, fmul(2.0f, __ldg(e.amp + o))) : gv;
            lam = fadd(lam, s);
        }
    }
    lam_out[ic] = lam;
    if (gc || e.G) {
        float L = hprev ? tile_lap<ORDER>(sy, r, q, k) : 0.0f;
        const float t = fmul(fmul(kb.X1, fmul(kb.Kc, L)), lam);
        if (e.G) {
            const float acc = fadd(0.f, t);
            e.G[cell] = e.first ? acc : fadd(e.G[cell], acc);
        } else {
            gc[ic] = t;
        }
    }
    if (e.grad_x) {
        for (int en = __ldg(e.srcmap + cell); en >= 0; en = __ldg(e.src_next + en)) {
            int row = __ldg(e.src_row + en);
            // per-instance rows only (own-row injections); broadcast rows are
            // reduced on the host side of the API.
            if (row < 0) e.grad_x[(size_t)inst * e.steps + e.t] = lam;
        }
    }
}

// ---------------------------------------------------------------------------
// Vector (float4) per-step kernels, for rows of a multiple of 4 cells with
// 16-byte aligned fields: a CTA of 8 x 32 threads covers an 8-row x
// 128-column tile, each thread 4 consecutive cells of one row.  The tile and
// its halo are staged with coalesced float4 loads (rows x0-1 .. x0+8, columns
// y0-4 .. y0+131, whole 4-cell chunks, zero outside the grid); a thread reads
// its centre, upper and lower rows as float4 and its left / right neighbours
// from the adjacent lanes.  The arithmetic per cell is the scalar kernels'.
constexpr int S4W = STEP4_TY + 8;      // staged columns per row (y0-4 .. y0+131)

WT_DEV void stage_tile4(float (*s)[S4W], const float* __restrict__ f, int nx, int ny, int x0,
                        int y0) {
    const int tid = threadIdx.y * 32 + threadIdx.x;
    constexpr int CH = S4W / 4;        // float4 chunks per staged row
    for (int i = tid; i < (STEP4_TX + 2) * CH; i += STEP4_TX * 32) {
        const int rr = i / CH, j = i - rr * CH;
        const int gx = x0 - 1 + rr, gy = y0 - 4 + 4 * j;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gx >= 0 && gx < nx && gy >= 0 && gy < ny)
            v = __ldg(reinterpret_cast<const float4*>(f + (size_t)gx * ny + gy));
        *reinterpret_cast<float4*>(&s[rr][4 * j]) = v;
    }
}

// The thread's 4 cells of row r (columns q0 .. q0+3 of the staged tile):
// centre, up, down and the left / right neighbours of each.
struct Quad {
    float c[4], u[4], d[4], l[4], r[4];
};
WT_DEV void load_quad(Quad& Q, float (*s)[S4W], int r, int q0) {
    float4 C = *reinterpret_cast<const float4*>(&s[r][q0]);
    float4 U = *reinterpret_cast<const float4*>(&s[r - 1][q0]);
    float4 D = *reinterpret_cast<const float4*>(&s[r + 1][q0]);
    Q.c[0] = C.x; Q.c[1] = C.y; Q.c[2] = C.z; Q.c[3] = C.w;
    Q.u[0] = U.x; Q.u[1] = U.y; Q.u[2] = U.z; Q.u[3] = U.w;
    Q.d[0] = D.x; Q.d[1] = D.y; Q.d[2] = D.z; Q.d[3] = D.w;
    float left = __shfl_up_sync(0xffffffffu, C.w, 1);
    float right = __shfl_down_sync(0xffffffffu, C.x, 1);
    if (threadIdx.x == 0) left = s[r][q0 - 1];
    if (threadIdx.x == 31) right = s[r][q0 + 4];
    Q.l[0] = left; Q.l[1] = C.x; Q.l[2] = C.y; Q.l[3] = C.z;
    Q.r[0] = C.y; Q.r[1] = C.z; Q.r[2] = C.w; Q.r[3] = right;
}

template <int ORDER, bool EPI>
__global__ void __launch_bounds__(STEP4_TX * 32)
step_fwd4_kernel(StepScalars k, int nx, int ny, int coef_batched, const float* __restrict__ b,
                 const float* __restrict__ c, const float* __restrict__ fco,
                 const float* __restrict__ y1, size_t bs1,
                 const float* __restrict__ y2, size_t bs2, float* __restrict__ y, size_t bs,
                 SeqEpilogue e) {
    __shared__ __align__(16) float s[STEP4_TX + 2][S4W];
    const int inst = blockIdx.z;
    const int x0 = blockIdx.y * STEP4_TX, y0 = blockIdx.x * STEP4_TY;
    const size_t plane = (size_t)nx * ny;
    const int gx = x0 + threadIdx.y, gy = y0 + 4 * threadIdx.x;
    const bool mine = gx < nx && gy < ny;
    const size_t cell = mine ? (size_t)gx * ny + gy : 0;
    const size_t ci = coef_batched ? inst * plane + cell : cell;
    // the thread's own operands first, in flight while the tile is staged;
    // with coefficient planes (fco: [A | Bc | c^2], formed once per sequence)
    // b4, c4, a4 carry A, Bc, c^2 instead of b, c
    float4 b4 = make_float4(0.f, 0.f, 0.f, 0.f), c4 = b4, a4 = b4, p4 = b4;
    if (mine) {
        if (fco) {
            a4 = __ldg(reinterpret_cast<const float4*>(fco + cell));
            b4 = __ldg(reinterpret_cast<const float4*>(fco + plane + cell));
            c4 = __ldg(reinterpret_cast<const float4*>(fco + 2 * plane + cell));
        } else {
            b4 = __ldg(reinterpret_cast<const float4*>(b + ci));
            c4 = __ldg(reinterpret_cast<const float4*>(c + ci));
        }
        p4 = __ldg(reinterpret_cast<const float4*>(y2 + inst * bs2 + cell));
    }
    stage_tile4(s, y1 + inst * bs1, nx, ny, x0, y0);
    __syncthreads();
    Quad Q;
    load_quad(Q, s, threadIdx.y + 1, 4 + 4 * threadIdx.x);   // all lanes: the shuffles need them
    if (!mine) return;
    const float bb[4] = {b4.x, b4.y, b4.z, b4.w}, cc[4] = {c4.x, c4.y, c4.z, c4.w};
    const float aa[4] = {a4.x, a4.y, a4.z, a4.w};
    const float pp[4] = {p4.x, p4.y, p4.z, p4.w};
    float v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        FwdCoef f;
        if (fco) { f.A = aa[j]; f.Bc = bb[j]; f.c2 = cc[j]; }
        else     f = fwd_coef(bb[j], cc[j], k);
        const float L = lap5<ORDER>(Q.u[j], Q.l[j], Q.c[j], Q.r[j], Q.d[j], k.lap_w, k.lap_w4);
        v[j] = leapfrog(f.A, f.Bc, f.c2, k.two_over, Q.c[j], pp[j], L);
    }
    if (EPI && (!e.tileflag || __ldg(e.tileflag + blockIdx.y * e.tiles_y + blockIdx.x))) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            for (int en = __ldg(e.srcmap + cell + j); en >= 0; en = __ldg(e.src_next + en)) {
                int row = __ldg(e.src_row + en);
                row = row < 0 ? inst : row;
                v[j] = fadd(v[j], __ldg(e.x + (size_t)row * e.steps + e.t));
            }
            for (int en = __ldg(e.probemap + cell + j); en >= 0; en = __ldg(e.probe_next + en)) {
                size_t o = ((size_t)inst * e.steps + e.t) * e.n_probe + en;
                e.out[o] = __ldg(e.probe_kind + en) ? fmul(v[j], v[j]) : v[j];
                if (e.amp) e.amp[o] = v[j];
            }
        }
    }
    *reinterpret_cast<float4*>(y + inst * bs + cell) = make_float4(v[0], v[1], v[2], v[3]);
}

// The same step with the coefficient planes, streamed by rows: a warp runs
// STEP4R_ROWS consecutive rows of one 128-column chunk (lane: 4 cells of
// each row), with every field and coefficient word it needs loaded before
// any is used -- the rows above and below from registers, the left / right
// neighbours from the adjacent lanes and, at a chunk's edges, from memory.
// No shared memory and no barrier: each warp keeps 22 16-byte loads in
// flight instead of a tile's staging round.  Warps of a CTA take
// consecutive row groups of one instance; all rows of a warp lie in one
// STEP4_TX-row tile.  The arithmetic per cell is step_fwd4_kernel's.
constexpr int STEP4R_ROWS = 4;
constexpr int STEP4R_WARPS = 4;
constexpr int ADJ4R_ROWS = 1;     // the adjoint's rows per warp (more operands per row)
// The row-streaming kernels serve sequences of at least this many cells per
// step (batch x grid); below it the tile kernels' shorter chains per warp win.
// Forward / adjoint us per step at 120x120, tiles against rows (CUDA graph):
// B=32 3.3 / 8.0 vs 4.5 / 9.1; B=128 7.1 / 17.3 vs 7.6 / 20.9; B=256 (3.7 M
// cells) 11.2 / 29.2 vs 11.3 / 29.9; B=512 21.3 / 60.3 vs 20.2 / 51.0; B=1024
// 45.4 / 118.6 vs 40.8 / 88.3.
constexpr size_t STREAM_MIN_CELLS = size_t(4) << 20;
static_assert(STEP4_TX % STEP4R_ROWS == 0, "row groups inside one tile");

template <int ORDER, bool EPI>
__global__ void __launch_bounds__(STEP4R_WARPS * 32, 4)
step_fwd4r_kernel(StepScalars k, int nx, int ny, const float* __restrict__ fco,
                  const float* __restrict__ y1, size_t bs1, const float* __restrict__ y2,
                  size_t bs2, float* __restrict__ y, size_t bs, SeqEpilogue e) {
    constexpr int R = STEP4R_ROWS;
    const int inst = blockIdx.z;
    const int x0 = (blockIdx.y * STEP4R_WARPS + threadIdx.y) * R;
    if (x0 >= nx) return;                       // whole warps only
    const int lane = threadIdx.x, y0 = blockIdx.x * STEP4_TY, gy = y0 + 4 * lane;
    const bool colv = gy < ny;
    const size_t plane = (size_t)nx * ny;
    const float* f1 = y1 + inst * bs1;
    const float* f2 = y2 + inst * bs2;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 Y[R + 2], P[R], A[R], B[R], C2[R];
    float le[R], re[R];
#pragma unroll
    for (int i = 0; i < R + 2; ++i) {
        const int gx = x0 - 1 + i;
        Y[i] = colv && gx >= 0 && gx < nx ? __ldg(reinterpret_cast<const float4*>(f1 + (size_t)gx * ny + gy))
                                          : z4;
    }
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const int gx = x0 + i;
        const bool v = colv && gx < nx;
        const size_t cell = (size_t)gx * ny + gy;
        P[i] = v ? __ldg(reinterpret_cast<const float4*>(f2 + cell)) : z4;
        A[i] = v ? __ldg(reinterpret_cast<const float4*>(fco + cell)) : z4;
        B[i] = v ? __ldg(reinterpret_cast<const float4*>(fco + plane + cell)) : z4;
        C2[i] = v ? __ldg(reinterpret_cast<const float4*>(fco + 2 * plane + cell)) : z4;
        le[i] = lane == 0 && y0 > 0 && gx < nx ? __ldg(f1 + (size_t)gx * ny + y0 - 1) : 0.f;
        re[i] = lane == 31 && y0 + STEP4_TY < ny && gx < nx
                    ? __ldg(f1 + (size_t)gx * ny + y0 + STEP4_TY) : 0.f;
    }
    const bool taps = EPI && (!e.tileflag ||
                              __ldg(e.tileflag + (x0 / STEP4_TX) * e.tiles_y + blockIdx.x));
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const int gx = x0 + i;
        if (gx >= nx) break;                    // uniform over the warp
        const float4 C = Y[i + 1], U = Y[i], D = Y[i + 2];
        float left = __shfl_up_sync(0xffffffffu, C.w, 1);
        float right = __shfl_down_sync(0xffffffffu, C.x, 1);
        if (lane == 0) left = le[i];
        if (lane == 31) right = re[i];
        const float c[4] = {C.x, C.y, C.z, C.w}, u[4] = {U.x, U.y, U.z, U.w};
        const float d[4] = {D.x, D.y, D.z, D.w};
        const float l[4] = {left, C.x, C.y, C.z}, r[4] = {C.y, C.z, C.w, right};
        const float aa[4] = {A[i].x, A[i].y, A[i].z, A[i].w};
        const float bb[4] = {B[i].x, B[i].y, B[i].z, B[i].w};
        const float cc[4] = {C2[i].x, C2[i].y, C2[i].z, C2[i].w};
        const float pp[4] = {P[i].x, P[i].y, P[i].z, P[i].w};
        if (!colv) continue;
        const size_t cell = (size_t)gx * ny + gy;
        float v[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float L = lap5<ORDER>(u[j], l[j], c[j], r[j], d[j], k.lap_w, k.lap_w4);
            v[j] = leapfrog(aa[j], bb[j], cc[j], k.two_over, c[j], pp[j], L);
        }
        if (taps) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                for (int en = __ldg(e.srcmap + cell + j); en >= 0; en = __ldg(e.src_next + en)) {
                    int row = __ldg(e.src_row + en);
                    row = row < 0 ? inst : row;
                    v[j] = fadd(v[j], __ldg(e.x + (size_t)row * e.steps + e.t));
                }
                for (int en = __ldg(e.probemap + cell + j); en >= 0; en = __ldg(e.probe_next + en)) {
                    size_t o = ((size_t)inst * e.steps + e.t) * e.n_probe + en;
                    e.out[o] = __ldg(e.probe_kind + en) ? fmul(v[j], v[j]) : v[j];
                    if (e.amp) e.amp[o] = v[j];
                }
            }
        }
        *reinterpret_cast<float4*>(y + inst * bs + cell) = make_float4(v[0], v[1], v[2], v[3]);
    }
}

// The forward's time-invariant coefficients as three planes [A | Bc | c^2]
// (wavetorch/cell.py:13-16, fwd_coef's arithmetic: A holds a division),
// formed once per sequence.
__global__ void fwd_coef_kernel(StepScalars k, size_t plane, const float* __restrict__ b,
                                const float* __restrict__ c, float* __restrict__ fco) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= plane) return;
    const FwdCoef f = fwd_coef(__ldg(b + q), __ldg(c + q), k);
    fco[q] = f.A;
    fco[plane + q] = f.Bc;
    fco[2 * plane + q] = f.c2;
}

// The adjoint's time-invariant coefficients as four planes [X1 | Kc | Kg |
// Ky2] (wavetorch/cell.py:33-42, bwd_coef's arithmetic), formed once per
// sequence instead of once per cell and step (each holds a division).
__global__ void adj_coef_kernel(StepScalars k, size_t plane, const float* __restrict__ b,
                                const float* __restrict__ c, float* __restrict__ kco) {
    const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= plane) return;
    const BwdCoef kb = bwd_coef(__ldg(b + q), __ldg(c + q), k);
    kco[q] = kb.X1;
    kco[plane + q] = kb.Kc;
    kco[2 * plane + q] = kb.Kg;
    kco[3 * plane + q] = kb.Ky2;
}

// The adjoint's staged field Kg * lam_{t+1} (Kg: the coefficient plane).
WT_DEV void stage_c2g4(float (*s)[S4W], const float* __restrict__ lam, const float* __restrict__ Kg,
                       int nx, int ny, int x0, int y0) {
    const int tid = threadIdx.y * 32 + threadIdx.x;
    constexpr int CH = S4W / 4;
    for (int i = tid; i < (STEP4_TX + 2) * CH; i += STEP4_TX * 32) {
        const int rr = i / CH, j = i - rr * CH;
        const int gx = x0 - 1 + rr, gy = y0 - 4 + 4 * j;
        float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
        if (lam && gx >= 0 && gx < nx && gy >= 0 && gy < ny) {
            const size_t hc = (size_t)gx * ny + gy;
            const float4 l4 = __ldg(reinterpret_cast<const float4*>(lam + hc));
            const float4 g4 = __ldg(reinterpret_cast<const float4*>(Kg + hc));
            o = make_float4(fmul(g4.x, l4.x), fmul(g4.y, l4.y), fmul(g4.z, l4.z), fmul(g4.w, l4.w));
        }
        *reinterpret_cast<float4*>(&s[rr][4 * j]) = o;
    }
}

template <int ORDER>
__global__ void __launch_bounds__(STEP4_TX * 32)
seq_adj_step4_kernel(StepScalars k, int nx, int ny, const float* __restrict__ kco,
                     const float* __restrict__ lam1,
                     const float* __restrict__ lam2, const float* __restrict__ hprev, size_t hbs,
                     float* __restrict__ lam_out, float* __restrict__ gc, AdjEpilogue e) {
    __shared__ __align__(16) float sg[STEP4_TX + 2][S4W];
    __shared__ __align__(16) float sy[STEP4_TX + 2][S4W];
    const int inst = blockIdx.z;
    const int x0 = blockIdx.y * STEP4_TX, y0 = blockIdx.x * STEP4_TY;
    const size_t plane = (size_t)nx * ny;
    const int gx = x0 + threadIdx.y, gy = y0 + 4 * threadIdx.x;
    const bool mine = gx < nx && gy < ny;
    const size_t cell = mine ? (size_t)gx * ny + gy : 0;
    const size_t ic = inst * plane + cell;
    // the thread's own operands first, so that their loads are in flight
    // while the tiles are staged
    float4 l1v = make_float4(0.f, 0.f, 0.f, 0.f), l2v = l1v, x1v = l1v, kcv = l1v, ky2v = l1v;
    if (mine) {
        if (lam1) l1v = __ldg(reinterpret_cast<const float4*>(lam1 + ic));
        if (lam2) l2v = __ldg(reinterpret_cast<const float4*>(lam2 + ic));
        x1v = __ldg(reinterpret_cast<const float4*>(kco + cell));
        kcv = __ldg(reinterpret_cast<const float4*>(kco + plane + cell));
        ky2v = __ldg(reinterpret_cast<const float4*>(kco + 3 * plane + cell));
    }
    stage_c2g4(sg, lam1 ? lam1 + inst * plane : nullptr, kco + 2 * plane, nx, ny, x0, y0);
    if (hprev) stage_tile4(sy, hprev + inst * hbs, nx, ny, x0, y0);
    __syncthreads();
    const int r = threadIdx.y + 1, q0 = 4 + 4 * threadIdx.x;
    Quad G, Y;
    load_quad(G, sg, r, q0);
    if (hprev) load_quad(Y, sy, r, q0);
    if (!mine) return;
    const float l1[4] = {l1v.x, l1v.y, l1v.z, l1v.w}, l2[4] = {l2v.x, l2v.y, l2v.z, l2v.w};
    const float X1s[4] = {x1v.x, x1v.y, x1v.z, x1v.w}, Kcs[4] = {kcv.x, kcv.y, kcv.z, kcv.w};
    const float Ky2s[4] = {ky2v.x, ky2v.y, ky2v.z, ky2v.w};
    const bool taps = !e.tileflag || __ldg(e.tileflag + blockIdx.y * e.tiles_y + blockIdx.x);
    float lam[4], g4[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        // gradient arriving at h_t: first gy2 from step t+2, then gy1 from t+1
        float lv = 0.f;
        if (lam2) lv = fmul(Ky2s[j], l2[j]);
        if (lam1) {
            const float lg = lap5<ORDER>(G.u[j], G.l[j], G.c[j], G.r[j], G.d[j], k.lap_w, k.lap_w4);
            const float gy1 = fadd(fmul(k.dt2, lg), fmul(fmul(2.0f, l1[j]), X1s[j]));
            lv = lam2 ? fadd(lv, gy1) : gy1;
        }
        lam[j] = lv;
    }
    // probe seeds, highest probe index first (descending chains), and dL/dx:
    // a block of its own, entered only in tiles that hold taps
    if (taps) {
#pragma unroll
        for (int j = 0; j < 4; ++j)
            for (int en = __ldg(e.probemap + cell + j); en >= 0; en = __ldg(e.probe_next + en)) {
                size_t o = ((size_t)inst * e.steps + e.t) * e.n_probe + en;
                float gv = __ldg(e.grad_out + o);
                float sd = __ldg(e.probe_kind + en) ? fmul(gv, fmul(2.0f, __ldg(e.amp + o))) : gv;
                lam[j] = fadd(lam[j], sd);
            }
        if (e.grad_x) {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                for (int en = __ldg(e.srcmap + cell + j); en >= 0; en = __ldg(e.src_next + en))
                    if (__ldg(e.src_row + en) < 0) e.grad_x[(size_t)inst * e.steps + e.t] = lam[j];
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float L = hprev ? lap5<ORDER>(Y.u[j], Y.l[j], Y.c[j], Y.r[j], Y.d[j], k.lap_w, k.lap_w4)
                              : 0.0f;
        g4[j] = fmul(fmul(X1s[j], fmul(Kcs[j], L)), lam[j]);
    }
    *reinterpret_cast<float4*>(lam_out + ic) = make_float4(lam[0], lam[1], lam[2], lam[3]);
    if (e.G) {
        float4* gp = reinterpret_cast<float4*>(e.G + cell);
        float acc[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[j] = fadd(0.f, g4[j]);
        if (!e.first) {
            const float4 o = *gp;
            acc[0] = fadd(o.x, acc[0]); acc[1] = fadd(o.y, acc[1]);
            acc[2] = fadd(o.z, acc[2]); acc[3] = fadd(o.w, acc[3]);
        }
        *gp = make_float4(acc[0], acc[1], acc[2], acc[3]);
    } else if (gc) {
        *reinterpret_cast<float4*>(gc + ic) = make_float4(g4[0], g4[1], g4[2], g4[3]);
    }
}

// The same adjoint step streamed by rows, as step_fwd4r_kernel: a warp runs
// R consecutive rows of one 128-column chunk with every operand loaded
// before any is used (Kg * lam_{t+1} and h_{t-1} for rows x0-1 .. x0+R, the
// rest for its own rows), the neighbours above and below from registers,
// left and right from the adjacent lanes or, at a chunk's edges, from
// memory.  The arithmetic per cell is seq_adj_step_kernel's.
//
// A CTA of W warps serves one row group for one block of 16 instances
// (blockIdx.z): the time-invariant coefficients of its rows are loaded once,
// then its warps take one instance each per round (instance base + w).
// After each round the warps' dL/dc terms go through shared memory to the
// threads that own the cells, which add them in instance order.  So the
// block's sum of the
// step's terms -- the first stage of the batch reduction, seq_adj_reduce_
// kernel's blocks of 16 summed from 0 in instance order -- is formed here
// and one plane per block goes to gsum instead of one term plane per
// instance; with one instance the owners accumulate into e.G.
constexpr int ADJ_BLOCK = 16;
template <int ORDER, int R, int W, int MINB>
__global__ void __launch_bounds__(W * 32, MINB)
seq_adj_step4r_kernel(StepScalars k, int batch, int nx, int ny, const float* __restrict__ kco,
                      const float* __restrict__ lam1, const float* __restrict__ lam2,
                      const float* __restrict__ hprev, size_t hbs, float* __restrict__ lam_out,
                      float* __restrict__ gsum, AdjEpilogue e) {
    static_assert(STEP4_TX % R == 0, "row groups inside one tile");
    static_assert(R <= W, "one owner thread per 4-cell slot");
    __shared__ float4 part[W][R * 32];
    const int w = threadIdx.y, lane = threadIdx.x;
    const int x0 = blockIdx.y * R;              // < nx: the grid has one CTA per row group
    const int y0 = blockIdx.x * STEP4_TY, gy = y0 + 4 * lane;
    const bool colv = gy < ny;
    const size_t plane = (size_t)nx * ny;
    const float* Kg = kco + 2 * plane;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const bool taps = !e.tileflag || __ldg(e.tileflag + (x0 / STEP4_TX) * e.tiles_y + blockIdx.x);
    auto g4 = [](float4 kg, float4 l) {
        return make_float4(fmul(kg.x, l.x), fmul(kg.y, l.y), fmul(kg.z, l.z), fmul(kg.w, l.w));
    };
    // the time-invariant words of the rows (Kg with the halo rows)
    float4 KG[R + 2], X1[R], KC[R], KY[R];
    float kgl[R], kgr[R];
#pragma unroll
    for (int i = 0; i < R + 2; ++i) {
        const int gx = x0 - 1 + i;
        KG[i] = colv && gx >= 0 && gx < nx && lam1 ? __ldg(reinterpret_cast<const float4*>(Kg + (size_t)gx * ny + gy))
                                                   : z4;
    }
    const bool edges = y0 > 0 || y0 + STEP4_TY < ny;
    const bool le = lane == 0 && y0 > 0, re = lane == 31 && y0 + STEP4_TY < ny;
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const int gx = x0 + i;
        const bool v = colv && gx < nx;
        const size_t cell = (size_t)gx * ny + gy;
        X1[i] = v ? __ldg(reinterpret_cast<const float4*>(kco + cell)) : z4;
        KC[i] = v ? __ldg(reinterpret_cast<const float4*>(kco + plane + cell)) : z4;
        KY[i] = v ? __ldg(reinterpret_cast<const float4*>(kco + 3 * plane + cell)) : z4;
        kgl[i] = le && gx < nx ? __ldg(Kg + (size_t)gx * ny + y0 - 1) : 0.f;
        kgr[i] = re && gx < nx ? __ldg(Kg + (size_t)gx * ny + y0 + STEP4_TY) : 0.f;
    }
    // the 4-cell slot this thread owns in the sums: row x0 + orow, lanes' chunk oln
    const int slot = w * 32 + lane, orow = slot / 32, oln = slot % 32;
    const bool owner = slot < R * 32 && x0 + orow < nx && y0 + 4 * oln < ny;
    float4 blk = z4;
    const int i0 = blockIdx.z * ADJ_BLOCK, i1 = min(batch, i0 + ADJ_BLOCK);
    for (int base = i0; base < i1; base += W) {
        const int inst = base + w;
        if (inst < i1) {                        // uniform over the warp
            // every load first
            const float* l1p = lam1 ? lam1 + inst * plane : nullptr;
            const float* hp = hprev ? hprev + inst * hbs : nullptr;
            const float* l2p = lam2 ? lam2 + inst * plane : nullptr;
            float4 L1[R + 2], H[R + 2], L2[R];
            float l1l[R], l1r[R], hl_[R], hr_[R];
#pragma unroll
            for (int i = 0; i < R + 2; ++i) {
                const int gx = x0 - 1 + i;
                const bool v = colv && gx >= 0 && gx < nx;
                const size_t cell = (size_t)gx * ny + gy;
                L1[i] = v && l1p ? __ldg(reinterpret_cast<const float4*>(l1p + cell)) : z4;
                H[i] = v && hp ? __ldg(reinterpret_cast<const float4*>(hp + cell)) : z4;
            }
#pragma unroll
            for (int i = 0; i < R; ++i) {
                const int gx = x0 + i;
                const bool v = colv && gx < nx;
                const size_t cell = (size_t)gx * ny + gy;
                L2[i] = v && l2p ? __ldg(reinterpret_cast<const float4*>(l2p + cell)) : z4;
                l1l[i] = l1r[i] = hl_[i] = hr_[i] = 0.f;
                if (edges) {                    // uniform: a chunk with a neighbour chunk
                    const size_t lc = (size_t)gx * ny + y0 - 1, rc = (size_t)gx * ny + y0 + STEP4_TY;
                    l1l[i] = le && gx < nx && l1p ? __ldg(l1p + lc) : 0.f;
                    l1r[i] = re && gx < nx && l1p ? __ldg(l1p + rc) : 0.f;
                    hl_[i] = le && gx < nx && hp ? __ldg(hp + lc) : 0.f;
                    hr_[i] = re && gx < nx && hp ? __ldg(hp + rc) : 0.f;
                }
            }
#pragma unroll
            for (int i = 0; i < R; ++i) {
                const int gx = x0 + i;
                if (gx >= nx) break;            // uniform over the warp
                const float4 GU = g4(KG[i], L1[i]), GC = g4(KG[i + 1], L1[i + 1]);
                const float4 GD = g4(KG[i + 2], L1[i + 2]);
                const float4 HU = H[i], HC = H[i + 1], HD = H[i + 2];
                float gl = __shfl_up_sync(0xffffffffu, GC.w, 1), gr = __shfl_down_sync(0xffffffffu, GC.x, 1);
                float hl = __shfl_up_sync(0xffffffffu, HC.w, 1), hr = __shfl_down_sync(0xffffffffu, HC.x, 1);
                if (lane == 0) { gl = fmul(kgl[i], l1l[i]); hl = hl_[i]; }
                if (lane == 31) { gr = fmul(kgr[i], l1r[i]); hr = hr_[i]; }
                if (!colv) continue;
                const float Gc[4] = {GC.x, GC.y, GC.z, GC.w}, Gu[4] = {GU.x, GU.y, GU.z, GU.w};
                const float Gd[4] = {GD.x, GD.y, GD.z, GD.w};
                const float Gl[4] = {gl, GC.x, GC.y, GC.z}, Gr[4] = {GC.y, GC.z, GC.w, gr};
                const float Hc[4] = {HC.x, HC.y, HC.z, HC.w}, Hu[4] = {HU.x, HU.y, HU.z, HU.w};
                const float Hd[4] = {HD.x, HD.y, HD.z, HD.w};
                const float Hl[4] = {hl, HC.x, HC.y, HC.z}, Hr[4] = {HC.y, HC.z, HC.w, hr};
                const float l1[4] = {L1[i + 1].x, L1[i + 1].y, L1[i + 1].z, L1[i + 1].w};
                const float l2[4] = {L2[i].x, L2[i].y, L2[i].z, L2[i].w};
                const float x1[4] = {X1[i].x, X1[i].y, X1[i].z, X1[i].w};
                const float kc[4] = {KC[i].x, KC[i].y, KC[i].z, KC[i].w};
                const float ky[4] = {KY[i].x, KY[i].y, KY[i].z, KY[i].w};
                const size_t cell = (size_t)gx * ny + gy;
                float lam[4], gt[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    // gradient arriving at h_t: first gy2 from step t+2, then gy1 from t+1
                    float lv = 0.f;
                    if (lam2) lv = fmul(ky[j], l2[j]);
                    if (lam1) {
                        const float lg = lap5<ORDER>(Gu[j], Gl[j], Gc[j], Gr[j], Gd[j], k.lap_w, k.lap_w4);
                        const float gy1 = fadd(fmul(k.dt2, lg), fmul(fmul(2.0f, l1[j]), x1[j]));
                        lv = lam2 ? fadd(lv, gy1) : gy1;
                    }
                    lam[j] = lv;
                }
                // probe seeds (descending chains) in their own block, entered
                // by the warps of tiles that hold taps only: inside the loop
                // above, their chains cost every warp ~20 % of its instructions
                if (taps) {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        for (int en = __ldg(e.probemap + cell + j); en >= 0; en = __ldg(e.probe_next + en)) {
                            size_t o = ((size_t)inst * e.steps + e.t) * e.n_probe + en;
                            float gv = __ldg(e.grad_out + o);
                            float sd = __ldg(e.probe_kind + en) ? fmul(gv, fmul(2.0f, __ldg(e.amp + o))) : gv;
                            lam[j] = fadd(lam[j], sd);
                        }
                    if (e.grad_x) {
#pragma unroll
                        for (int j = 0; j < 4; ++j)
                            for (int en = __ldg(e.srcmap + cell + j); en >= 0; en = __ldg(e.src_next + en))
                                if (__ldg(e.src_row + en) < 0) e.grad_x[(size_t)inst * e.steps + e.t] = lam[j];
                    }
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const float L = hp ? lap5<ORDER>(Hu[j], Hl[j], Hc[j], Hr[j], Hd[j], k.lap_w, k.lap_w4)
                                       : 0.0f;
                    gt[j] = fmul(fmul(x1[j], fmul(kc[j], L)), lam[j]);
                }
                *reinterpret_cast<float4*>(lam_out + inst * plane + cell) =
                    make_float4(lam[0], lam[1], lam[2], lam[3]);
                part[w][i * 32 + lane] = make_float4(gt[0], gt[1], gt[2], gt[3]);
            }
        }
        __syncthreads();
        if (owner) {
            const int n = min(W, i1 - base);
            for (int q = 0; q < n; ++q) {       // instance order
                const float4 v = part[q][slot];
                blk = make_float4(fadd(blk.x, v.x), fadd(blk.y, v.y), fadd(blk.z, v.z), fadd(blk.w, v.w));
            }
        }
        __syncthreads();
    }
    if (!owner) return;
    const size_t cell = (size_t)(x0 + orow) * ny + y0 + 4 * oln;
    if (e.G) {          // one instance: blk holds fadd(0, term), as the reduction's
        float4* gp = reinterpret_cast<float4*>(e.G + cell);
        float4 acc = blk;
        if (!e.first) {
            const float4 o = *gp;
            acc = make_float4(fadd(o.x, acc.x), fadd(o.y, acc.y), fadd(o.z, acc.z), fadd(o.w, acc.w));
        }
        *gp = acc;
    } else if (gsum) {
        *reinterpret_cast<float4*>(gsum + blockIdx.z * plane + cell) = blk;
    }
}

// Second stage of the batch reduction after seq_adj_step4r_kernel: G (+)= the
// block sums in block order (seq_adj_reduce_kernel's acc).
__global__ void seq_adj_sum_blocks_kernel(int nb, size_t plane, const float* __restrict__ gsum,
                                          float* __restrict__ G, int first) {
    const size_t cell = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= plane) return;
    float acc = 0.f;
    for (int j0 = 0; j0 < nb; j0 += 64) {       // 64 loads in flight, then the sums in order
        float v[64];
#pragma unroll
        for (int u = 0; u < 64; ++u) v[u] = j0 + u < nb ? __ldg(gsum + (size_t)(j0 + u) * plane + cell) : 0.f;
#pragma unroll
        for (int u = 0; u < 64; ++u)
            if (j0 + u < nb) acc = j0 + u == 0 ? v[u] : fadd(acc, v[u]);
    }
    G[cell] = first ? acc : fadd(G[cell], acc);
}

// Phase 2: G_c += chunked batch sum of gc (wavetorch autograd: sum-to-shape of
// each step's [batch,nx,ny] grad_c, then accumulation over steps).
__global__ void seq_adj_reduce_kernel(int batch, size_t plane, const float* __restrict__ gc,
                                      float* __restrict__ G, int first) {
    size_t cell = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= plane) return;
    float acc = 0.f, blk = 0.f;
    for (int i = 0; i < batch; ++i) {
        blk = fadd(blk, __ldg(gc + (size_t)i * plane + cell));
        if ((i & 15) == 15 || i == batch - 1) {
            acc = i < 16 ? blk : fadd(acc, blk);
            blk = 0.f;
        }
    }
    G[cell] = first ? acc : fadd(G[cell], acc);
}

// The same sums with the blocks of 16 instances in parallel: thread (x, y)
// forms the block sums j = y, y + blockDim.y, ... of cell x of its 32 cells
// (warps read 32 consecutive cells of one instance), then row 0 adds the
// blocks in order -- seq_adj_reduce_kernel's arithmetic, operand for operand.
constexpr int RED_CELLS = 32;
__global__ void seq_adj_reduce_blocks_kernel(int batch, size_t plane, const float* __restrict__ gc,
                                             float* __restrict__ G, int first) {
    extern __shared__ float part[];   // [blocks of 16][RED_CELLS]
    const int nb = (batch + 15) / 16;
    const size_t cell = (size_t)blockIdx.x * RED_CELLS + threadIdx.x;
    for (int j = threadIdx.y; j < nb; j += blockDim.y) {
        float blk = 0.f;
        if (cell < plane) {
            const int i1 = min(batch, 16 * j + 16);
            for (int i = 16 * j; i < i1; ++i) blk = fadd(blk, __ldg(gc + (size_t)i * plane + cell));
        }
        part[j * RED_CELLS + threadIdx.x] = blk;
    }
    __syncthreads();
    if (threadIdx.y != 0 || cell >= plane) return;
    float acc = part[threadIdx.x];
    for (int j = 1; j < nb; ++j) acc = fadd(acc, part[j * RED_CELLS + threadIdx.x]);
    G[cell] = first ? acc : fadd(G[cell], acc);
}

__global__ void fill_zero_kernel(float* p, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = 0.f;
}

}  // namespace wt

// ---------------------------------------------------------------------------
// Launch helpers used by api.cu
// The vector kernels need rows of a multiple of 4 cells and 16-byte aligned
// fields and strides.
static bool vec4_ok(int ny, std::initializer_list<const void*> ptrs,
                    std::initializer_list<size_t> strides) {
    if (ny % 4) return false;
    for (const void* p : ptrs)
        if (p && (reinterpret_cast<uintptr_t>(p) & 15)) return false;
    for (size_t s : strides)
        if (s % 4) return false;
    return true;
}

int wt_launch_step_fwd(const StepScalars& k, int batch, int nx, int ny, int coef_batched,
                       const float* b, const float* c, const float* y1, size_t bs1,
                       const float* y2, size_t bs2, float* y, size_t bs,
                       const wt::SeqEpilogue* epi, cudaStream_t st, const float* fco) {
    // (grid rows: one per CTA of STEP4R_WARPS row groups, at most 65535)
    constexpr int RPC = wt::STEP4R_ROWS * wt::STEP4R_WARPS;
    if (fco && !coef_batched && (size_t)batch * nx * ny >= wt::STREAM_MIN_CELLS &&
        (nx + RPC - 1) / RPC <= 65535 &&
        vec4_ok(ny, {fco, y1, y2, y}, {bs1, bs2, bs, (size_t)nx * ny})) {
        const int groups = (nx + wt::STEP4R_ROWS - 1) / wt::STEP4R_ROWS;
        dim3 blk(32, wt::STEP4R_WARPS);
        dim3 grd((ny + wt::STEP4_TY - 1) / wt::STEP4_TY, (groups + wt::STEP4R_WARPS - 1) / wt::STEP4R_WARPS,
                 batch);
        wt::SeqEpilogue e{};
        if (epi) e = *epi;
        const bool ep = epi != nullptr;
        if ((k.lap_order & 1) == WT_LAP_SEQ) {
            if (ep) wt::step_fwd4r_kernel<WT_LAP_SEQ, true><<<grd, blk, 0, st>>>(k, nx, ny, fco, y1, bs1, y2, bs2, y, bs, e);
            else    wt::step_fwd4r_kernel<WT_LAP_SEQ, false><<<grd, blk, 0, st>>>(k, nx, ny, fco, y1, bs1, y2, bs2, y, bs, e);
        } else {
            if (ep) wt::step_fwd4r_kernel<WT_LAP_PAIRED, true><<<grd, blk, 0, st>>>(k, nx, ny, fco, y1, bs1, y2, bs2, y, bs, e);
            else    wt::step_fwd4r_kernel<WT_LAP_PAIRED, false><<<grd, blk, 0, st>>>(k, nx, ny, fco, y1, bs1, y2, bs2, y, bs, e);
        }
        wt_count_launches(1);
        return wt_cuda_status(cudaGetLastError());
    }
    if (vec4_ok(ny, {b, c, fco, y1, y2, y}, {bs1, bs2, bs, (size_t)nx * ny})) {
        dim3 blk(32, wt::STEP4_TX);
        dim3 grd((ny + wt::STEP4_TY - 1) / wt::STEP4_TY, (nx + wt::STEP4_TX - 1) / wt::STEP4_TX, batch);
        wt::SeqEpilogue e{};
        if (epi) e = *epi;
        const bool ep = epi != nullptr;
        if ((k.lap_order & 1) == WT_LAP_SEQ) {
            if (ep) wt::step_fwd4_kernel<WT_LAP_SEQ, true><<<grd, blk, 0, st>>>(k, nx, ny, coef_batched, b, c, fco, y1, bs1, y2, bs2, y, bs, e);
            else    wt::step_fwd4_kernel<WT_LAP_SEQ, false><<<grd, blk, 0, st>>>(k, nx, ny, coef_batched, b, c, fco, y1, bs1, y2, bs2, y, bs, e);
        } else {
            if (ep) wt::step_fwd4_kernel<WT_LAP_PAIRED, true><<<grd, blk, 0, st>>>(k, nx, ny, coef_batched, b, c, fco, y1, bs1, y2, bs2, y, bs, e);
            else    wt::step_fwd4_kernel<WT_LAP_PAIRED, false><<<grd, blk, 0, st>>>(k, nx, ny, coef_batched, b, c, fco, y1, bs1, y2, bs2, y, bs, e);
        }
        wt_count_launches(1);
        return wt_cuda_status(cudaGetLastError());
    }
    dim3 blk(wt::TY, wt::TX);
    dim3 grd((ny + wt::TY - 1) / wt::TY, (nx + wt::TX - 1) / wt::TX, batch);
    if (epi) {
        const wt::SeqEpilogue& e = *epi;
        if ((k.lap_order & 1) == WT_LAP_SEQ)
            wt::step_fwd_kernel<WT_LAP_SEQ, true><<<grd, blk, 0, st>>>(k, nx, ny, coef_batched, b, c, y1, bs1, y2, bs2, y, bs, e);
        else
            wt::step_fwd_kernel<WT_LAP_PAIRED, true><<<grd, blk, 0, st>>>(k, nx, ny, coef_batched, b, c, y1, bs1, y2, bs2, y, bs, e);
    } else {
        wt::SeqEpilogue e{};
        if ((k.lap_order & 1) == WT_LAP_SEQ)
            wt::step_fwd_kernel<WT_LAP_SEQ, false><<<grd, blk, 0, st>>>(k, nx, ny, coef_batched, b, c, y1, bs1, y2, bs2, y, bs, e);
        else
            wt::step_fwd_kernel<WT_LAP_PAIRED, false><<<grd, blk, 0, st>>>(k, nx, ny, coef_batched, b, c, y1, bs1, y2, bs2, y, bs, e);
    }
    wt_count_launches(1);
    return wt_cuda_status(cudaGetLastError());
}

int wt_launch_step_bwd(const StepScalars& k, int batch, int nx, int ny, int coef_batched,
                       const float* b, const float* c, const float* y1, const float* y2,
                       const float* g, float* gb, float* gcp, float* gy1, float* gy2,
                       cudaStream_t st) {
    dim3 blk(wt::TY, wt::TX);
    dim3 grd((ny + wt::TY - 1) / wt::TY, (nx + wt::TX - 1) / wt::TX, 1);
    if ((k.lap_order & 1) == WT_LAP_SEQ)
        wt::step_bwd_kernel<WT_LAP_SEQ><<<grd, blk, 0, st>>>(k, batch, nx, ny, coef_batched, b, c, y1, y2, g, gb, gcp, gy1, gy2);
    else
        wt::step_bwd_kernel<WT_LAP_PAIRED><<<grd, blk, 0, st>>>(k, batch, nx, ny, coef_batched, b, c, y1, y2, g, gb, gcp, gy1, gy2);
    wt_count_launches(1);
    return wt_cuda_status(cudaGetLastError());
}

int wt_launch_fwd_coef(const StepScalars& k, size_t plane, const float* b, const float* c,
                       float* fco, cudaStream_t st) {
    wt::fwd_coef_kernel<<<(unsigned)((plane + 255) / 256), 256, 0, st>>>(k, plane, b, c, fco);
    wt_count_launches(1);
    return wt_cuda_status(cudaGetLastError());
}
int wt_launch_adj_coef(const StepScalars& k, size_t plane, const float* b, const float* c,
                       float* kco, cudaStream_t st) {
    wt::adj_coef_kernel<<<(unsigned)((plane + 255) / 256), 256, 0, st>>>(k, plane, b, c, kco);
    wt_count_launches(1);
    return wt_cuda_status(cudaGetLastError());
}

int wt_launch_seq_adj_step(const StepScalars& k, int batch, int nx, int ny, const float* b,
                           const float* c, const float* kco, const float* lam1, const float* lam2,
                           const float* hprev, size_t hbs, float* lam_out, float* gc, float* G,
                           int first, const wt::AdjEpilogue& e, cudaStream_t st) {
    const size_t plane = (size_t)nx * ny;
    if (kco && vec4_ok(ny, {kco, lam1, lam2, hprev, lam_out, gc, e.G}, {hbs, plane})) {
        // row-streaming with block sums (grid rows: one per row, at most 65535)
        if ((size_t)batch * plane >= wt::STREAM_MIN_CELLS && nx <= 65535 * wt::ADJ4R_ROWS) {
            constexpr int R = wt::ADJ4R_ROWS;
            const int nb = (batch + wt::ADJ_BLOCK - 1) / wt::ADJ_BLOCK;
            dim3 grd((ny + wt::STEP4_TY - 1) / wt::STEP4_TY, (nx + R - 1) / R, nb);
            dim3 blk(32, 4);
            if ((k.lap_order & 1) == WT_LAP_SEQ)
                wt::seq_adj_step4r_kernel<WT_LAP_SEQ, R, 4, 5><<<grd, blk, 0, st>>>(k, batch, nx, ny, kco, lam1, lam2, hprev, hbs, lam_out, gc, e);
            else
                wt::seq_adj_step4r_kernel<WT_LAP_PAIRED, R, 4, 5><<<grd, blk, 0, st>>>(k, batch, nx, ny, kco, lam1, lam2, hprev, hbs, lam_out, gc, e);
            wt_count_launches(1);
            cudaError_t ce = cudaGetLastError();
            if (ce != cudaSuccess || e.G || !G) return wt_cuda_status(ce);
            wt::seq_adj_sum_blocks_kernel<<<(unsigned)((plane + 255) / 256), 256, 0, st>>>(nb, plane, gc, G, first);
            wt_count_launches(1);
            return wt_cuda_status(cudaGetLastError());
        }
        dim3 blk(32, wt::STEP4_TX);           // tiles, one term plane per instance
        dim3 grd((ny + wt::STEP4_TY - 1) / wt::STEP4_TY, (nx + wt::STEP4_TX - 1) / wt::STEP4_TX, batch);
        if ((k.lap_order & 1) == WT_LAP_SEQ)
            wt::seq_adj_step4_kernel<WT_LAP_SEQ><<<grd, blk, 0, st>>>(k, nx, ny, kco, lam1, lam2, hprev, hbs, lam_out, gc, e);
        else
            wt::seq_adj_step4_kernel<WT_LAP_PAIRED><<<grd, blk, 0, st>>>(k, nx, ny, kco, lam1, lam2, hprev, hbs, lam_out, gc, e);
        wt_count_launches(1);
        cudaError_t ce = cudaGetLastError();
        if (ce != cudaSuccess || e.G || !G) return wt_cuda_status(ce);
        return wt_launch_seq_adj_reduce(batch, plane, gc, G, first, st);
    }
    dim3 blk(wt::TY, wt::TX);
    dim3 grd((ny + wt::TY - 1) / wt::TY, (nx + wt::TX - 1) / wt::TX, batch);
    if ((k.lap_order & 1) == WT_LAP_SEQ)
        wt::seq_adj_step_kernel<WT_LAP_SEQ><<<grd, blk, 0, st>>>(k, nx, ny, b, c, lam1, lam2, hprev, hbs, lam_out, gc, e);
    else
        wt::seq_adj_step_kernel<WT_LAP_PAIRED><<<grd, blk, 0, st>>>(k, nx, ny, b, c, lam1, lam2, hprev, hbs, lam_out, gc, e);
    wt_count_launches(1);
    cudaError_t ce = cudaGetLastError();
    if (ce != cudaSuccess || e.G || !G) return wt_cuda_status(ce);
    return wt_launch_seq_adj_reduce(batch, plane, gc, G, first, st);
}

int wt_launch_seq_adj_reduce(int batch, size_t plane, const float* gc, float* G, int first,
                             cudaStream_t st) {
    const int nb = (batch + 15) / 16;
    const size_t smem = (size_t)nb * wt::RED_CELLS * sizeof(float);
    if (batch > 16 && smem <= 48 * 1024) {   // blocks of 16 in parallel
        dim3 blk(wt::RED_CELLS, 8);
        wt::seq_adj_reduce_blocks_kernel<<<(unsigned)((plane + wt::RED_CELLS - 1) / wt::RED_CELLS),
                                           blk, smem, st>>>(batch, plane, gc, G, first);
        wt_count_launches(1);
        return wt_cuda_status(cudaGetLastError());
    }
    int thr = 256;
    wt::seq_adj_reduce_kernel<<<(unsigned)((plane + thr - 1) / thr), thr, 0, st>>>(batch, plane, gc, G, first);
    wt_count_launches(1);
    return wt_cuda_status(cudaGetLastError());
}

int wt_launch_fill_zero(float* p, size_t n, cudaStream_t st) {
    if (n == 0) return WT_OK;
    int thr = 256;
    wt::fill_zero_kernel<<<(unsigned)((n + thr - 1) / thr), thr, 0, st>>>(p, n);
    wt_count_launches(1);
    return wt_cuda_status(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Lookup tables of the sequence entry points, written without a host copy:
// the -1 fill of the per-cell maps, then the entries themselves, carried in
// the kernel's parameters (so the host never waits for a staging copy).
namespace wt {
__global__ void fill_int_kernel(int* __restrict__ p, size_t n, int v) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}
__global__ void scatter_ints_kernel(int* __restrict__ base, IntScatter s) {
    for (int i = threadIdx.x; i < s.n; i += blockDim.x) base[s.idx[i]] = s.val[i];
}
}  // namespace wt

int wt_launch_fill_int(int* p, size_t n, int v, cudaStream_t st) {
    if (n == 0) return WT_OK;
    int thr = 256;
    wt::fill_int_kernel<<<(unsigned)((n + thr - 1) / thr), thr, 0, st>>>(p, n, v);
    wt_count_launches(1);
    return wt_cuda_status(cudaGetLastError());
}

int wt_launch_scatter_ints(int* base, const wt::IntScatter& s, cudaStream_t st) {
    if (s.n <= 0) return WT_OK;
    wt::scatter_ints_kernel<<<1, 256, 0, st>>>(base, s);
    wt_count_launches(1);
    return wt_cuda_status(cudaGetLastError());
}
