// Fused persistent sequence kernels: the whole time loop of WaveRNN.forward
// (wavetorch/rnn.py:50-70) and the whole adjoint sweep of its T TimeStep
// nodes (wavetorch/cell.py:26-44) each run as ONE launch.
//
// Decomposition.  One thread-block cluster of C CTAs owns one instance of the
// batch.  CTA k of the cluster owns rows [k*R, k*R + R) of the nx x ny grid
// (rows past nx are padding cells whose coefficients are zero, so they stay
// exactly 0).  Thread (col, strip) owns the M vertically consecutive cells
// (strip*M .. strip*M+M-1, col) of its CTA and keeps their state (fields,
// coefficients, adjoint accumulators) in registers.
//
// Exchange.  Each step every thread writes its M new values into a
// column-major shared-memory tile  F[col+1][OFF + row]  (zero columns at
// y = -1 and y = ny), double buffered, with one __syncthreads per step.  The
// CTA's first and last rows also go to the neighbouring CTAs as tagged
// 64-bit words (see the exchange section below); only the thread that needs
// a neighbour's value waits for it, so nothing on the cluster path is a
// barrier or a fence, and global stores never stall the exchange.
//
// Waits are bounded (~2 s).  A wait that gives up records WT_DEVERR_TIMEOUT
// in the status word, the CTA leaves its loop within 32 steps, its
// neighbours' waits then give up too, and the cluster meets at one final
// barrier before exiting.
//
// Adjoint.  The forward stores the pair (h_{t-1}, h_{t-2}) every `seg` steps.
// The adjoint walks the segments backwards: it reloads the checkpoint,
// recomputes the segment's forward steps to rebuild Lap(h_{t-1}) for each of
// its steps (the "stash"), then runs the segment's adjoint steps from the
// stash.  Adjoint state per cell (pending grad_y1/grad_y2 terms and the
// running dL/dc sum of this instance) stays in registers across segments;
// the coefficients of each phase are re-formed from b and c when the phase
// starts (once per segment), so only one phase's coefficients occupy
// registers at a time.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <type_traits>

#include "internal.cuh"

namespace wt {

constexpr int OFF = 4;       // first own row in a tile column (16-byte aligned)
constexpr int SRCMAX = 4;    // source entries one thread may own
constexpr int PRBMAX = 4;    // probe entries one thread may own
constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;   // bounded halo waits (2 s)

// load M consecutive floats from a 16-byte aligned (M%4==0) shared address
template <int M>
WT_DEV void lds_col(float (&d)[M], const float* p) {
    if constexpr (M % 4 == 0) {
#pragma unroll
        for (int i = 0; i < M; i += 4) {
            float4 v = *reinterpret_cast<const float4*>(p + i);
            d[i] = v.x; d[i + 1] = v.y; d[i + 2] = v.z; d[i + 3] = v.w;
        }
    } else if constexpr (M % 2 == 0) {
#pragma unroll
        for (int i = 0; i < M; i += 2) {
            float2 v = *reinterpret_cast<const float2*>(p + i);
            d[i] = v.x; d[i + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < M; ++i) d[i] = p[i];
    }
}
template <int M>
WT_DEV void sts_col(float* p, const float (&s)[M]) {
    if constexpr (M % 4 == 0) {
#pragma unroll
        for (int i = 0; i < M; i += 4)
            *reinterpret_cast<float4*>(p + i) = make_float4(s[i], s[i + 1], s[i + 2], s[i + 3]);
    } else if constexpr (M % 2 == 0) {
#pragma unroll
        for (int i = 0; i < M; i += 2) *reinterpret_cast<float2*>(p + i) = make_float2(s[i], s[i + 1]);
    } else {
#pragma unroll
        for (int i = 0; i < M; ++i) p[i] = s[i];
    }
}

// Chunk-major block of a CTA's M values per thread: chunk j (V = 4, 2 or 1
// consecutive values, the widest vector M allows) of thread `tid` sits at
// (j * NT + tid) * V.  A warp's access to one chunk is one contiguous run
// (coalesced in global memory, conflict-free in shared memory).
template <int M>
constexpr int chunk_width() { return M % 4 == 0 ? 4 : M % 2 == 0 ? 2 : 1; }

// Chunk-major store from the thread's own chunk-0 address p (stride: floats
// between chunks).
template <int M>
WT_DEV void st_chunks_at(float* p, int stride, const float (&s)[M]) {
    constexpr int V = chunk_width<M>();
#pragma unroll
    for (int j = 0; j < M / V; ++j) {
        float* q = p + j * stride;
        if constexpr (V == 4)
            *reinterpret_cast<float4*>(q) = make_float4(s[4 * j], s[4 * j + 1], s[4 * j + 2], s[4 * j + 3]);
        else if constexpr (V == 2)
            *reinterpret_cast<float2*>(q) = make_float2(s[2 * j], s[2 * j + 1]);
        else
            *q = s[j];
    }
}
template <int M>
WT_DEV void ld_chunks_at(float (&d)[M], const float* p, int stride) {
    constexpr int V = chunk_width<M>();
#pragma unroll
    for (int j = 0; j < M / V; ++j) {
        const float* q = p + j * stride;
        if constexpr (V == 4) {
            float4 v = *reinterpret_cast<const float4*>(q);
            d[4 * j] = v.x; d[4 * j + 1] = v.y; d[4 * j + 2] = v.z; d[4 * j + 3] = v.w;
        } else if constexpr (V == 2) {
            float2 v = *reinterpret_cast<const float2*>(q);
            d[2 * j] = v.x; d[2 * j + 1] = v.y;
        } else {
            d[j] = *q;
        }
    }
}
template <int M>
WT_DEV void ld_chunks(float (&d)[M], const float* base, int NT, int tid) {
    constexpr int V = chunk_width<M>();
#pragma unroll
    for (int j = 0; j < M / V; ++j) {
        const float* p = base + ((size_t)j * NT + tid) * V;
        if constexpr (V == 4) {
            float4 v = *reinterpret_cast<const float4*>(p);
            d[4 * j] = v.x; d[4 * j + 1] = v.y; d[4 * j + 2] = v.z; d[4 * j + 3] = v.w;
        } else if constexpr (V == 2) {
            float2 v = *reinterpret_cast<const float2*>(p);
            d[2 * j] = v.x; d[2 * j + 1] = v.y;
        } else {
            d[j] = *p;
        }
    }
}

// Thread geometry shared by both kernels.
struct Geo {
    int inst, cta, col, strip, xl0, gx0, S;
    bool colv;          // column inside the grid
    bool has_up, has_dn;
};

WT_DEV Geo make_geo(const FusedParams& P, int M) {
    Geo g;
    g.cta = (int)cluster_ctarank();
    g.inst = blockIdx.x / P.C;
    g.col = threadIdx.x % P.NCP;
    g.strip = threadIdx.x / P.NCP;
    g.xl0 = g.strip * M;
    g.gx0 = g.cta * P.R + g.xl0;
    g.S = P.R / M;
    g.colv = g.col < P.ny;
    g.has_up = g.cta > 0;
    g.has_dn = g.cta + 1 < P.C;
    return g;
}

// ---- neighbour exchange ----------------------------------------------------
// Inside a CTA the strips exchange through a double-buffered column-major
// tile (one __syncthreads per exchange).  Between the CTAs of a cluster only
// the boundary rows travel: each value goes as one 64-bit word {float bits,
// tag = exchange index + 1} stored with st.relaxed.cluster into the
// receiving CTA's halo array [2][NCP] (parity of the exchange index), and
// the single thread that needs it spins on that word until the tag matches
// (an aligned 8-byte store is single-copy atomic, so the value is valid
// whenever the tag is).  No barrier, fence or mbarrier is on this path.
//
// Double buffering is enough: a neighbour writes parity p for exchange k+2
// only after it received this CTA's exchange k+1 value, which this CTA's
// same thread sent after reading its exchange-k word.
struct Xchg {
    float* tiles;           // slot 0 (slots are `tile` floats apart)
    int tile;               // floats per slot
    unsigned long long* hup;    // [2][NCP] words from the up neighbour (its last row)
    unsigned long long* hdn;    // [2][NCP] words from the down neighbour (its first row)
    uint32_t up_hdn;        // shared::cluster address of the up neighbour's hdn
    uint32_t dn_hup;        // shared::cluster address of the down neighbour's hup
    int NCP;
    int* abort;             // CTA-wide abort flag (shared)
};

// smem layout: [2 tile slots][hup 2*NCP words][hdn 2*NCP words] (+ callers' areas)
WT_DEV void xchg_setup(Xchg& X, const FusedParams& P, const Geo& g, float* tiles, int tile,
                       int* abort) {
    X.tiles = tiles;
    X.tile = tile;
    X.NCP = P.NCP;
    X.hup = reinterpret_cast<unsigned long long*>(tiles + 2 * tile);
    X.hdn = X.hup + 2 * P.NCP;
    X.abort = abort;
    for (int i = threadIdx.x; i < 4 * P.NCP; i += blockDim.x) X.hup[i] = 0ull;   // tag 0: nothing yet
    X.up_hdn = g.has_up ? map_shared_rank(X.hdn, g.cta - 1) : 0u;
    X.dn_hup = g.has_dn ? map_shared_rank(X.hup, g.cta + 1) : 0u;
    if (threadIdx.x == 0) *abort = 0;
}

// Words (bytes) of the exchange area that follows the two tile slots.
constexpr int xchg_words(int NCP) { return 4 * NCP; }

// Send the CTA's first / last row values of exchange k (this thread's cell
// 0 / M-1 when its strip is a CTA boundary strip).
WT_DEV void send_halo(const Geo& g, const Xchg& X, int k, float first, float last) {
    const unsigned long long tag = (unsigned long long)(uint32_t)(k + 1) << 32;
    const uint32_t off = 8u * (uint32_t)((k & 1) * X.NCP + g.col);
    if (g.strip == 0 && g.has_up) st_cluster_u64(X.up_hdn + off, tag | __float_as_uint(first));
    if (g.strip == g.S - 1 && g.has_dn) st_cluster_u64(X.dn_hup + off, tag | __float_as_uint(last));
}

// Wait (bounded) for exchange k's word at w and return its value.
WT_DEV float recv_word(const FusedParams& P, const Xchg& X, const unsigned long long* w, int k) {
    const uint32_t a = smem_addr(w);
    const uint32_t tag = (uint32_t)(k + 1);
    unsigned long long v = ld_cluster_u64(a);
    if ((uint32_t)(v >> 32) != tag) {
        const uint64_t t0 = global_ns();
        for (uint32_t it = 1;; ++it) {
            v = ld_cluster_u64(a);
            if ((uint32_t)(v >> 32) == tag) break;
            if ((it & 1023u) == 0) {
                if (*(volatile int*)X.abort) return 0.f;   // another wait gave up
                if (global_ns() - t0 > WAIT_LIMIT_NS) {
                    atomicExch(P.err, WT_DEVERR_TIMEOUT);
                    *(volatile int*)X.abort = 1;
                    return 0.f;
                }
            }
        }
    }
    return __uint_as_float((uint32_t)v);
}

// Per-thread addresses of the forward's step path, formed once before the
// loop (recomputing them every step cost a quarter of the step's
// instructions): the thread's column in tile slot 0 (slot 1 is `tile` floats
// further), and for the CTA's boundary strips the halo words it reads and
// the neighbour words it writes, for exchange parity 0 (parity 1 is `pstride`
// bytes further).  0 where the thread has no such word.
struct Lane {
    float* col0;
    int tile;
    uint32_t rup, rdn, sup, sdn, pstride;
};

WT_DEV Lane make_lane(const FusedParams& P, const Geo& g, const Xchg& X) {
    Lane l;
    l.col0 = X.tiles + (g.col + 1) * P.LD + OFF + g.xl0;
    l.tile = X.tile;
    const bool top = g.strip == 0 && g.has_up, bot = g.strip == g.S - 1 && g.has_dn;
    l.rup = top ? smem_addr(X.hup + g.col) : 0u;
    l.rdn = bot ? smem_addr(X.hdn + g.col) : 0u;
    // (the missing-arrival test hook: a muted CTA keeps its rows to itself)
    const bool mute = P.mute_cta1 == g.cta + 1 && g.inst == 0;
    l.sup = top && !mute ? X.up_hdn + 8u * (uint32_t)g.col : 0u;
    l.sdn = bot && !mute ? X.dn_hup + 8u * (uint32_t)g.col : 0u;
    l.pstride = 8u * (uint32_t)X.NCP;
    return l;
}

// Wait (bounded) for exchange k's word at shared address a and return its value.
WT_DEV float recv_at(const FusedParams& P, const Xchg& X, uint32_t a, int k) {
    const uint32_t tag = (uint32_t)(k + 1);
    unsigned long long v = ld_cluster_u64(a);
    if ((uint32_t)(v >> 32) != tag) {
        const uint64_t t0 = global_ns();
        for (uint32_t it = 1;; ++it) {
            v = ld_cluster_u64(a);
            if ((uint32_t)(v >> 32) == tag) break;
            if ((it & 1023u) == 0) {
                if (*(volatile int*)X.abort) return 0.f;   // another wait gave up
                if (global_ns() - t0 > WAIT_LIMIT_NS) {
                    atomicExch(P.err, WT_DEVERR_TIMEOUT);
                    *(volatile int*)X.abort = 1;
                    return 0.f;
                }
            }
        }
    }
    return __uint_as_float((uint32_t)v);
}

template <int M>
WT_DEV void store_column(const FusedParams& P, const Geo& g, const Xchg& X, int s,
                         const float (&v)[M]) {
    sts_col<M>(X.tiles + s * X.tile + (g.col + 1) * P.LD + OFF + g.xl0, v);
}

// Publish the thread's M values as exchange k: halo words, then own column
// into tile slot s.
template <int M>
WT_DEV void publish(const FusedParams& P, const Geo& g, const Xchg& X, int s, int k,
                    const float (&v)[M]) {
    if (!g.colv) return;
    send_halo(g, X, k, v[0], v[M - 1]);
    store_column<M>(P, g, X, s, v);
}

// The thread's column of slot `slot`: left/right neighbour columns of its M
// cells, and the two cells just above and below its strip (from the tile, or
// for a CTA boundary strip the neighbour's word of exchange k; k < 0: none,
// the tile's zero halo rows stand for the field h_{-1} = 0).
template <int M>
struct Column {
    float lf[M], rt[M];
    float up, dn;
};
template <int M>
WT_DEV void load_sides(Column<M>& c, const FusedParams& P, const Geo& g, const Xchg& X, int slot,
                       int k) {
    const float* colp = X.tiles + slot * X.tile + (g.col + 1) * P.LD + OFF + g.xl0;
    lds_col<M>(c.lf, colp - P.LD);
    lds_col<M>(c.rt, colp + P.LD);
    c.up = colp[-1];
    c.dn = colp[M];
    if (k >= 0) {
        if (g.strip == 0 && g.has_up) c.up = recv_word(P, X, X.hup + (k & 1) * X.NCP + g.col, k);
        if (g.strip == g.S - 1 && g.has_dn) c.dn = recv_word(P, X, X.hdn + (k & 1) * X.NCP + g.col, k);
    }
}

// Laplacian of cell i (0 < i < M-1 use registers for up/down).
template <int M, int ORDER>
WT_DEV float lap_cell(const FusedParams& P, const Column<M>& c, const float (&ctr)[M], int i) {
    float u = i == 0 ? c.up : ctr[i - 1];
    float d = i == M - 1 ? c.dn : ctr[i + 1];
    return lap5<ORDER>(u, c.lf[i], ctr[i], c.rt[i], d, P.k.lap_w, P.k.lap_w4);
}

WT_DEV void zero_smem(float* s, int n) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) s[i] = 0.f;
}

// Per-thread source list (table order) and probe list (descending order),
// packed into scalar words so they stay in registers:
//   source e: (input row << 5) | cell index i      probe e: (column << 6) | (kind << 5) | i
struct Taps {
    int ns, np;
    bool src_edge;        // a source sits on a cell this thread sends as a halo
    // some thread of the warp holds a source / a probe (warp-uniform), tested
    // before the per-step tap work.  On their own these guards did not change
    // the compiled step (same instruction count); what lets warps without
    // probes skip the seeds is the loop on the thread's own count in
    // seed_and_read.
    bool wsrc, wprb;
    int s0, s1, s2, s3;
    int p0, p1, p2, p3;
    WT_DEV int s(int e) const { return e == 0 ? s0 : e == 1 ? s1 : e == 2 ? s2 : s3; }
    WT_DEV int p(int e) const { return e == 0 ? p0 : e == 1 ? p1 : e == 2 ? p2 : p3; }
    WT_DEV int src_i(int e) const { return s(e) & 31; }
    WT_DEV int src_row(int e) const { return s(e) >> 5; }
    WT_DEV int prb_i(int e) const { return p(e) & 31; }
    WT_DEV int prb_col(int e) const { return p(e) >> 6; }
    WT_DEV bool prb_intensity(int e) const { return (p(e) & 32) != 0; }
};

template <int M>
WT_DEV void build_taps(const FusedParams& P, const Geo& g, Taps& tp) {
    int ns = 0, np = 0;
    int s0 = 0, s1 = 0, s2 = 0, s3 = 0, p0 = 0, p1 = 0, p2 = 0, p3 = 0;
    if (g.colv) {
        for (int e = 0; e < P.n_src; ++e) {
            int cell = __ldg(P.src_cell + e);
            int cx = cell / P.ny, cy = cell - cx * P.ny;
            int i = cx - g.gx0;
            if (cy == g.col && i >= 0 && i < M) {
                int row = __ldg(P.src_row + e);
                int v = ((row < 0 ? g.inst : row) << 5) | i;
                if (ns == 0) s0 = v; else if (ns == 1) s1 = v; else if (ns == 2) s2 = v;
                else if (ns == 3) s3 = v; else atomicExch(P.err, WT_DEVERR_BOUNDS);
                ++ns;
            }
        }
        for (int e = 0; e < P.n_prb; ++e) {
            int cell = __ldg(P.prb_cell + e);
            int cx = cell / P.ny, cy = cell - cx * P.ny;
            int i = cx - g.gx0;
            if (cy == g.col && i >= 0 && i < M) {
                int v = (__ldg(P.prb_col + e) << 6) | (__ldg(P.prb_kind + e) << 5) | i;
                if (np == 0) p0 = v; else if (np == 1) p1 = v; else if (np == 2) p2 = v;
                else if (np == 3) p3 = v; else atomicExch(P.err, WT_DEVERR_BOUNDS);
                ++np;
            }
        }
    }
    tp.ns = min(ns, SRCMAX); tp.np = min(np, PRBMAX);
    tp.s0 = s0; tp.s1 = s1; tp.s2 = s2; tp.s3 = s3;
    tp.p0 = p0; tp.p1 = p1; tp.p2 = p2; tp.p3 = p3;
    tp.src_edge = false;
#pragma unroll
    for (int e = 0; e < SRCMAX; ++e) {
        const int i = tp.src_i(e);
        if (e < tp.ns && ((i == 0 && g.strip == 0 && g.has_up) ||
                          (i == M - 1 && g.strip == g.S - 1 && g.has_dn)))
            tp.src_edge = true;
    }
    tp.wsrc = __any_sync(0xffffffffu, tp.ns > 0);   // every thread of the CTA gets here
    tp.wprb = __any_sync(0xffffffffu, tp.np > 0);
}

// Per-cell coefficients of one phase, re-formed from b and c.
template <int M>
WT_DEV void load_fwd_coef(const FusedParams& P, const Geo& g, float (&A)[M], float (&Bc)[M],
                          float (&C2)[M]) {
#pragma unroll
    for (int i = 0; i < M; ++i) {
        A[i] = Bc[i] = C2[i] = 0.f;
        int gx = g.gx0 + i;
        if (g.colv && gx < P.nx) {
            size_t cell = P.coef_stride * g.inst + (size_t)gx * P.ny + g.col;
            FwdCoef f = fwd_coef(__ldg(P.b + cell), __ldg(P.c + cell), P.k);
            A[i] = f.A; Bc[i] = f.Bc; C2[i] = f.c2;
        }
    }
}
template <int M>
WT_DEV void load_bwd_coef(const FusedParams& P, const Geo& g, float (&X1)[M], float (&Kg)[M],
                          float (&Ky2)[M]) {
#pragma unroll
    for (int i = 0; i < M; ++i) {
        X1[i] = Kg[i] = Ky2[i] = 0.f;
        int gx = g.gx0 + i;
        if (g.colv && gx < P.nx) {
            size_t cell = P.coef_stride * g.inst + (size_t)gx * P.ny + g.col;
            BwdCoef k = bwd_coef(__ldg(P.b + cell), __ldg(P.c + cell), P.k);
            X1[i] = k.X1; Kg[i] = k.Kg; Ky2[i] = k.Ky2;
        }
    }
}

// Per-step factor of a cell's dL/dc (wavetorch/cell.py:36):
// grad_c = (X1 * (Kc * Lap(h_{t-1}))) * g, so dL/dc = (X1 * Kc) * sum_t Lap * g.
WT_DEV float dc_scale(const FusedParams& P, size_t cell) {
    const BwdCoef k = bwd_coef(__ldg(P.b + cell), __ldg(P.c + cell), P.k);
    return fmul(k.X1, k.Kc);
}

// Write the thread's per-instance dL/dc: its sums scaled by dc_scale.
template <int M>
WT_DEV void store_dc(const FusedParams& P, const Geo& g, const float (&acc)[M]) {
    float* o = P.gc_part + (size_t)g.inst * P.nx * P.ny;
#pragma unroll
    for (int i = 0; i < M; ++i) {
        int gx = g.gx0 + i;
        if (gx < P.nx) {
            const size_t cell = (size_t)gx * P.ny + g.col;
            o[cell] = fmul(dc_scale(P, P.coef_stride * g.inst + cell), acc[i]);
        }
    }
}



// v added to cell i of y, where i is a per-thread value: one select per cell
// (a runtime register index costs a jump per step on the owning warp, and a
// round trip through shared memory made that warp pace its whole cluster).
template <int M>
WT_DEV void add_at(float (&y)[M], int i, float v) {
#pragma unroll
    for (int k = 0; k < M; ++k) y[k] = (k == i) ? fadd(y[k], v) : y[k];
}
template <int M>
WT_DEV float value_at(const float (&y)[M], int i) {
    float v = 0.f;
#pragma unroll
    for (int k = 0; k < M; ++k) v = (k == i) ? y[k] : v;
    return v;
}

// Sources (in table order) with the inputs prefetched one step ahead.
template <int M>
WT_DEV void apply_sources(const FusedParams& P, const Taps& tp, float (&y)[M], float (&xv)[SRCMAX],
                          int tnext) {
#pragma unroll
    for (int e = 0; e < SRCMAX; ++e)
        if (e < tp.ns) add_at<M>(y, tp.src_i(e), xv[e]);   // xv: a register per entry
    if (tnext >= 0 && tnext < P.steps) {
#pragma unroll
        for (int e = 0; e < SRCMAX; ++e)
            if (e < tp.ns) xv[e] = __ldg(P.x + (size_t)tp.src_row(e) * P.steps + tnext);
    }
}

// h_t for the thread's cells from cur = h_{t-1} (registers + tile slot rs,
// halo words of exchange kr) and inout = h_{t-2}; the result overwrites inout
// (ping-pong register sets) and is published as exchange ks into slot ws
// (ks < 0: no halo words, the last step's have no reader).  The strip's end
// cells are updated and sent first, so a neighbour's halo is in flight while
// the interior cells are computed.  L receives Lap(h_{t-1}).  A thread that
// owns a source cell on a halo row injects before it sends.
template <int M, int ORDER>
WT_DEV void fwd_update(const FusedParams& P, const Geo& g, const Xchg& X, const Taps& tp, int rs,
                       int kr, int ws, int ks, float (&xv)[SRCMAX], int tnext,
                       const float (&A)[M], const float (&Bc)[M], const float (&C2)[M],
                       const float (&cur)[M], float (&inout)[M], float (&L)[M]) {
    if (!g.colv) return;   // padding columns read nothing (their tile columns do not exist)
    Column<M> c;
    load_sides<M>(c, P, g, X, rs, kr);
    L[0] = lap_cell<M, ORDER>(P, c, cur, 0);
    inout[0] = leapfrog(A[0], Bc[0], C2[0], P.k.two_over, cur[0], inout[0], L[0]);
    L[M - 1] = lap_cell<M, ORDER>(P, c, cur, M - 1);
    inout[M - 1] = leapfrog(A[M - 1], Bc[M - 1], C2[M - 1], P.k.two_over, cur[M - 1],
                            inout[M - 1], L[M - 1]);
    if (ks >= 0 && !tp.src_edge) send_halo(g, X, ks, inout[0], inout[M - 1]);
#pragma unroll
    for (int i = 1; i < M - 1; ++i) {
        L[i] = lap_cell<M, ORDER>(P, c, cur, i);
        inout[i] = leapfrog(A[i], Bc[i], C2[i], P.k.two_over, cur[i], inout[i], L[i]);
    }
    if (tp.wsrc && tp.ns) {
        apply_sources<M>(P, tp, inout, xv, tnext);
        if (ks >= 0 && tp.src_edge) send_halo(g, X, ks, inout[0], inout[M - 1]);
    }
    store_column<M>(P, g, X, ws, inout);
}

// Field-dependent coefficients of the nonlinear cell, in the reference's
// operation order (wavetorch/cell.py:8-9, :93-101):
//   sat = b0 / (1 + |h1 / uth|^2),  b = b_pml + rho * sat     (if b0 > 0)
//   c = c_lin + (rho * c_nl) * h1^2                           (if c_nl != 0)
struct NLCoef { float b, c, sat, q; };
WT_DEV NLCoef nl_coef(const FusedParams& P, float bpml, float clin, float rho, float h1) {
    NLCoef r;
    r.b = bpml; r.c = clin; r.sat = 0.f; r.q = 0.f;
    if (P.b0 > 0.f) {
        r.q = fdiv(h1, P.uth);
        const float a = fabsf(r.q);
        r.sat = fdiv(P.b0, fadd(1.0f, fmul(a, a)));
        r.b = fadd(bpml, fmul(rho, r.sat));
    }
    if (P.cnl != 0.f) r.c = fadd(clin, fmul(fmul(rho, P.cnl), fmul(h1, h1)));
    return r;
}

// fwd_update for the forward kernel's step loop, on precomputed addresses:
// step t reads tile slot RS = t & 1 and the halo words of exchange t-1
// (parity RS ^ 1), writes slot RS ^ 1 and sends exchange t (parity RS).
// Nonlinear cell (NL): k0, k1, k2 hold b_pml, c_lin and rho, and the update
// coefficients are formed from them and h_{t-1} every step; linear: k0, k1,
// k2 are the update coefficients A, Bc, c^2 themselves.
template <bool NL>
WT_DEV void cell_coef(const FusedParams& P, float k0, float k1, float k2, float h1, float& A,
                      float& Bc, float& C2) {
    if constexpr (NL) {
        const NLCoef n = nl_coef(P, k0, k1, k2, h1);
        const FwdCoef f = fwd_coef(n.b, n.c, P.k);
        A = f.A; Bc = f.Bc; C2 = f.c2;
    } else {
        A = k0; Bc = k1; C2 = k2;
    }
}

template <int M, int ORDER, int RS, bool NL = false>
WT_DEV void fwd_update_lane(const FusedParams& P, const Geo& g, const Xchg& X, const Lane& ln,
                            const Taps& tp, int t, bool send, float (&xv)[SRCMAX],
                            const float (&k0)[M], const float (&k1)[M], const float (&k2)[M],
                            const float (&cur)[M], float (&inout)[M], float (&L)[M]) {
    if (!g.colv) return;
    const float* rcol = ln.col0 + RS * ln.tile;
    float* wcol = ln.col0 + (RS ^ 1) * ln.tile;
    Column<M> c;
    lds_col<M>(c.lf, rcol - P.LD);
    lds_col<M>(c.rt, rcol + P.LD);
    c.up = rcol[-1];
    c.dn = rcol[M];
    if (t > 0) {
        if (ln.rup) c.up = recv_at(P, X, ln.rup + (RS ^ 1) * ln.pstride, t - 1);
        if (ln.rdn) c.dn = recv_at(P, X, ln.rdn + (RS ^ 1) * ln.pstride, t - 1);
    }
    auto update = [&](int i) {
        float A, Bc, C2;
        cell_coef<NL>(P, k0[i], k1[i], k2[i], cur[i], A, Bc, C2);
        L[i] = lap_cell<M, ORDER>(P, c, cur, i);
        inout[i] = leapfrog(A, Bc, C2, P.k.two_over, cur[i], inout[i], L[i]);
    };
    update(0);
    update(M - 1);
    const unsigned long long tag = (unsigned long long)(uint32_t)(t + 1) << 32;
    if (send && !tp.src_edge) {
        if (ln.sup) st_cluster_u64(ln.sup + RS * ln.pstride, tag | __float_as_uint(inout[0]));
        if (ln.sdn) st_cluster_u64(ln.sdn + RS * ln.pstride, tag | __float_as_uint(inout[M - 1]));
    }
#pragma unroll
    for (int i = 1; i < M - 1; ++i) update(i);
    if (tp.wsrc && tp.ns) {
        apply_sources<M>(P, tp, inout, xv, t + 1);
        if (send && tp.src_edge) {
            if (ln.sup) st_cluster_u64(ln.sup + RS * ln.pstride, tag | __float_as_uint(inout[0]));
            if (ln.sdn) st_cluster_u64(ln.sdn + RS * ln.pstride, tag | __float_as_uint(inout[M - 1]));
        }
    }
    sts_col<M>(wcol, inout);
}

struct FwdState {
    int pc;                   // step index within the probe chunk
    int pb;                   // probe ring buffer in use (0/1)
    float xv[SRCMAX];         // this step's source inputs
};

// Shared probe ring buffers of the forward: [2][n_prb][PB] raw amplitudes
// plus an ownership flag per probe column.  A probe's owner thread stores one
// value per step; every PB steps the whole CTA writes the finished chunk to
// the outputs, so the per-step cost on the owner's warp is one shared store.
struct ProbeRing {
    float* buf;
    int* own;
    float* ksum;    // [2][n_prb]: running Kahan sum and compensation of each owned column
};

// Write chunk `b` (steps t0 .. t0+n-1) of the probes this CTA owns.
WT_DEV void flush_probes(const FusedParams& P, const Geo& g, const ProbeRing& pr, int b, int t0,
                         int n) {
    const int tot = P.n_prb * P.PB;
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        const int q = idx / P.PB, tt = idx - q * P.PB;
        if (tt >= n || !pr.own[q]) continue;
        const float v = pr.buf[(b * P.n_prb + q) * P.PB + tt];
        const size_t oi = ((size_t)g.inst * P.steps + t0 + tt) * P.n_prb + q;
        P.out[oi] = (pr.own[q] == 2) ? fmul(v, v) : v;   // own: 1 amplitude, 2 intensity
        P.amp[oi] = v;
    }
    if (!P.psum) return;
    // Kahan-compensated time sums of the outputs, one thread per column, in
    // step order (the arithmetic of probe_sum_kernel)
    for (int q = threadIdx.x; q < P.n_prb; q += blockDim.x) {
        if (!pr.own[q]) continue;
        float s = pr.ksum[q], comp = pr.ksum[P.n_prb + q];
        const float* vb = pr.buf + (size_t)(b * P.n_prb + q) * P.PB;
        for (int tt = 0; tt < n; ++tt) {
            const float v = vb[tt];
            const float y = fsub((pr.own[q] == 2) ? fmul(v, v) : v, comp);
            const float tk = fadd(s, y);
            comp = fsub(fsub(tk, s), y);
            s = tk;
        }
        pr.ksum[q] = s;
        pr.ksum[P.n_prb + q] = comp;
    }
}

// The owned columns' sums, at the end of the forward.
WT_DEV void write_probe_sums(const FusedParams& P, const Geo& g, const ProbeRing& pr) {
    if (!P.psum) return;
    for (int q = threadIdx.x; q < P.n_prb; q += blockDim.x)
        if (pr.own[q]) P.psum[(size_t)g.inst * P.n_prb + q] = pr.ksum[q];
}

// Checkpoint of segment t/seg: the state before step t, (h_{t-1}, h_{t-2}).
template <int M>
WT_DEV void store_checkpoint(const FusedParams& P, const Geo& g, int t, const float (&h1)[M],
                             const float (&h2)[M]) {
    if (!g.colv) return;
    const size_t plane = (size_t)P.nx * P.ny;
    const size_t bplane = (size_t)P.batch * plane;
    float* cp = P.ckpt + (size_t)(t / P.seg) * 2 * bplane + (size_t)g.inst * plane;
#pragma unroll
    for (int i = 0; i < M; ++i) {
        int gx = g.gx0 + i;
        if (gx < P.nx) {
            size_t cell = (size_t)gx * P.ny + g.col;
            __stcg(cp + cell, h1[i]);
            __stcg(cp + bplane + cell, h2[i]);
        }
    }
}

// One step of the forward kernel (everything but the closing barrier).
// RS = t & 1 (the tile slot holding h_{t-1}); tape points at this thread's
// chunk 0 of step t's tape slice.
template <int M, int ORDER, bool FIELDS, int RS>
WT_DEV void fwd_step(const FusedParams& P, const Geo& g, const Xchg& X, const Lane& ln,
                     const Taps& tp, FwdState& st, const ProbeRing& pr, int t, float* tape,
                     const float (&A)[M], const float (&Bc)[M], const float (&C2)[M],
                     const float (&cur)[M], float (&inout)[M]) {
    float L[M];
    // exchange t carries h_t; tile slot RS ^ 1 holds it (h_{-1} = 0 is slot 0)
    fwd_update_lane<M, ORDER, RS>(P, g, X, ln, tp, t, t + 1 < P.steps, st.xv, A, Bc, C2, cur,
                                  inout, L);
    if (!g.colv) return;
    if (tape) {           // tape for the adjoint: this thread's M values of Lap(h_{t-1})
        constexpr int V = chunk_width<M>();
        const int stride = (int)blockDim.x * V;
#pragma unroll
        for (int j = 0; j < M / V; ++j) {
            float* p = tape + j * stride;
            if constexpr (V == 4)
                *reinterpret_cast<float4*>(p) = make_float4(L[4 * j], L[4 * j + 1], L[4 * j + 2], L[4 * j + 3]);
            else if constexpr (V == 2)
                *reinterpret_cast<float2*>(p) = make_float2(L[2 * j], L[2 * j + 1]);
            else
                *p = L[j];
        }
    }
    if (tp.wprb && tp.np) {   // probe values from the column just stored (no register indexing)
        const float* colp = ln.col0 + (RS ^ 1) * ln.tile;
        float* row = pr.buf + (size_t)st.pb * P.n_prb * P.PB + st.pc;
#pragma unroll
        for (int e = 0; e < PRBMAX; ++e)
            if (e < tp.np) row[tp.prb_col(e) * P.PB] = colp[tp.prb_i(e)];
    }
    if (FIELDS) {
        const size_t plane = (size_t)P.nx * P.ny;
        float* fo = P.fields + ((size_t)g.inst * P.steps + t) * plane;
#pragma unroll
        for (int i = 0; i < M; ++i) {
            int gx = g.gx0 + i;
            if (gx < P.nx) fo[(size_t)gx * P.ny + g.col] = inout[i];
        }
    }
}

// CTA barrier closing an exchange; false when the CTA must leave its loop.
// The abort word (set only after a 2 s wait gave up) is read every 32nd
// barrier: all threads read it after the same barrier, so they agree.
WT_DEV bool exchange_end(const Xchg& X, int k) {
    __syncthreads();
    return (k & 31) != 0 || *(volatile int*)X.abort == 0;
}

// Threads per CTA a strip height allows (register budget per thread): the
// forward keeps 5 values per cell, the adjoint about twice as many.
constexpr int fwd_max_threads(int M) {
    return M <= 5 ? 768 : M == 6 ? 640 : M == 8 ? 512 : M <= 10 ? 384 : 256;
}
constexpr int bwd_max_threads(int M) { return M >= 10 ? 384 : 512; }
// Per-thread coefficient words of the nonlinear adjoint (b_pml, c_lin, rho).
// Per-thread shared words of the nonlinear adjoint: b_pml, c_lin, rho of its
// cells, and with CACHE also the step's X1, q and sat from the first half of
// the step (the exchange of Kg * lambda) for the second (odd: conflict-free)
__host__ __device__ constexpr int nl_coef_stride(int M, bool cache) { return ((cache ? 6 : 3) * M) | 1; }

// ============================================================================
// Forward
template <int M, int ORDER, bool FIELDS>
__global__ void __launch_bounds__(fwd_max_threads(M), 1) seq_fwd_fused_kernel(FusedParams P) {
    extern __shared__ __align__(16) float smem[];
    __shared__ int abort_flag;
    const Geo g = make_geo(P, M);
    const int tile = (P.ny + 2) * P.LD;
    ProbeRing pr;
    pr.buf = smem + 2 * tile + 2 * xchg_words(P.NCP);
    pr.own = reinterpret_cast<int*>(pr.buf + 2 * P.n_prb * P.PB);
    pr.ksum = reinterpret_cast<float*>(pr.own + P.n_prb);
    zero_smem(smem, 2 * tile);
    for (int q = threadIdx.x; q < P.n_prb; q += blockDim.x) {
        pr.own[q] = 0;
        pr.ksum[q] = pr.ksum[P.n_prb + q] = 0.f;
    }
    Xchg X;
    xchg_setup(X, P, g, smem, tile, &abort_flag);

    float A[M], Bc[M], C2[M], ya[M], yb[M];
    load_fwd_coef<M>(P, g, A, Bc, C2);
#pragma unroll
    for (int i = 0; i < M; ++i) ya[i] = yb[i] = 0.f;
    Taps tp;
    build_taps<M>(P, g, tp);
    FwdState st;
    st.pc = 0;
    st.pb = 0;
#pragma unroll
    for (int e = 0; e < SRCMAX; ++e)
        st.xv[e] = e < tp.ns ? __ldg(P.x + (size_t)tp.src_row(e) * P.steps) : 0.f;
    __syncthreads();      // ownership flags cleared before the owners mark theirs
    if (g.colv && tp.np) {
#pragma unroll
        for (int e = 0; e < PRBMAX; ++e)
            if (e < tp.np) pr.own[tp.prb_col(e)] = tp.prb_intensity(e) ? 2 : 1;
    }
    cluster_sync_all();   // zeroed tiles, halo words and flags, cluster-wide

    // ya holds h_{t-1} at even t, yb at odd t (the update overwrites h_{t-2});
    // the outer loop runs one checkpoint segment per iteration
    const Lane ln = make_lane(P, g, X);
    // tape: this thread's chunk 0 of step 0's slice, advanced one step at a time
    float* tape = P.lap ? P.lap + ((size_t)g.inst * P.C + g.cta) * blockDim.x * M +
                              (size_t)threadIdx.x * chunk_width<M>()
                        : nullptr;
    const size_t tape_step = (size_t)P.batch * P.C * blockDim.x * M;
    int chunk0 = 0;       // first step of the probe chunk being filled
    bool ok = true;
    for (int t0 = 0; t0 < P.steps && ok; t0 += P.seg) {
        if (t0 > 0) {
            if (t0 & 1) store_checkpoint<M>(P, g, t0, yb, ya);
            else        store_checkpoint<M>(P, g, t0, ya, yb);
        }
        const int t1 = min(P.steps, t0 + P.seg);
        for (int t = t0; t < t1; ++t) {
            if (t & 1) fwd_step<M, ORDER, FIELDS, 1>(P, g, X, ln, tp, st, pr, t, tape, A, Bc, C2, yb, ya);
            else       fwd_step<M, ORDER, FIELDS, 0>(P, g, X, ln, tp, st, pr, t, tape, A, Bc, C2, ya, yb);
            if (tape) tape += tape_step;
            if (!(ok = exchange_end(X, t))) break;
            if (++st.pc == P.PB) {
                flush_probes(P, g, pr, st.pb, chunk0, P.PB);
                st.pc = 0;
                st.pb ^= 1;
                chunk0 = t + 1;
            }
        }
    }
    if (st.pc > 0) flush_probes(P, g, pr, st.pb, chunk0, st.pc);
    write_probe_sums(P, g, pr);
    cluster_sync_all();
}

// ============================================================================
// Nonlinear cell, forward (tape mode): as seq_fwd_fused_kernel, with b and c
// formed every step from h_{t-1} (nl_coef) and a two-part tape per step:
// Lap(h_{t-1}) and h_{t-1}, each chunk-major (threads x M floats).
template <int M>
WT_DEV void load_nl_coef(const FusedParams& P, const Geo& g, float (&bp)[M], float (&cl)[M],
                         float (&rh)[M]) {
#pragma unroll
    for (int i = 0; i < M; ++i) {
        bp[i] = cl[i] = rh[i] = 0.f;
        int gx = g.gx0 + i;
        if (g.colv && gx < P.nx) {
            size_t cell = P.coef_stride * g.inst + (size_t)gx * P.ny + g.col;
            bp[i] = __ldg(P.b + cell);
            cl[i] = __ldg(P.c + cell);
            rh[i] = __ldg(P.rho + cell);
        }
    }
}

template <int M, int ORDER, int RS>
WT_DEV void fwd_step_nl(const FusedParams& P, const Geo& g, const Xchg& X, const Lane& ln,
                        const Taps& tp, FwdState& st, const ProbeRing& pr, int t, float* tape,
                        const float (&bp)[M], const float (&cl)[M], const float (&rh)[M],
                        const float (&cur)[M], float (&inout)[M]) {
    float L[M];
    fwd_update_lane<M, ORDER, RS, true>(P, g, X, ln, tp, t, t + 1 < P.steps, st.xv, bp, cl, rh,
                                        cur, inout, L);
    if (!g.colv) return;
    const int stride = (int)blockDim.x * chunk_width<M>();
    st_chunks_at<M>(tape, stride, L);
    st_chunks_at<M>(tape + (size_t)blockDim.x * M, stride, cur);
    if (tp.wprb && tp.np) {
        const float* colp = ln.col0 + (RS ^ 1) * ln.tile;
        float* row = pr.buf + (size_t)st.pb * P.n_prb * P.PB + st.pc;
#pragma unroll
        for (int e = 0; e < PRBMAX; ++e)
            if (e < tp.np) row[tp.prb_col(e) * P.PB] = colp[tp.prb_i(e)];
    }
}

template <int M, int ORDER>
__global__ void __launch_bounds__(fwd_max_threads(M), 1) seq_fwd_nl_kernel(FusedParams P) {
    extern __shared__ __align__(16) float smem[];
    __shared__ int abort_flag;
    const Geo g = make_geo(P, M);
    const int tile = (P.ny + 2) * P.LD;
    ProbeRing pr;
    pr.buf = smem + 2 * tile + 2 * xchg_words(P.NCP);
    pr.own = reinterpret_cast<int*>(pr.buf + 2 * P.n_prb * P.PB);
    pr.ksum = reinterpret_cast<float*>(pr.own + P.n_prb);
    zero_smem(smem, 2 * tile);
    for (int q = threadIdx.x; q < P.n_prb; q += blockDim.x) {
        pr.own[q] = 0;
        pr.ksum[q] = pr.ksum[P.n_prb + q] = 0.f;
    }
    Xchg X;
    xchg_setup(X, P, g, smem, tile, &abort_flag);

    float bp[M], cl[M], rh[M], ya[M], yb[M];
    load_nl_coef<M>(P, g, bp, cl, rh);
#pragma unroll
    for (int i = 0; i < M; ++i) ya[i] = yb[i] = 0.f;
    Taps tp;
    build_taps<M>(P, g, tp);
    FwdState st;
    st.pc = 0;
    st.pb = 0;
#pragma unroll
    for (int e = 0; e < SRCMAX; ++e)
        st.xv[e] = e < tp.ns ? __ldg(P.x + (size_t)tp.src_row(e) * P.steps) : 0.f;
    __syncthreads();
    if (g.colv && tp.np) {
#pragma unroll
        for (int e = 0; e < PRBMAX; ++e)
            if (e < tp.np) pr.own[tp.prb_col(e)] = tp.prb_intensity(e) ? 2 : 1;
    }
    cluster_sync_all();

    const Lane ln = make_lane(P, g, X);
    const size_t part = (size_t)blockDim.x * M;       // floats per tape part
    float* tape = P.lap + ((size_t)g.inst * P.C + g.cta) * 2 * part +
                  (size_t)threadIdx.x * chunk_width<M>();
    const size_t tape_step = (size_t)P.batch * P.C * 2 * part;
    int chunk0 = 0;
    bool ok = true;
    for (int t = 0; t < P.steps; ++t) {
        if (t & 1) fwd_step_nl<M, ORDER, 1>(P, g, X, ln, tp, st, pr, t, tape, bp, cl, rh, yb, ya);
        else       fwd_step_nl<M, ORDER, 0>(P, g, X, ln, tp, st, pr, t, tape, bp, cl, rh, ya, yb);
        tape += tape_step;
        if (!(ok = exchange_end(X, t))) break;
        if (++st.pc == P.PB) {
            flush_probes(P, g, pr, st.pb, chunk0, P.PB);
            st.pc = 0;
            st.pb ^= 1;
            chunk0 = t + 1;
        }
    }
    if (st.pc > 0) flush_probes(P, g, pr, st.pb, chunk0, st.pc);
    write_probe_sums(P, g, pr);
    cluster_sync_all();
}

// ============================================================================
// Adjoint with segment recompute.
// Per-thread stash: step s of the segment holds the thread's M values
// contiguously at p + s*NT*M (vector stores/loads; the per-lane stride of M
// floats keeps float2/float4 accesses conflict-free for M = 10 / 8 / 4).
template <int M>
struct Stash {
    float* p;       // this thread's step-0 entry
    int NT;
    WT_DEV float* step(int s) const { return p + (size_t)s * NT * M; }
};

// Recompute step: like fwd_step, but stashes Lap(h_{t-1}) instead of writing outputs.
template <int M, int ORDER>
WT_DEV void rec_step(const FusedParams& P, const Geo& g, const Xchg& X, const Taps& tp,
                     float (&xv)[SRCMAX], int t, int t0, int t1, int kx,
                     const Stash<M>& sh, const float (&A)[M], const float (&Bc)[M],
                     const float (&C2)[M], const float (&cur)[M], float (&inout)[M]) {
    float L[M];
    // reads exchange kx (slot kx&1), publishes exchange kx+1 when the segment goes on
    fwd_update<M, ORDER>(P, g, X, tp, kx & 1, kx, (kx + 1) & 1, t + 1 < t1 ? kx + 1 : -1, xv,
                         t + 1 < t1 ? t + 1 : -1, A, Bc, C2, cur, inout, L);
    if (!g.colv) return;
    sts_col<M>(sh.step(t - t0), L);
}

// Stage the adjoint seeds of chunk c (adjoint steps u = c*PB .. c*PB+PB-1,
// i.e. t = T-1-u) of every probe column into ring buffer c & 1:
// intensity g * (2 y) (autograd's PowBackward), amplitude g.
WT_DEV void stage_seeds(const FusedParams& P, const Geo& g, float* seeds, int c) {
    float* dst = seeds + (size_t)(c & 1) * P.n_prb * P.PB;
    const int tot = P.n_prb * P.PB;
    for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        const int q = idx / P.PB, k = idx - q * P.PB;
        const int t = P.steps - 1 - (c * P.PB + k);
        float sd = 0.f;
        if (t >= 0) {
            const size_t oi = ((size_t)g.inst * P.steps + t) * P.n_prb + q;
            const float gv = P.grad_w ? __ldg(P.grad_w + (size_t)g.inst * P.n_prb + q)
                                      : __ldg(P.grad_out + oi);
            sd = __ldg(P.prb_kind_col + q) ? fmul(gv, fmul(2.0f, __ldg(P.amp + oi))) : gv;
        }
        dst[q * P.PB + k] = sd;
    }
}

// Probe seeds into lam (descending reference order) and dL/dx at the
// source, for the few threads that own such cells, in registers (add_at).
template <int M>
WT_DEV void seed_and_read(const FusedParams& P, const Geo& g, const Taps& tp, int t,
                          float (&lam)[M], const float* sr) {
    // a loop on the thread's own count, not unrolled: threads without probes
    // (whole warps, nearly always) branch over it rather than run it
    // predicated off on every step
#pragma unroll 1
    for (int e = 0; e < tp.np; ++e) add_at<M>(lam, tp.prb_i(e), sr[tp.prb_col(e) * P.PB]);
    if (P.grad_x && tp.ns) {
#pragma unroll
        for (int e = 0; e < SRCMAX; ++e)
            if (e < tp.ns && tp.src_row(e) == g.inst)
                P.grad_x[(size_t)g.inst * P.steps + t] = value_at<M>(lam, tp.src_i(e));
    }
}

// Adjoint of one cell (wavetorch/cell.py:36-42): pending grad_y1 / grad_y2
// terms in autograd's order, and the running sum acc = sum_t Lap(h_{t-1}) *
// lam_t of the cell's dL/dc = X1 * Kc * acc (the per-step factor
// X1 * Kc = (b dt + 1)^-1 * 2 c dt^2 is applied once, when the sum is
// written: dc_scale).
WT_DEV void adj_cell(float lg, float lam, float Ly, float X1, float Ky2, float dt2,
                     float& acc, float& gy1, float& gy2a, float& gy2b) {
    acc = ffma(Ly, lam, acc);
    gy1 = fadd(fmul(dt2, lg), fmul(fmul(2.0f, lam), X1));
    gy2b = gy2a;
    gy2a = fmul(Ky2, lam);
}

// adj_cell with lambda formed one step ahead: lam enters as this step's
// (seeded) lambda and leaves as the next step's, fadd(grad_y2 term of the
// step after this one, this step's grad_y1 term) in autograd's order; pend
// carries this step's grad_y2 term one step.  Same operations as adj_cell
// followed by the next step's sum (which the checkpoint kernel forms at the
// start of that step).
WT_DEV void adj_cell_lp(float lg, float& lam, float Ly, float X1, float Ky2, float dt2,
                        float& acc, float& pend) {
    acc = ffma(Ly, lam, acc);
    const float gy1 = fadd(fmul(dt2, lg), fmul(fmul(2.0f, lam), X1));
    const float g2 = fmul(Ky2, lam);
    lam = fadd(pend, gy1);
    pend = g2;
}

template <int M, int ORDER>
__global__ void __launch_bounds__(bwd_max_threads(M), 1) seq_bwd_fused_kernel(FusedParams P) {
    extern __shared__ __align__(16) float smem[];
    __shared__ int abort_flag;
    const Geo g = make_geo(P, M);
    const int NT = blockDim.x;
    const int tile = (P.ny + 2) * P.LD;
    zero_smem(smem, 2 * tile);
    Xchg X;
    xchg_setup(X, P, g, smem, tile, &abort_flag);
    Taps tp;
    build_taps<M>(P, g, tp);

    const size_t plane = (size_t)P.nx * P.ny;
    const size_t bplane = (size_t)P.batch * plane;
    // adjoint seeds of all probe columns, staged per chunk of PB adjoint
    // steps: seeds[2][n_prb][PB], u = T-1-t counts adjoint steps
    float* seeds = smem + 2 * tile + 2 * xchg_words(P.NCP);
    Stash<M> sh;
    sh.NT = NT;
    sh.p = P.stash_smem ? seeds + ((2 * P.n_prb * P.PB + 3) & ~3) + (size_t)threadIdx.x * M
                        : P.stash + ((size_t)(g.inst * P.C + g.cta) * P.seg) * M * NT +
                              (size_t)threadIdx.x * M;

    // adjoint state: gy1 pending from t+1, gy2 pending from t+1 (a) and t+2 (b).
    // Zero-initialised, so the first arrivals reproduce autograd's "first
    // gradient is stored" up to the sign of an exact zero.
    float gy1[M], gy2a[M], gy2b[M], acc[M];
#pragma unroll
    for (int i = 0; i < M; ++i) gy1[i] = gy2a[i] = gy2b[i] = acc[i] = 0.f;
    stage_seeds(P, g, seeds, 0);
    int u = 0;            // adjoint steps done

    cluster_sync_all();
    const int nseg = (P.steps + P.seg - 1) / P.seg;
    int kx = 0;           // exchange index (tile slot kx & 1)
    bool ok = true;
    for (int sgi = nseg - 1; sgi >= 0 && ok; --sgi) {
        const int t0 = sgi * P.seg;
        const int t1 = min(P.steps, t0 + P.seg);
        // ---- recompute the segment's forward, stashing Lap(h_{t-1}) ----
        {
            float ya[M], yb[M];   // h_{t0-1}, h_{t0-2}
#pragma unroll
            for (int i = 0; i < M; ++i) ya[i] = yb[i] = 0.f;
            if (sgi > 0 && g.colv) {
                const float* cp = P.ckpt + (size_t)sgi * 2 * bplane + (size_t)g.inst * plane;
#pragma unroll
                for (int i = 0; i < M; ++i) {
                    int gx = g.gx0 + i;
                    if (gx < P.nx) {
                        size_t cell = (size_t)gx * P.ny + g.col;
                        ya[i] = __ldcg(cp + cell);
                        yb[i] = __ldcg(cp + bplane + cell);
                    }
                }
            }
            publish<M>(P, g, X, kx & 1, kx, ya);
            if (!(ok = exchange_end(X, 0))) break;
            float A[M], Bc[M], C2[M];
            load_fwd_coef<M>(P, g, A, Bc, C2);
            float xv[SRCMAX];
#pragma unroll
            for (int e = 0; e < SRCMAX; ++e)
                xv[e] = (e < tp.ns) ? __ldg(P.x + (size_t)tp.src_row(e) * P.steps + t0) : 0.f;
            for (int t = t0; t < t1;) {
                rec_step<M, ORDER>(P, g, X, tp, xv, t, t0, t1, kx, sh, A, Bc, C2, ya, yb);
                ++kx;             // exchange kx consumed (the last one of the segment too)
                if (++t >= t1) break;
                if (!(ok = exchange_end(X, t))) break;
                rec_step<M, ORDER>(P, g, X, tp, xv, t, t0, t1, kx, sh, A, Bc, C2, yb, ya);
                ++kx;
                if (++t >= t1) break;
                if (!(ok = exchange_end(X, t))) break;
            }
            if (!ok) break;
        }
        // the last recompute step's stash entries were written by this thread
        // itself, so the adjoint reads them back without a barrier
        // ---- adjoint sweep over the segment ----
        float X1[M], Kg[M], Ky2[M];
        load_bwd_coef<M>(P, g, X1, Kg, Ky2);
        for (int t = t1 - 1; t >= t0; --t) {
            float lam[M], c2g[M];
#pragma unroll
            for (int i = 0; i < M; ++i) {
                lam[i] = fadd(gy2b[i], gy1[i]);
                c2g[i] = 0.f;
            }
            if (u % P.PB == 0 && u + P.PB < P.steps)   // next chunk, a barrier ahead of use
                stage_seeds(P, g, seeds, u / P.PB + 1);
            if (g.colv) {
                if ((tp.wprb || tp.wsrc) && (tp.np || (P.grad_x && tp.ns)))
                    seed_and_read<M>(P, g, tp, t, lam,
                                     seeds + (size_t)((u / P.PB) & 1) * P.n_prb * P.PB + u % P.PB);
#pragma unroll
                for (int i = 0; i < M; ++i) c2g[i] = fmul(Kg[i], lam[i]);
                publish<M>(P, g, X, kx & 1, kx, c2g);
            }
            if (!(ok = exchange_end(X, u))) break;
            ++u;
            if (g.colv) {
                Column<M> c;
                load_sides<M>(c, P, g, X, kx & 1, -1);   // interior first; halo words below
                float Ly[M];
                lds_col<M>(Ly, sh.step(t - t0));
#pragma unroll
                for (int i = 1; i < M - 1; ++i)
                    adj_cell(lap_cell<M, ORDER>(P, c, c2g, i), lam[i], Ly[i], X1[i], Ky2[i],
                             P.k.dt2, acc[i], gy1[i], gy2a[i], gy2b[i]);
                if (g.strip == 0 && g.has_up)
                    c.up = recv_word(P, X, X.hup + (kx & 1) * X.NCP + g.col, kx);
                if (g.strip == g.S - 1 && g.has_dn)
                    c.dn = recv_word(P, X, X.hdn + (kx & 1) * X.NCP + g.col, kx);
                adj_cell(lap_cell<M, ORDER>(P, c, c2g, 0), lam[0], Ly[0], X1[0], Ky2[0],
                         P.k.dt2, acc[0], gy1[0], gy2a[0], gy2b[0]);
                adj_cell(lap_cell<M, ORDER>(P, c, c2g, M - 1), lam[M - 1], Ly[M - 1], X1[M - 1],
                         Ky2[M - 1], P.k.dt2, acc[M - 1], gy1[M - 1], gy2a[M - 1],
                         gy2b[M - 1]);
            }
            ++kx;
        }
    }
    if (g.colv && ok) store_dc<M>(P, g, acc);
    cluster_sync_all();
}

// ============================================================================
// Adjoint in tape mode: the forward stored Lap(h_{t-1}) of every cell and
// step, so the adjoint runs its T steps in one sweep with no recompute.  The
// tape is laid out [step][instance][cta][chunk][thread] (chunk-major, see
// chunk_width): both kernels use the same strips, so a CTA's values of one
// step are one contiguous slice, written with coalesced vector stores and
// read back from shared memory without bank conflicts.  Slices
// arrive by bulk copy into a ring of `nbuf` shared-memory slots, issued by
// thread 0 nbuf-1 steps ahead of use; slot t % nbuf holds step t, and its
// mbarrier's phase parity for step t is ((T-1-t) / nbuf) & 1.
struct TapeRing {
    float* buf;                     // nbuf slices
    unsigned long long* full;       // nbuf mbarriers
    int slice;                      // floats per slice (threads * M)
};

// Issue step t's slice into slot s; false when the missing-slice test hook
// holds it back (from its step on, the producer issues nothing more, so every
// copy in flight still has its slot's expected phase).
WT_DEV bool tape_issue(const FusedParams& P, const Geo& g, const TapeRing& r, int t, int s) {
    if (t + 1 <= P.skip_slice1) return false;
    const float* src = P.lap + (((size_t)t * P.batch + g.inst) * P.C + g.cta) * r.slice;
    const uint32_t mb = smem_addr(r.full + s);
    const uint32_t bytes = (uint32_t)(r.slice * sizeof(float));
    mbar_arrive_expect_tx(mb, bytes);
    bulk_g2s(smem_addr(r.buf + (size_t)s * r.slice), src, bytes, mb);
    return true;
}

// Bounded wait for the phase of parity `par` of slot s.  A wait that sees
// the abort word gives up at once, unless it drains the copies in flight
// before the kernel leaves (heed_abort false).
WT_DEV bool tape_wait(const FusedParams& P, const Xchg& X, const TapeRing& r, int s, uint32_t par,
                      bool heed_abort = true) {
    const uint32_t mb = smem_addr(r.full + s);
    if (mbar_try_wait_parity_cta(mb, par)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait_parity_cta(mb, par)) {
        if (heed_abort && *(volatile int*)X.abort) return false;   // another wait gave up
        if (global_ns() - t0 > WAIT_LIMIT_NS) {
            atomicExch(P.err, WT_DEVERR_TIMEOUT);
            *(volatile int*)X.abort = 1;
            return false;
        }
    }
    return true;
}

template <int M, int ORDER>
__global__ void __launch_bounds__(bwd_max_threads(M), 1) seq_bwd_tape_kernel(FusedParams P) {
    extern __shared__ __align__(16) float smem[];
    __shared__ int abort_flag;
    const Geo g = make_geo(P, M);
    const int tile = (P.ny + 2) * P.LD;
    zero_smem(smem, 2 * tile);
    Xchg X;
    xchg_setup(X, P, g, smem, tile, &abort_flag);
    Taps tp;
    build_taps<M>(P, g, tp);

    float* seeds = smem + 2 * tile + 2 * xchg_words(P.NCP);
    TapeRing ring;
    ring.buf = seeds + ((2 * P.n_prb * P.PB + 3) & ~3);
    ring.slice = (int)blockDim.x * M;
    ring.full = reinterpret_cast<unsigned long long*>(ring.buf + (size_t)P.nbuf * ring.slice);
    if (threadIdx.x == 0) {
        for (int s = 0; s < P.nbuf; ++s) mbar_init(smem_addr(ring.full + s), 1);
        fence_mbarrier_init_cluster();
    }

    float X1[M], Kg[M], Ky2[M];
    load_bwd_coef<M>(P, g, X1, Kg, Ky2);
    // adjoint state: lam (this step's lambda before its seeds), pend (the
    // grad_y2 term of the previous step), the running dL/dc
    float lam[M], pend[M], acc[M];
#pragma unroll
    for (int i = 0; i < M; ++i) lam[i] = pend[i] = acc[i] = 0.f;
    stage_seeds(P, g, seeds, 0);
    cluster_sync_all();   // zeroed tiles, ring and halo words; barriers initialised

    int lo = P.steps;     // lowest step issued (thread 0)
    if (threadIdx.x == 0) {
        for (int j = 0; j < P.nbuf && P.steps - 1 - j >= 0; ++j) {
            const int t = P.steps - 1 - j;
            if (tape_issue(P, g, ring, t, t % P.nbuf)) lo = t;
        }
    }
    // per-step counters kept incrementally (no division on the step path):
    // slot = t % nbuf, phase bit s = parity of the next wait on slot s,
    // pk = u % PB, pc = u / PB
    int slot = (P.steps - 1) % P.nbuf;
    uint32_t phase = 0;
    int pk = 0, pc = 0;
    bool ok = true;
    const Lane ln = make_lane(P, g, X);
    const bool issuer = threadIdx.x == 0;
    const bool taps_here = tp.np || (P.grad_x && tp.ns);   // seeds to add / dL/dx to read
    const bool taps_warp = tp.wprb || (P.grad_x && tp.wsrc);
    // this thread's chunk 0 in the slot of the current step (kept
    // incrementally), and the chunk stride of a slice
    constexpr int V = chunk_width<M>();
    const int cstride = (int)blockDim.x * V;
    const float* ly_top = ring.buf + (size_t)(P.nbuf - 1) * ring.slice + (size_t)threadIdx.x * V;
    const float* ly = ly_top - (size_t)(P.nbuf - 1 - slot) * ring.slice;
    // One adjoint step on the precomputed addresses; exchange u uses tile
    // slot and word parity PAR = u & 1.
    auto step = [&](auto par, int u) -> bool {
        constexpr int PAR = decltype(par)::value;
        const int t = P.steps - 1 - u;
        float* col = ln.col0 + PAR * ln.tile;
        float c2g[M];
        if (pk == 0 && u + P.PB < P.steps)   // next chunk, a barrier ahead of use
            stage_seeds(P, g, seeds, pc + 1);
        if (g.colv) {
            if (taps_warp && taps_here)
                seed_and_read<M>(P, g, tp, t, lam, seeds + (size_t)(pc & 1) * P.n_prb * P.PB + pk);
#pragma unroll
            for (int i = 0; i < M; ++i) c2g[i] = fmul(Kg[i], lam[i]);
            const unsigned long long tag = (unsigned long long)(uint32_t)(u + 1) << 32;
            if (ln.sup) st_cluster_u64(ln.sup + PAR * ln.pstride, tag | __float_as_uint(c2g[0]));
            if (ln.sdn) st_cluster_u64(ln.sdn + PAR * ln.pstride, tag | __float_as_uint(c2g[M - 1]));
            sts_col<M>(col, c2g);
        }
        if (!exchange_end(X, u)) return false;
        // step t+1's slice was read before this barrier: refill its slot
        // (not once a wait gave up: a wait that saw the abort word may have
        // left its slot's copy in flight, which the drain below then covers)
        if (issuer && u > 0 && t + 1 - P.nbuf >= 0 && *(volatile int*)X.abort == 0) {
            fence_proxy_async_smem();
            if (tape_issue(P, g, ring, t + 1 - P.nbuf, slot + 1 == P.nbuf ? 0 : slot + 1))
                lo = t + 1 - P.nbuf;
        }
        if (g.colv) {
            Column<M> c;
            lds_col<M>(c.lf, col - P.LD);
            lds_col<M>(c.rt, col + P.LD);
            c.up = col[-1];
            c.dn = col[M];
            tape_wait(P, X, ring, slot, (phase >> slot) & 1u);
            phase ^= 1u << slot;
            float Ly[M];
            ld_chunks_at<M>(Ly, ly, cstride);
#pragma unroll
            for (int i = 1; i < M - 1; ++i)
                adj_cell_lp(lap_cell<M, ORDER>(P, c, c2g, i), lam[i], Ly[i], X1[i], Ky2[i],
                            P.k.dt2, acc[i], pend[i]);
            if (ln.rup) c.up = recv_at(P, X, ln.rup + PAR * ln.pstride, u);
            if (ln.rdn) c.dn = recv_at(P, X, ln.rdn + PAR * ln.pstride, u);
            adj_cell_lp(lap_cell<M, ORDER>(P, c, c2g, 0), lam[0], Ly[0], X1[0], Ky2[0],
                        P.k.dt2, acc[0], pend[0]);
            adj_cell_lp(lap_cell<M, ORDER>(P, c, c2g, M - 1), lam[M - 1], Ly[M - 1], X1[M - 1],
                        Ky2[M - 1], P.k.dt2, acc[M - 1], pend[M - 1]);
        }
        if (slot == 0) { slot = P.nbuf - 1; ly = ly_top; }
        else           { --slot; ly -= ring.slice; }
        if (++pk == P.PB) { pk = 0; ++pc; }
        return true;
    };
    // two steps per iteration: the exchange parity is fixed in each
    for (int u = 0; u < P.steps && ok; u += 2) {
        ok = step(std::integral_constant<int, 0>{}, u);
        if (ok && u + 1 < P.steps) ok = step(std::integral_constant<int, 1>{}, u + 1);
    }
    if (!ok && threadIdx.x == 0) {
        // leaving early: let the copies still in flight land first (the last
        // nbuf issued steps hold one copy per slot, step s in slot s % nbuf
        // at parity ((T-1-s) / nbuf) & 1; waits are bounded)
        for (int s = lo; s < lo + P.nbuf && s < P.steps; ++s)
            tape_wait(P, X, ring, s % P.nbuf, (uint32_t)(((P.steps - 1 - s) / P.nbuf) & 1), false);
    }
    if (g.colv && ok) store_dc<M>(P, g, acc);
    cluster_sync_all();
}

// ============================================================================
// Checkpoint adjoint with the segment recompute running beside the adjoint.
// The CTA's threads form two groups of NG = blockDim.x / 2 with the same
// strip layout: group R (threads [0, NG)) recomputes the forward of segment
// s - 1 from its checkpoint while group A (threads [NG, 2 NG)) runs the
// adjoint steps of segment s, from the Laplacians R stored in the phase
// before.  Phase p pairs R on segment nseg-1-p with A on segment nseg-p, and
// the CTA meets at one barrier per phase.  Each group is a step chain whose
// pace is set by its exchanges with the neighbouring CTAs rather than by
// issue, so each group's instructions fill the other's idle issue slots.
//
// R writes the Laplacians of segment s into half (s & 1) of this CTA's stash
// [2][seg][slice] in global memory (a slice: NG x M floats in the tape's
// chunk-major layout), and A streams them back through the tape kernel's
// ring of bulk copies.  Each group has its own tile slots, halo words and
// exchange sequence and synchronises on its own named barrier; the per-cell
// coefficients of both live in shared memory (the groups share the register
// file).  The arithmetic is the tape kernels', operand for operand.
constexpr int WS_BAR_R = 1, WS_BAR_A = 2;

WT_DEV void ws_bar(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }

// Group barrier closing an exchange; false when the CTA must leave its loop
// (the abort word, read every 32nd barrier by the whole group).
WT_DEV bool ws_exchange_end(const Xchg& X, int id, int n, int k) {
    ws_bar(id, n);
    return (k & 31) != 0 || *(volatile int*)X.abort == 0;
}

WT_DEV Geo ws_geo(const FusedParams& P, int M, int ltid) {
    Geo g;
    g.cta = (int)cluster_ctarank();
    g.inst = blockIdx.x / P.C;
    g.col = ltid % P.NCP;
    g.strip = ltid / P.NCP;
    g.xl0 = g.strip * M;
    g.gx0 = g.cta * P.R + g.xl0;
    g.S = P.R / M;
    g.colv = g.col < P.ny;
    g.has_up = g.cta > 0;
    g.has_dn = g.cta + 1 < P.C;
    return g;
}

WT_DEV void ws_xchg(Xchg& X, const FusedParams& P, const Geo& g, float* tiles, int tile,
                    unsigned long long* words, int* abort) {
    X.tiles = tiles;
    X.tile = tile;
    X.NCP = P.NCP;
    X.hup = words;
    X.hdn = words + 2 * P.NCP;
    X.abort = abort;
    X.up_hdn = g.has_up ? map_shared_rank(X.hdn, g.cta - 1) : 0u;
    X.dn_hup = g.has_dn ? map_shared_rank(X.hup, g.cta + 1) : 0u;
}

// Taps of seq_bwd_ws_kernel, two 16-bit entries per word (the entries'
// fields fit 16 bits: input rows < 2048, probe columns < 1024, cells < 32,
// which the host checks before it plans this kernel).
struct PTaps {
    int meta;                 // ns | np << 3 | src_edge << 6
    int s01, s23, p01, p23;
    WT_DEV int ns() const { return meta & 7; }
    WT_DEV int np() const { return (meta >> 3) & 7; }
    WT_DEV bool src_edge() const { return (meta >> 6) & 1; }
    WT_DEV int s(int e) const { return ((e < 2 ? s01 : s23) >> (16 * (e & 1))) & 0xffff; }
    WT_DEV int p(int e) const { return ((e < 2 ? p01 : p23) >> (16 * (e & 1))) & 0xffff; }
    WT_DEV int src_i(int e) const { return s(e) & 31; }
    WT_DEV int src_row(int e) const { return s(e) >> 5; }
    WT_DEV int prb_i(int e) const { return p(e) & 31; }
    WT_DEV int prb_col(int e) const { return p(e) >> 6; }
};

WT_DEV PTaps pack_taps(const Taps& t) {
    PTaps q;
    q.meta = t.ns | (t.np << 3) | ((t.src_edge ? 1 : 0) << 6);
    q.s01 = (t.s0 & 0xffff) | (t.s1 << 16);
    q.s23 = (t.s2 & 0xffff) | (t.s3 << 16);
    q.p01 = (t.p0 & 0xffff) | (t.p1 << 16);
    q.p23 = (t.p2 & 0xffff) | (t.p3 << 16);
    return q;
}

// apply_sources and seed_and_read on packed taps.
template <int M>
WT_DEV void apply_sources_p(const FusedParams& P, const PTaps& tp, float (&y)[M],
                            float (&xv)[SRCMAX], int tnext) {
#pragma unroll
    for (int e = 0; e < SRCMAX; ++e)
        if (e < tp.ns()) add_at<M>(y, tp.src_i(e), xv[e]);
    if (tnext >= 0 && tnext < P.steps) {
#pragma unroll
        for (int e = 0; e < SRCMAX; ++e)
            if (e < tp.ns()) xv[e] = __ldg(P.x + (size_t)tp.src_row(e) * P.steps + tnext);
    }
}
template <int M>
WT_DEV void seed_and_read_p(const FusedParams& P, const Geo& g, const PTaps& tp, int t,
                            float (&lam)[M], const float* sr) {
    // a loop on the thread's own count (see seed_and_read)
#pragma unroll 1
    for (int e = 0; e < tp.np(); ++e) add_at<M>(lam, tp.prb_i(e), sr[tp.prb_col(e) * P.PB]);
    if (P.grad_x && tp.ns()) {
#pragma unroll
        for (int e = 0; e < SRCMAX; ++e)
            if (e < tp.ns() && tp.src_row(e) == g.inst)
                P.grad_x[(size_t)g.inst * P.steps + t] = value_at<M>(lam, tp.src_i(e));
    }
}

// One recompute step of group R.  Exchange kx (tile slot RS = kx & 1, halo
// parity RS) holds h_{t-1}; h_t overwrites inout (h_{t-2}), goes to slot
// RS ^ 1 and, when `send`, out as exchange kx + 1.  L receives Lap(h_{t-1}).
// Coefficients cf: [A | Bc | c^2] of the thread's M cells.
template <int M, int ORDER, int RS>
WT_DEV void ws_rec_step(const FusedParams& P, const Geo& g, const Xchg& X, const Lane& ln,
                        const PTaps& tp, int kx, bool send, float (&xv)[SRCMAX], int tnext,
                        const float* cf, const float (&cur)[M], float (&inout)[M],
                        float (&L)[M]) {
    const float* rcol = ln.col0 + RS * ln.tile;
    float* wcol = ln.col0 + (RS ^ 1) * ln.tile;
    // the neighbour columns by 8-byte loads (conflict-free: the tile stride
    // is an odd number of 8-byte words)
    float lf[M], rt[M];
    lds_col<M>(lf, rcol - P.LD);
    lds_col<M>(rt, rcol + P.LD);
    float up = rcol[-1], dn = rcol[M];
    if (ln.rup) up = recv_at(P, X, ln.rup + RS * ln.pstride, kx);
    if (ln.rdn) dn = recv_at(P, X, ln.rdn + RS * ln.pstride, kx);
    auto update = [&](int i, float u, float d) {
        L[i] = lap5<ORDER>(u, lf[i], cur[i], rt[i], d, P.k.lap_w, P.k.lap_w4);
        inout[i] = leapfrog(cf[i], cf[M + i], cf[2 * M + i], P.k.two_over, cur[i], inout[i], L[i]);
    };
    update(0, up, cur[1]);
    update(M - 1, cur[M - 2], dn);
    const unsigned long long tag = (unsigned long long)(uint32_t)(kx + 2) << 32;
    if (send && !tp.src_edge()) {
        if (ln.sup) st_cluster_u64(ln.sup + (RS ^ 1) * ln.pstride, tag | __float_as_uint(inout[0]));
        if (ln.sdn) st_cluster_u64(ln.sdn + (RS ^ 1) * ln.pstride, tag | __float_as_uint(inout[M - 1]));
    }
#pragma unroll
    for (int i = 1; i < M - 1; ++i) update(i, cur[i - 1], cur[i + 1]);
    if (tp.ns()) {
        apply_sources_p<M>(P, tp, inout, xv, tnext);
        if (send && tp.src_edge()) {
            if (ln.sup) st_cluster_u64(ln.sup + (RS ^ 1) * ln.pstride, tag | __float_as_uint(inout[0]));
            if (ln.sdn) st_cluster_u64(ln.sdn + (RS ^ 1) * ln.pstride, tag | __float_as_uint(inout[M - 1]));
        }
    }
    sts_col<M>(wcol, inout);
}

// The adjoint group's ring of stash slices: copies are issued and consumed
// in the same order (descending steps within a segment, segments descending),
// so the k-th copy sits in slot k % nbuf at mbarrier phase parity
// (k / nbuf) & 1.
struct WsRing {
    uint32_t buf, full;     // shared addresses of slot 0 and of its mbarrier
    int slice, nbuf;        // floats per slice, slots
};

// Issue the copy of one stash slice into slot `slot`.
WT_DEV void ws_issue(const WsRing& r, const float* src, int slot) {
    const uint32_t mb = r.full + 8u * (uint32_t)slot;
    const uint32_t bytes = (uint32_t)(r.slice * sizeof(float));
    mbar_arrive_expect_tx(mb, bytes);
    bulk_g2s(r.buf + (uint32_t)(slot * r.slice) * 4u, src, bytes, mb);
}

// Bounded wait for the phase of parity `par` of slot s (tape_wait's rule).
WT_DEV bool ws_wait(const FusedParams& P, const Xchg& X, const WsRing& r, int s, uint32_t par,
                    bool heed_abort = true) {
    const uint32_t mb = r.full + 8u * (uint32_t)s;
    if (mbar_try_wait_parity_cta(mb, par)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait_parity_cta(mb, par)) {
        if (heed_abort && *(volatile int*)X.abort) return false;
        if (global_ns() - t0 > WAIT_LIMIT_NS) {
            atomicExch(P.err, WT_DEVERR_TIMEOUT);
            *(volatile int*)X.abort = 1;
            return false;
        }
    }
    return true;
}

// 8-byte load from a shared address (8-byte aligned).
WT_DEV float2 lds_f32x2(uint32_t a) {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
    return v;
}

// Group R of seq_bwd_ws_kernel: phase p recomputes segment nseg-1-p into
// stash half (segment & 1); one phase barrier per phase.
template <int M, int ORDER>
WT_DEV void ws_recompute_group(const FusedParams& P, const Geo& g, const Xchg& X, const Lane& ln,
                               const PTaps& tp, const float* cf, float* seeds, const float* gxs,
                               int slice, int nseg, int ltid, int NG) {
    constexpr int V = chunk_width<M>();
    const int cstride = NG * V;
    const size_t cta_stash = ((size_t)g.inst * P.C + g.cta) * 2 * P.seg * (size_t)slice;
    int kx = 0;           // exchange index (tile slot and halo parity kx & 1)
    // dL/dx of the segment group A finished in phase q (staged in gxs)
    // (dL/dx is served for one point source: the CTA whose rows hold it)
    auto copy_gx = [&](int q) {
        const int s = nseg - q;
        if (!P.grad_x || s >= nseg || g.cta != (__ldg(P.src_cell) / P.ny) / P.R) return;
        const int t0 = s * P.seg, n = min(P.steps, t0 + P.seg) - t0;
        for (int k = ltid; k < n; k += NG)
            P.grad_x[(size_t)g.inst * P.steps + t0 + k] = gxs[(s & 1) * P.seg + k];
    };
    bool ok = true;
    for (int p = 0; p <= nseg && ok; ++p) {
        if (p > 0) copy_gx(p - 1);
        const int sR = nseg - 1 - p;
        if (sR >= 0) {
            const int t0 = sR * P.seg, t1 = min(P.steps, t0 + P.seg);
            float ya[M], yb[M];   // h_{t0-1}, h_{t0-2}
#pragma unroll
            for (int i = 0; i < M; ++i) ya[i] = yb[i] = 0.f;
            if (sR > 0 && g.colv) {
                const size_t plane = (size_t)P.nx * P.ny, bplane = (size_t)P.batch * plane;
                const float* cp = P.ckpt + (size_t)sR * 2 * bplane + (size_t)g.inst * plane;
#pragma unroll
                for (int i = 0; i < M; ++i) {
                    const int gx = g.gx0 + i;
                    if (gx < P.nx) {
                        const size_t cell = (size_t)gx * P.ny + g.col;
                        ya[i] = __ldcg(cp + cell);
                        yb[i] = __ldcg(cp + bplane + cell);
                    }
                }
            }
            if (g.colv) publish<M>(P, g, X, kx & 1, kx, ya);
            ok = ws_exchange_end(X, WS_BAR_R, NG, 0);
            float xv[SRCMAX];
#pragma unroll
            for (int e = 0; e < SRCMAX; ++e)
                xv[e] = (e < tp.ns()) ? __ldg(P.x + (size_t)tp.src_row(e) * P.steps + t0) : 0.f;
            float* out = P.stash + cta_stash + (size_t)(sR & 1) * P.seg * slice + (size_t)ltid * V;
            for (int t = t0; t < t1 && ok; ++t) {
                float L[M];
                const bool send = t + 1 < t1;
                const int tn = t + 1 < t1 ? t + 1 : -1;
                if (g.colv) {
                    if (kx & 1) {
                        if ((t - t0) & 1) ws_rec_step<M, ORDER, 1>(P, g, X, ln, tp, kx, send, xv, tn, cf, yb, ya, L);
                        else              ws_rec_step<M, ORDER, 1>(P, g, X, ln, tp, kx, send, xv, tn, cf, ya, yb, L);
                    } else {
                        if ((t - t0) & 1) ws_rec_step<M, ORDER, 0>(P, g, X, ln, tp, kx, send, xv, tn, cf, yb, ya, L);
                        else              ws_rec_step<M, ORDER, 0>(P, g, X, ln, tp, kx, send, xv, tn, cf, ya, yb, L);
                    }
                    st_chunks_at<M>(out + (size_t)(t - t0) * slice, cstride, L);
                }
                ++kx;
                if (t + 1 < t1) ok = ws_exchange_end(X, WS_BAR_R, NG, t - t0 + 1);
            }
            // the adjoint seeds of the segment's steps, for group A in the
            // next phase: seeds[sR & 1][t - t0][q], intensity g * (2 y)
            // (autograd's PowBackward), amplitude g
            float* sd = seeds + (size_t)(sR & 1) * P.seg * P.n_prb;
            const int tot = (t1 - t0) * P.n_prb;
            for (int idx = ltid; idx < tot; idx += NG) {
                const int k = idx / P.n_prb, q = idx - k * P.n_prb;
                const size_t oi = ((size_t)g.inst * P.steps + t0 + k) * P.n_prb + q;
                const float gv = P.grad_w ? __ldg(P.grad_w + (size_t)g.inst * P.n_prb + q)
                                          : __ldg(P.grad_out + oi);
                sd[idx] = __ldg(P.prb_kind_col + q) ? fmul(gv, fmul(2.0f, __ldg(P.amp + oi))) : gv;
            }
            // the stash's generic writes before the adjoint group's bulk
            // copies read them (after the phase barrier)
            asm volatile("fence.proxy.async;" ::: "memory");
        }
        __syncthreads();   // phase barrier
        ok = ok && *(volatile int*)X.abort == 0;
    }
    if (ok) copy_gx(nseg);
}

// Group A of seq_bwd_ws_kernel: phase p runs the adjoint steps of segment
// nseg-p (t descending) from stash half (segment & 1), then writes dL/dc.
template <int M, int ORDER>
WT_DEV void ws_adjoint_group(const FusedParams& P, const Geo& g, const Xchg& X, const Lane& ln,
                             const PTaps& tp, const float* cf, const float* seeds, float* gxs,
                             const WsRing& ring, int nseg, int ltid, int NG) {
    constexpr int V = chunk_width<M>();
    const int cstride = NG * V;
    float lam[M], pend[M], acc[M];
#pragma unroll
    for (int i = 0; i < M; ++i) lam[i] = pend[i] = acc[i] = 0.f;
    int u = 0;                        // adjoint steps done (and stash slices consumed)
    int cslot = 0, islot = 0;         // ring slots of the next wait / issue
    uint32_t phase = 0;               // per slot: parity of its next wait
    // the issuer's record per slot: a copy in flight that its own wait has
    // not seen land (inflight), that copy's phase parity (ppar), the parity of
    // the slot's next copy (ipar); it refills a slot only after its own wait
    // saw the slot's copy land, and issues nothing once a wait gave up (or
    // from the missing-slice test hook's step down), so every slot holds at
    // most one copy it has not seen land, and it waits for those before the
    // kernel leaves
    uint32_t inflight = 0, ppar = 0, ipar = 0;
    bool halted = false;
    const bool issuer = ltid == 0;
    auto issue = [&](const float* src, int t) {
        if (halted || t + 1 <= P.skip_slice1 || *(volatile int*)X.abort) {
            halted = true;
            return;
        }
        const uint32_t bit = 1u << islot;
        ws_issue(ring, src, islot);
        inflight |= bit;
        ppar = (ppar & ~bit) | (ipar & bit);
        ipar ^= bit;
        islot = islot + 1 == ring.nbuf ? 0 : islot + 1;
    };
    const bool taps_here = tp.np() || (P.grad_x && tp.ns());
    bool ok = true;
    for (int p = 0; p <= nseg && ok; ++p) {
        const int sA = nseg - p;
        if (sA < nseg) {
            const int t0 = sA * P.seg, t1 = min(P.steps, t0 + P.seg);
            // this CTA's stash half of the segment: step t at (t - t0) slices
            auto stash_at = [&](int t) {
                return P.stash + ((((size_t)g.inst * P.C + g.cta) * 2 + (sA & 1)) * P.seg +
                                  (t - t0)) * (size_t)ring.slice;
            };
            if (issuer) {
                fence_proxy_async_smem();   // the slots' last readers passed the phase barrier
                for (int j = 0; j < ring.nbuf && t1 - 1 - j >= t0; ++j)
                    issue(stash_at(t1 - 1 - j), t1 - 1 - j);
            }
            for (int t = t1 - 1; t >= t0 && ok; --t) {
                const int par = u & 1;
                float* col = ln.col0 + par * ln.tile;
                if (g.colv) {
                    if (taps_here) {
                        // seeds at their cells (descending reference order)
                        // and dL/dx at the source, through the thread's column
                        // of the slot it is about to publish into
#pragma unroll
                        for (int i = 0; i < M; ++i) col[i] = lam[i];
                        const float* sr = seeds + ((size_t)(sA & 1) * P.seg + (t - t0)) * P.n_prb;
#pragma unroll
                        for (int e = 0; e < PRBMAX; ++e)
                            if (e < tp.np()) col[tp.prb_i(e)] = fadd(col[tp.prb_i(e)], sr[tp.prb_col(e)]);
                        if (P.grad_x) {   // one such cell per instance (a point source)
#pragma unroll
                            for (int e = 0; e < SRCMAX; ++e)
                                if (e < tp.ns() && tp.src_row(e) == g.inst)
                                    gxs[(sA & 1) * P.seg + (t - t0)] = col[tp.src_i(e)];
                        }
#pragma unroll
                        for (int i = 0; i < M; ++i) lam[i] = col[i];
                    }
                    // Kg * lambda: sent for the end cells, stored into the tile
                    // column (read back after the barrier, by this thread too)
                    float c2g[M];
#pragma unroll
                    for (int i = 0; i < M; ++i) c2g[i] = fmul(cf[M + i], lam[i]);
                    const unsigned long long tag = (unsigned long long)(uint32_t)(u + 1) << 32;
                    if (ln.sup) st_cluster_u64(ln.sup + par * ln.pstride, tag | __float_as_uint(c2g[0]));
                    if (ln.sdn) st_cluster_u64(ln.sdn + par * ln.pstride, tag | __float_as_uint(c2g[M - 1]));
                    sts_col<M>(col, c2g);
                }
                if (!(ok = ws_exchange_end(X, WS_BAR_A, NG, u))) break;
                // step t+1's slice was read before this barrier: refill its slot
                if (issuer && t < t1 - 1 && t + 1 - ring.nbuf >= t0) {
                    fence_proxy_async_smem();
                    issue(stash_at(t + 1 - ring.nbuf), t + 1 - ring.nbuf);
                }
                if (g.colv) {
                    const int LD = P.LD;
                    const float w = P.k.lap_w, w4 = P.k.lap_w4, dt2 = P.k.dt2;
                    if (ws_wait(P, X, ring, cslot, (phase >> cslot) & 1u) && issuer)
                        inflight &= ~(1u << cslot);
                    // this thread's chunk 0 of the slice (chunk j of 2 cells
                    // at + j * cstride floats)
                    const uint32_t ly = ring.buf + 4u * (uint32_t)(cslot * ring.slice + ltid * V);
                    float own[M];
                    lds_col<M>(own, col);
                    auto update = [&](int i, float up, float dn, float lf, float rt, float Ly) {
                        const float lg = lap5<ORDER>(up, lf, own[i], rt, dn, w, w4);
                        adj_cell_lp(lg, lam[i], Ly, cf[i], cf[2 * M + i], dt2, acc[i], pend[i]);
                    };
                    // cells in pairs (8-byte accesses); the end cells last,
                    // after the halo words
                    const float2 l0 = *reinterpret_cast<const float2*>(col - LD);
                    const float2 r0 = *reinterpret_cast<const float2*>(col + LD);
                    const float2 y0 = lds_f32x2(ly);
                    update(1, own[0], own[2], l0.y, r0.y, y0.y);
#pragma unroll
                    for (int j = 1; j < M / 2 - 1; ++j) {
                        const float2 l = *reinterpret_cast<const float2*>(col - LD + 2 * j);
                        const float2 r = *reinterpret_cast<const float2*>(col + LD + 2 * j);
                        const float2 y = lds_f32x2(ly + 4u * (uint32_t)(j * cstride));
                        update(2 * j, own[2 * j - 1], own[2 * j + 1], l.x, r.x, y.x);
                        update(2 * j + 1, own[2 * j], own[2 * j + 2], l.y, r.y, y.y);
                    }
                    const float2 l9 = *reinterpret_cast<const float2*>(col - LD + M - 2);
                    const float2 r9 = *reinterpret_cast<const float2*>(col + LD + M - 2);
                    const float2 y9 = lds_f32x2(ly + 4u * (uint32_t)((M / 2 - 1) * cstride));
                    update(M - 2, own[M - 3], own[M - 1], l9.x, r9.x, y9.x);
                    float up = col[-1], dn = col[M];
                    if (ln.rup) up = recv_at(P, X, ln.rup + par * ln.pstride, u);
                    if (ln.rdn) dn = recv_at(P, X, ln.rdn + par * ln.pstride, u);
                    update(0, up, own[1], l0.x, r0.x, y0.x);
                    update(M - 1, own[M - 2], dn, l9.y, r9.y, y9.y);
                }
                phase ^= 1u << cslot;
                cslot = cslot + 1 == ring.nbuf ? 0 : cslot + 1;
                ++u;
            }
        }
        __syncthreads();   // phase barrier: the stash half group R filled is complete
        ok = ok && *(volatile int*)X.abort == 0;
    }
    if (issuer && inflight) {
        // leaving early: let the copies still in flight land first (bounded waits)
        for (int sl = 0; sl < ring.nbuf; ++sl)
            if ((inflight >> sl) & 1u) ws_wait(P, X, ring, sl, (ppar >> sl) & 1u, false);
    }
    if (g.colv && ok) {
        // dL/dc = (X1 * Kc) * sum_t Lap * lam (store_dc's arithmetic, X1 from
        // the coefficient words)
        float* o = P.gc_part + (size_t)g.inst * P.nx * P.ny;
#pragma unroll
        for (int i = 0; i < M; ++i) {
            const int gx = g.gx0 + i;
            if (gx < P.nx) {
                const size_t cell = (size_t)gx * P.ny + g.col;
                const float Kc = fmul(fmul(2.0f, __ldg(P.c + P.coef_stride * g.inst + cell)), P.k.dt2);
                o[cell] = fmul(fmul(cf[i], Kc), acc[i]);
            }
        }
    }
}

template <int M, int ORDER>
__global__ void __launch_bounds__(ws_max_threads(M), 1) seq_bwd_ws_kernel(FusedParams P) {
    extern __shared__ __align__(16) float smem[];
    __shared__ int abort_flag;
    const int NG = blockDim.x >> 1;
    const bool grpA = (int)threadIdx.x >= NG;
    const int ltid = grpA ? (int)threadIdx.x - NG : (int)threadIdx.x;
    const Geo g = ws_geo(P, M, ltid);
    const WsLayout lay(P.ny, P.LD, P.NCP, NG, M, P.n_prb, P.seg, P.nbuf);
    constexpr int CS = ws_coef_stride(M);
    // zero both groups' tiles and halo words
    for (int i = threadIdx.x; i < lay.coefR; i += blockDim.x) smem[i] = 0.f;
    if (threadIdx.x == 0) abort_flag = 0;
    Xchg X;
    ws_xchg(X, P, g, smem + (grpA ? 2 * lay.tile : 0), lay.tile,
            reinterpret_cast<unsigned long long*>(smem + (grpA ? lay.haloA : lay.haloR)),
            &abort_flag);
    float* cf = smem + (grpA ? lay.coefA : lay.coefR) + ltid * CS;
    // per-cell coefficients: R [A | Bc | c^2], A [X1 | Kg | Ky2]
#pragma unroll
    for (int i = 0; i < M; ++i) {
        float k0 = 0.f, k1 = 0.f, k2 = 0.f;
        const int gx = g.gx0 + i;
        if (g.colv && gx < P.nx) {
            const size_t cell = P.coef_stride * g.inst + (size_t)gx * P.ny + g.col;
            const float bv = __ldg(P.b + cell), cv = __ldg(P.c + cell);
            if (grpA) {
                const BwdCoef k = bwd_coef(bv, cv, P.k);
                k0 = k.X1; k1 = k.Kg; k2 = k.Ky2;
            } else {
                const FwdCoef f = fwd_coef(bv, cv, P.k);
                k0 = f.A; k1 = f.Bc; k2 = f.c2;
            }
        }
        cf[i] = k0;
        cf[M + i] = k1;
        cf[2 * M + i] = k2;
    }
    PTaps tp;
    {
        Taps t;
        build_taps<M>(P, g, t);
        tp = pack_taps(t);
    }
    float* seeds = smem + lay.seeds;
    WsRing ring;
    ring.buf = smem_addr(smem + lay.ring);
    ring.full = smem_addr(smem) + (uint32_t)lay.mbar;
    ring.slice = NG * M;
    ring.nbuf = P.nbuf;
    if (threadIdx.x == 0) {
        for (int s = 0; s < P.nbuf; ++s) mbar_init(ring.full + 8u * (uint32_t)s, 1);
        fence_mbarrier_init_cluster();
    }
    const Lane ln = make_lane(P, g, X);
    cluster_sync_all();   // zeroed tiles and halo words, coefficients, barriers

    const int nseg = (P.steps + P.seg - 1) / P.seg;
    // each group runs its own loop over the nseg + 1 phases (its state lives
    // only on its own path); both meet at the same phase barriers
    float* gxs = smem + lay.gx;
    if (grpA) ws_adjoint_group<M, ORDER>(P, g, X, ln, tp, cf, seeds, gxs, ring, nseg, ltid, NG);
    else      ws_recompute_group<M, ORDER>(P, g, X, ln, tp, cf, seeds, gxs, ring.slice, nseg, ltid, NG);
    cluster_sync_all();
}

// ============================================================================
// Nonlinear cell, adjoint (tape mode).  Per step s, with g = lam_s and the
// tape's Lap(h1), h1 = h_{s-1} (slot s) and h2 = h_{s-2} (part 1 of slot
// s-1), TimeStep's backward (wavetorch/cell.py:33-42) at the step's own b, c,
// then autograd's chain through b(h1, rho) and c(h1, rho).  lam enters as
// this step's (seeded) lambda and leaves as the next step's, pend carries
// the grad_y2 term one step:
//   dL/dh1  += grad_b * rho * dsat/dh1 + grad_c * (rho c_nl) * 2 h1
//   dL/drho += grad_b * sat + grad_c * h1^2 * c_nl      (direct; accr)
//   dL/dc_lin += grad_c                                  (accc)
// n and X1 = 1 / (b*dt + 1) are the step's coefficients at h1 (formed by the
// caller, or kept from the first half of the step).
WT_DEV void adj_cell_nl(const FusedParams& P, float lg, float& lam, float Ly, float h1, float h2,
                        const NLCoef& n, float X1, float rh, float& accc, float& accr, float& pend) {
    const float dt = P.k.dt, dt2 = P.k.dt2;
    const float v = fadd(fmul(n.b, dt), 1.0f);                          // b*dt + 1
    const float gc = fmul(fmul(X1, fmul(fmul(fmul(2.0f, n.c), dt2), Ly)), lam);
    float gh = fadd(fmul(dt2, lg), fmul(fmul(2.0f, lam), X1));            // grad_y1
    const float g2 = fmul(fmul(fsub(fmul(n.b, dt), 1.0f), X1), lam);      // grad_y2
    accc = fadd(accc, gc);
    float dr = 0.f;
    if (P.b0 > 0.f) {
        const float kb1 = fmul(-fdiv(1.0f, fmul(v, v)), dt);
        const float inner = fsub(fadd(fmul(fmul(fmul(n.c, n.c), dt2), Ly), fmul(2.0f, h1)),
                                 fmul(2.0f, h2));
        const float gb = fmul(fmul(kb1, inner), lam);                     // grad_b
        dr = fmul(gb, n.sat);                                             // b = b_pml + rho*sat
        const float gs = fmul(gb, rh);
        const float a = fabsf(n.q);                                       // sat = b0 / d
        const float d = fadd(1.0f, fmul(a, a));
        const float gd = fdiv(fmul(-gs, P.b0), fmul(d, d));
        const float ga = fmul(gd, fmul(2.0f, a));                         // d = 1 + a^2
        const float gq = n.q > 0.f ? ga : (n.q < 0.f ? -ga : 0.f);        // a = |q|
        gh = fadd(gh, fdiv(gq, P.uth));                                   // q = h1 / uth
    }
    if (P.cnl != 0.f) {                                                   // c = c_lin + (rho c_nl) h1^2
        dr = fadd(dr, fmul(fmul(gc, fmul(h1, h1)), P.cnl));
        gh = fadd(gh, fmul(fmul(gc, fmul(rh, P.cnl)), fmul(2.0f, h1)));
    }
    accr = fadd(accr, dr);
    // the next step's lambda: its grad_y2 term (from the step after this one)
    // plus this step's grad_y1 term, in autograd's order; this step's grad_y2
    // term waits one step
    lam = fadd(pend, gh);
    pend = g2;
}

template <int M, int ORDER, bool CACHE>
__global__ void __launch_bounds__(bwd_max_threads(M), 1) seq_bwd_nl_kernel(FusedParams P) {
    extern __shared__ __align__(16) float smem[];
    __shared__ int abort_flag;
    const Geo g = make_geo(P, M);
    const int tile = (P.ny + 2) * P.LD;
    zero_smem(smem, 2 * tile);
    Xchg X;
    xchg_setup(X, P, g, smem, tile, &abort_flag);
    Taps tp;
    build_taps<M>(P, g, tp);

    const size_t plane = (size_t)P.nx * P.ny;
    float* seeds = smem + 2 * tile + 2 * xchg_words(P.NCP);
    // b_pml, c_lin and rho of the thread's cells: per-thread shared words at
    // constant offsets (stride 3M rounded up to odd: conflict-free), then the
    // tape ring (16-byte aligned)
    constexpr int CS = nl_coef_stride(M, CACHE);
    float* coefs = seeds + ((2 * P.n_prb * P.PB + 3) & ~3);
    float* cw = coefs + threadIdx.x * CS;
    TapeRing ring;
    ring.buf = coefs + ((CS * (int)blockDim.x + 3) & ~3);
    ring.slice = 2 * (int)blockDim.x * M;             // two parts: Lap(h1), h1
    ring.full = reinterpret_cast<unsigned long long*>(ring.buf + (size_t)P.nbuf * ring.slice);
    if (threadIdx.x == 0) {
        for (int s = 0; s < P.nbuf; ++s) mbar_init(smem_addr(ring.full + s), 1);
        fence_mbarrier_init_cluster();
    }
    {
        float bp[M], cl[M], rh[M];
        load_nl_coef<M>(P, g, bp, cl, rh);
#pragma unroll
        for (int i = 0; i < M; ++i) {
            cw[i] = bp[i];
            cw[M + i] = cl[i];
            cw[2 * M + i] = rh[i];
        }
    }
    // adjoint state: lam (this step's lambda before its seeds), pend (the
    // grad_y2 term of the previous step), the two accumulators
    float lam[M], pend[M], accc[M], accr[M];
#pragma unroll
    for (int i = 0; i < M; ++i) lam[i] = pend[i] = accc[i] = accr[i] = 0.f;
    stage_seeds(P, g, seeds, 0);
    cluster_sync_all();

    int lo = P.steps;
    if (threadIdx.x == 0) {
        for (int j = 0; j < P.nbuf && P.steps - 1 - j >= 0; ++j) {
            const int t = P.steps - 1 - j;
            if (tape_issue(P, g, ring, t, t % P.nbuf)) lo = t;
        }
    }
    const Lane ln = make_lane(P, g, X);
    const int part = (int)blockDim.x * M;
    const int stride = (int)blockDim.x * chunk_width<M>();
    const int lane_off = threadIdx.x * chunk_width<M>();
    int slot = (P.steps - 1) % P.nbuf;
    uint32_t phase = 0;
    int pk = 0, pc = 0;
    bool ok = true;
    auto step = [&](auto par, int u) -> bool {
        constexpr int PAR = decltype(par)::value;
        const int t = P.steps - 1 - u;
        float* col = ln.col0 + PAR * ln.tile;
        const int prev = slot == 0 ? P.nbuf - 1 : slot - 1;     // slot of step t-1
        const float* sl = ring.buf + (size_t)slot * ring.slice;
        if (pk == 0 && u + P.PB < P.steps)
            stage_seeds(P, g, seeds, pc + 1);
        if (g.colv) {
            // c2g needs b and c at h1: the step's field first
            tape_wait(P, X, ring, slot, (phase >> slot) & 1u);
            float h1[M];
            ld_chunks_at<M>(h1, sl + part + lane_off, stride);
            if ((tp.wprb || tp.wsrc) && (tp.np || (P.grad_x && tp.ns)))
                seed_and_read<M>(P, g, tp, t, lam, seeds + (size_t)(pc & 1) * P.n_prb * P.PB + pk);
            float c2g[M];
#pragma unroll
            for (int i = 0; i < M; ++i) {
                const NLCoef n = nl_coef(P, cw[i], cw[M + i], cw[2 * M + i], h1[i]);
                const float X1 = fdiv(1.0f, fadd(fmul(n.b, P.k.dt), 1.0f));
                c2g[i] = fmul(fmul(X1, fmul(n.c, n.c)), lam[i]);   // (b*dt+1)^-1 * c^2 * g
                if constexpr (CACHE) {      // the divisions' results for the second half
                    cw[3 * M + i] = X1;
                    cw[4 * M + i] = n.q;
                    cw[5 * M + i] = n.sat;
                }
            }
            const unsigned long long tag = (unsigned long long)(uint32_t)(u + 1) << 32;
            if (ln.sup) st_cluster_u64(ln.sup + PAR * ln.pstride, tag | __float_as_uint(c2g[0]));
            if (ln.sdn) st_cluster_u64(ln.sdn + PAR * ln.pstride, tag | __float_as_uint(c2g[M - 1]));
            sts_col<M>(col, c2g);
        }
        if (!exchange_end(X, u)) return false;
        // (no refill once a wait gave up, as in the linear tape adjoint)
        if (threadIdx.x == 0 && u > 0 && t + 1 - P.nbuf >= 0 && *(volatile int*)X.abort == 0) {
            fence_proxy_async_smem();
            if (tape_issue(P, g, ring, t + 1 - P.nbuf, slot + 1 == P.nbuf ? 0 : slot + 1))
                lo = t + 1 - P.nbuf;
        }
        if (g.colv) {
            // Kg*lambda of the thread's own cells and its neighbours' from
            // the tile; the step's tape values from the ring again
            Column<M> c;
            lds_col<M>(c.lf, col - P.LD);
            lds_col<M>(c.rt, col + P.LD);
            c.up = col[-1];
            c.dn = col[M];
            float c2g[M], h1[M], h2[M], Ly[M];
            lds_col<M>(c2g, col);
            ld_chunks_at<M>(h1, sl + part + lane_off, stride);
            ld_chunks_at<M>(Ly, sl + lane_off, stride);
            if (t > 0) {
                tape_wait(P, X, ring, prev, (phase >> prev) & 1u);
                ld_chunks_at<M>(h2, ring.buf + (size_t)prev * ring.slice + part + lane_off, stride);
            } else {
#pragma unroll
                for (int i = 0; i < M; ++i) h2[i] = 0.f;
            }
            phase ^= 1u << slot;
            // the step's coefficients at h1, as in the first half (kept from it
            // with CACHE: the same operations on the same values)
            auto cell = [&](int i, float lg) {
                NLCoef n;
                float X1;
                if constexpr (CACHE) {
                    X1 = cw[3 * M + i];
                    n.q = cw[4 * M + i];
                    n.sat = cw[5 * M + i];
                    n.b = P.b0 > 0.f ? fadd(cw[i], fmul(cw[2 * M + i], n.sat)) : cw[i];
                    n.c = P.cnl != 0.f ? fadd(cw[M + i], fmul(fmul(cw[2 * M + i], P.cnl), fmul(h1[i], h1[i])))
                                       : cw[M + i];
                } else {
                    n = nl_coef(P, cw[i], cw[M + i], cw[2 * M + i], h1[i]);
                    X1 = fdiv(1.0f, fadd(fmul(n.b, P.k.dt), 1.0f));
                }
                adj_cell_nl(P, lg, lam[i], Ly[i], h1[i], h2[i], n, X1, cw[2 * M + i], accc[i], accr[i],
                            pend[i]);
            };
#pragma unroll
            for (int i = 1; i < M - 1; ++i) cell(i, lap_cell<M, ORDER>(P, c, c2g, i));
            if (ln.rup) c.up = recv_at(P, X, ln.rup + PAR * ln.pstride, u);
            if (ln.rdn) c.dn = recv_at(P, X, ln.rdn + PAR * ln.pstride, u);
            cell(0, lap_cell<M, ORDER>(P, c, c2g, 0));
            cell(M - 1, lap_cell<M, ORDER>(P, c, c2g, M - 1));
        }
        slot = prev;
        if (++pk == P.PB) { pk = 0; ++pc; }
        return true;
    };
    for (int u = 0; u < P.steps && ok; ++u)
        ok = (u & 1) ? step(std::integral_constant<int, 1>{}, u)
                     : step(std::integral_constant<int, 0>{}, u);
    if (!ok && threadIdx.x == 0) {
        for (int s = lo; s < lo + P.nbuf && s < P.steps; ++s)
            tape_wait(P, X, ring, s % P.nbuf, (uint32_t)(((P.steps - 1 - s) / P.nbuf) & 1), false);
    }
    if (g.colv && ok) {
        float* oc = P.gc_part + (size_t)g.inst * plane;
        float* orh = P.grho_part + (size_t)g.inst * plane;
#pragma unroll
        for (int i = 0; i < M; ++i) {
            int gx = g.gx0 + i;
            if (gx < P.nx) {
                oc[(size_t)gx * P.ny + g.col] = accc[i];
                orh[(size_t)gx * P.ny + g.col] = accr[i];
            }
        }
    }
    cluster_sync_all();
}

}  // namespace wt

// ---------------------------------------------------------------------------
// Host side: configuration and launch.
// The file is compiled as four parts so that the kernels of the three
// Laplacian orders build in parallel: WT_FUSED_PART 0 holds the planner, the
// small kernels and the dispatch by order; parts 1, 2 and 3 instantiate the
// sequence kernels of WT_LAP_SEQ, WT_LAP_SEQ | WT_LAP_UNIT and
// WT_LAP_PAIRED | WT_LAP_UNIT.  Without WT_FUSED_PART the file holds all.
#ifndef WT_FUSED_PART
#define WT_FUSED_PART -1
#endif
#define WT_FUSED_HAS(part) (WT_FUSED_PART == -1 || WT_FUSED_PART == (part))

#if WT_FUSED_HAS(0)
// Column stride of a tile: room for OFF + rows + 1 floats, and conflict-free
// column accesses of the width the M-cell strips use (float4: LD/4 odd;
// float2: LD/2 odd; scalar: LD odd).
static int tile_ld(int rows, int M) {
    int ld = rows + wt::OFF + 1;
    if (M % 4 == 0) { while (ld % 8 != 4) ++ld; }
    else if (M % 2 == 0) { while (ld % 4 != 2) ++ld; }
    else { while (ld % 2 != 1) ++ld; }
    return ld;
}

// Strip height with the fewest padding rows for R rows per CTA (ties: the
// first in `Ms`), within the thread budget of that height.
static int pick_strip(int nx, int C, int NCP, const int* Ms, int nM, bool fwd, bool allow_empty) {
    int best = -1, best_pad = 1 << 30;
    for (int mi = 0; mi < nM; ++mi) {
        int M = Ms[mi];
        int rows = (nx + C - 1) / C;
        int R = ((rows + M - 1) / M) * M;
        if (!allow_empty && (C - 1) * R >= nx) continue;   // a CTA of padding rows only
        if ((R / M) * NCP > (fwd ? wt::fwd_max_threads(M) : wt::bwd_max_threads(M))) continue;
        int pad = C * R - nx;
        if (pad < best_pad) { best_pad = pad; best = M; }
    }
    return best;
}

// Pick the cluster size C and the strip heights (10-cell strips where they
// fit: per-step overhead amortised over more cells); then the checkpoint
// interval: the largest stash that fits in shared memory next to the two
// tiles, the halo words and the probe ring buffers (at least 4 steps), else
// a sqrt(T) interval with the stash in global memory.
int wt_fused_plan(int nx, int ny, int steps, int n_prb, int cluster_req, int seg_req,
                  WtFusedLaunch* L) {
    const int NCP = ((ny + 31) / 32) * 32;
    const int Mb[3] = {10, 8, 4};
    const int Mf[7] = {10, 15, 30, 8, 6, 5, 4};
    const int Cs[5] = {4, 2, 8, 1, 16};
    const size_t SMEM_MAX = 227 * 1024 - 64;   // dynamic smem per CTA (static: 28 B)
    const int PB = n_prb > 0 ? std::max(1, std::min(32, 2048 / n_prb)) : 32;
    auto r16 = [](size_t v) { return (v + 15) / 16 * 16; };
    const size_t aux_fwd = r16((size_t)(2 * n_prb * PB + 3 * n_prb) * 4);   // ring, owners, sums
    const size_t aux_bwd = r16((size_t)(2 * n_prb * PB) * 4);
    for (int ci = 0; ci < 5; ++ci) {
        int C = Cs[ci];
        if (cluster_req > 0 && C != cluster_req) continue;
        // 16 CTAs (a non-portable cluster size) only for grids the portable
        // sizes cannot hold; there the last CTAs may hold padding rows only
        const bool big = C > 8;
        const int M = pick_strip(nx, C, NCP, Mb, 3, false, big);
        const int fM = pick_strip(nx, C, NCP, Mf, 7, true, big);
        if (M < 0 || fM < 0) continue;
        const int rows = (nx + C - 1) / C;
        const int R = ((rows + M - 1) / M) * M, fR = ((rows + fM - 1) / fM) * fM;
        const int LD = tile_ld(R, M), fLD = tile_ld(fR, fM);
        // two tile slots + the halo words [2 parities][up, down][NCP]
        const size_t words = (size_t)wt::xchg_words(NCP) * 8;
        const size_t tiles = 2 * (size_t)(ny + 2) * LD * sizeof(float) + words;
        const size_t ftiles = 2 * (size_t)(ny + 2) * fLD * sizeof(float) + words;
        if (tiles + aux_bwd > SMEM_MAX || ftiles + aux_fwd > SMEM_MAX) continue;
        L->C = C; L->NCP = NCP; L->PB = PB;
        L->M = M; L->R = R; L->S = R / M; L->LD = LD; L->threads = (R / M) * NCP;
        L->fM = fM; L->fR = fR; L->fS = fR / fM; L->fLD = fLD; L->fthreads = (fR / fM) * NCP;
        L->smem_fwd = ftiles + aux_fwd;
        const size_t per_step = (size_t)M * L->threads * sizeof(float);
        const int fit = (int)((SMEM_MAX - tiles - aux_bwd) / per_step);
        int seg = seg_req > 0 ? seg_req : (fit >= 4 ? fit : (int)std::ceil(std::sqrt((double)steps)));
        seg = std::max(1, std::min(seg, steps));
        L->seg = seg;
        L->stash_smem = seg <= fit;
        L->smem_bwd = tiles + aux_bwd + (L->stash_smem ? (size_t)seg * per_step : 0);
        // tape mode: both kernels on the adjoint's strips; the adjoint keeps
        // a ring of up to 8 slices (threads x M floats) plus one mbarrier per
        // slice; one slice must stay below the mbarrier's transaction-count
        // limit (2^20 - 1 bytes)
        const size_t slice = per_step;
        const int tfit = slice < (1u << 20) ? (int)((SMEM_MAX - tiles - aux_bwd) / (slice + 8)) : 0;
        L->nbuf = std::min(8, tfit);
        L->smem_tape = tiles + aux_bwd + (size_t)L->nbuf * (slice + 8);
        L->smem_fwd_tape = tiles + aux_fwd;
        L->smem_bwd_base = tiles + aux_bwd;
        // the nonlinear adjoint keeps its cells' b_pml, c_lin, rho in shared
        // memory before the ring, and the step's X1, q, sat between the two
        // halves of a step where that leaves the ring 3 slots
        const size_t nl_room = SMEM_MAX - tiles - aux_bwd;
        auto nl_fit = [&](bool cache, size_t& words) {
            words = r16((size_t)wt::nl_coef_stride(M, cache) * L->threads * sizeof(float));
            const int n = 2 * slice < (1u << 20) && nl_room > words
                              ? (int)((nl_room - words) / (2 * slice + 8)) : 0;
            return std::min(8, n);
        };
        L->nl_cache = nl_fit(true, L->smem_nl_coef) >= 3;
        L->nbuf_nl = nl_fit(L->nl_cache != 0, L->smem_nl_coef);
        if (L->smem_fwd_tape > SMEM_MAX || L->threads > wt::fwd_max_threads(M)) L->nbuf = 0;
        // checkpoints with the recompute beside the adjoint: 10-cell strips
        // (two groups of at most 384 threads share the register file); its
        // ring and shared memory are sized once the interval is known
        // (wt_ws_plan)
        L->nbuf_ws = 0;
        L->smem_ws = 0;
        L->ws = 0;
        return 0;
    }
    return WT_ERR_UNSUPPORTED;
}

int wt_ws_plan(int batch, int ny, int n_prb, WtFusedLaunch* L) {
    const size_t SMEM_MAX = 227 * 1024 - 64;
    const size_t slice = (size_t)L->M * L->threads * sizeof(float);
    // packed taps (PTaps): input rows < 2048, probe columns < 1024
    if (L->M != 10 || 2 * L->threads > wt::ws_max_threads(L->M) || slice >= (1u << 20) ||
        batch >= 2048 || n_prb >= 1024 || L->seg < 1)
        return WT_ERR_UNSUPPORTED;
    for (int nb = 4; nb >= 2; --nb) {
        const wt::WsLayout lay(ny, L->LD, L->NCP, L->threads, L->M, n_prb, L->seg, nb);
        if (lay.bytes(nb) <= SMEM_MAX) {
            L->nbuf_ws = nb;
            L->smem_ws = lay.bytes(nb);
            return WT_OK;
        }
    }
    return WT_ERR_UNSUPPORTED;
}

// Kahan-compensated time sums of the probe series: one thread per
// (instance, column), sequential over t.
__global__ void probe_sum_kernel(int batch, int steps, int n_prb, const float* __restrict__ out,
                                 float* __restrict__ sum) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= batch * n_prb) return;
    const int b = idx / n_prb, q = idx - b * n_prb;
    const float* p = out + (size_t)b * steps * n_prb + q;
    float s = 0.f, comp = 0.f;
    for (int t = 0; t < steps; ++t) {
        float y = fsub(__ldg(p + (size_t)t * n_prb), comp);
        float tk = fadd(s, y);
        comp = fsub(fsub(tk, s), y);
        s = tk;
    }
    sum[idx] = s;
}

int wt_launch_probe_sum(int batch, int steps, int n_prb, const float* out, float* sum,
                        cudaStream_t st) {
    const int n = batch * n_prb;
    if (n == 0) return WT_OK;
    probe_sum_kernel<<<(n + 127) / 128, 128, 0, st>>>(batch, steps, n_prb, out, sum);
    wt_count_launches(1);
    return wt_cuda_status(cudaGetLastError());
}

// The reference's training loss on the time-summed probe outputs
// (wavetorch/train.py:61-62, utils.py:35-36), and its gradient:
//   p = I / sum_q I,  loss = mean_b CE(p_b, label_b) = mean_b (lse(p_b) - p_b[label])
//   dL/dp = (softmax(p) - onehot) / B,  dL/dI_k = (dL/dp_k - sum_j dL/dp_j p_j) / sum_q I
// One block; thread b handles instance b, the batch mean is a shared sum.
__global__ void loss_ce_np_kernel(int batch, int n_prb, const float* __restrict__ sum,
                                  const int64_t* __restrict__ labels, float* __restrict__ loss,
                                  float* __restrict__ grad_sum) {
    __shared__ float part[256];
    float acc = 0.f;
    for (int bi = threadIdx.x; bi < batch; bi += blockDim.x) {
        const float* I = sum + (size_t)bi * n_prb;
        float* gI = grad_sum + (size_t)bi * n_prb;
        float S = 0.f;
        for (int q = 0; q < n_prb; ++q) S = fadd(S, I[q]);
        float m = -INFINITY;
        for (int q = 0; q < n_prb; ++q) m = fmaxf(m, fdiv(I[q], S));
        float se = 0.f;
        for (int q = 0; q < n_prb; ++q) se = fadd(se, expf(fsub(fdiv(I[q], S), m)));
        const float lse = fadd(m, logf(se));
        const int lab = (int)labels[bi];
        const float pl = (lab >= 0 && lab < n_prb) ? fdiv(I[lab], S) : 0.f;
        acc = fadd(acc, fsub(lse, pl));
        float dot = 0.f;
        for (int q = 0; q < n_prb; ++q) {      // dL/dp into grad_sum first
            const float p = fdiv(I[q], S);
            const float dp = fdiv(fsub(fdiv(expf(fsub(p, m)), se), q == lab ? 1.f : 0.f), (float)batch);
            gI[q] = dp;
            dot = fadd(dot, fmul(dp, p));
        }
        for (int q = 0; q < n_prb; ++q) gI[q] = fdiv(fsub(gI[q], dot), S);
    }
    part[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int i = 0; i < (int)blockDim.x; ++i) t = fadd(t, part[i]);
        *loss = fdiv(t, (float)batch);
    }
}

int wt_launch_loss_ce_np(int batch, int n_prb, const float* sum, const int64_t* labels,
                         float* loss, float* grad_sum, cudaStream_t st) {
    loss_ce_np_kernel<<<1, 256, 0, st>>>(batch, n_prb, sum, labels, loss, grad_sum);
    wt_count_launches(1);
    return wt_cuda_status(cudaGetLastError());
}

#endif  // part 0

#if !WT_FUSED_HAS(0) || WT_FUSED_PART == -1
// Kernel attributes (dynamic shared memory size, non-portable cluster size)
// are set once per kernel and device, and raised when a launch needs more:
// not repeated on every launch, which keeps launches cheap on the host and
// free of extra runtime calls while a stream is being captured.
static int ensure_attributes(void (*kern)(wt::FusedParams), size_t smem, bool nonportable) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return wt_cuda_status(e);
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, std::pair<size_t, bool>> done;
    std::lock_guard<std::mutex> lock(mu);
    auto& v = done[{dev, reinterpret_cast<const void*>(kern)}];
    if (v.first < smem) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return wt_cuda_status(e);
        v.first = smem;
    }
    if (nonportable && !v.second) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return wt_cuda_status(e);
        v.second = true;
    }
    return WT_OK;
}

static int launch_kernel(void (*kern)(wt::FusedParams), const wt::FusedParams& P, int C,
                         int threads, size_t smem, cudaStream_t st) {
    int rc = ensure_attributes(kern, smem, C > 8);
    if (rc) return rc;
    cudaError_t e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C * P.batch, 1, 1);
    cfg.blockDim = dim3(threads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, kern, P);
    wt_count_launches(1);
    return wt_cuda_status(e);
}

template <int M, int ORDER>
static int launch_fwd(const wt::FusedParams& P0, const WtFusedLaunch& L, cudaStream_t st) {
    wt::FusedParams P = P0;
    P.R = L.fR;
    P.LD = L.fLD;
    return launch_kernel(P.fields ? wt::seq_fwd_fused_kernel<M, ORDER, true>
                                  : wt::seq_fwd_fused_kernel<M, ORDER, false>,
                         P, L.C, L.fthreads, L.smem_fwd, st);
}

template <int M, int ORDER>
static int launch_bwd(const wt::FusedParams& P0, const WtFusedLaunch& L, cudaStream_t st) {
    wt::FusedParams P = P0;
    P.R = L.R;
    P.LD = L.LD;
    if (P.lap)
        return launch_kernel(wt::seq_bwd_tape_kernel<M, ORDER>, P, L.C, L.threads, L.smem_tape, st);
    if constexpr (M == 10) {
        if (L.ws) {
            P.nbuf = L.nbuf_ws;
            return launch_kernel(wt::seq_bwd_ws_kernel<M, ORDER>, P, L.C, 2 * L.threads, L.smem_ws, st);
        }
    }
    return launch_kernel(wt::seq_bwd_fused_kernel<M, ORDER>, P, L.C, L.threads, L.smem_bwd, st);
}

template <int ORDER>
static int launch_order(bool fwd, const wt::FusedParams& P, const WtFusedLaunch& L, cudaStream_t st) {
    if (fwd) {
        switch (L.fM) {
            case 30: return launch_fwd<30, ORDER>(P, L, st);
            case 15: return launch_fwd<15, ORDER>(P, L, st);
            case 10: return launch_fwd<10, ORDER>(P, L, st);
            case 8: return launch_fwd<8, ORDER>(P, L, st);
            case 6: return launch_fwd<6, ORDER>(P, L, st);
            case 5: return launch_fwd<5, ORDER>(P, L, st);
            case 4: return launch_fwd<4, ORDER>(P, L, st);
        }
    } else {
        switch (L.M) {
            case 10: return launch_bwd<10, ORDER>(P, L, st);
            case 8: return launch_bwd<8, ORDER>(P, L, st);
            case 4: return launch_bwd<4, ORDER>(P, L, st);
        }
    }
    return WT_ERR_UNSUPPORTED;
}

template <int M, int ORDER>
static int launch_nl(bool fwd, const wt::FusedParams& P0, const WtFusedLaunch& L, cudaStream_t st) {
    wt::FusedParams P = P0;
    P.R = L.R;
    P.LD = L.LD;
    if (fwd) return launch_kernel(wt::seq_fwd_nl_kernel<M, ORDER>, P, L.C, L.threads, L.smem_fwd_tape, st);
    const size_t smem = L.smem_bwd_base + L.smem_nl_coef +
                        (size_t)P.nbuf * (2 * (size_t)L.threads * M * sizeof(float) + 8);
    if (L.nl_cache) return launch_kernel(wt::seq_bwd_nl_kernel<M, ORDER, true>, P, L.C, L.threads, smem, st);
    return launch_kernel(wt::seq_bwd_nl_kernel<M, ORDER, false>, P, L.C, L.threads, smem, st);
}

template <int ORDER>
static int launch_nl_order(bool fwd, const wt::FusedParams& P, const WtFusedLaunch& L, cudaStream_t st) {
    switch (L.M) {
        case 10: return launch_nl<10, ORDER>(fwd, P, L, st);
        case 8: return launch_nl<8, ORDER>(fwd, P, L, st);
        case 4: return launch_nl<4, ORDER>(fwd, P, L, st);
    }
    return WT_ERR_UNSUPPORTED;
}

#endif  // kernel parts

#define WT_FUSED_ORDER_ENTRY(part, name, order)                                                  \
    int wt_launch_fused_##name(bool fwd, const wt::FusedParams& P, const WtFusedLaunch& L,       \
                               cudaStream_t st) {                                                \
        return launch_order<order>(fwd, P, L, st);                                               \
    }                                                                                            \
    int wt_launch_fused_nl_##name(bool fwd, const wt::FusedParams& P, const WtFusedLaunch& L,    \
                                  cudaStream_t st) {                                             \
        return launch_nl_order<order>(fwd, P, L, st);                                            \
    }
#if WT_FUSED_HAS(1)
WT_FUSED_ORDER_ENTRY(1, seq, WT_LAP_SEQ)
#endif
#if WT_FUSED_HAS(2)
WT_FUSED_ORDER_ENTRY(2, seq_unit, WT_LAP_SEQ | WT_LAP_UNIT)
#endif
#if WT_FUSED_HAS(3)
WT_FUSED_ORDER_ENTRY(3, paired_unit, WT_LAP_PAIRED | WT_LAP_UNIT)
#endif

#if WT_FUSED_HAS(0)
int wt_launch_fused_nl(bool fwd, const wt::FusedParams& P, const WtFusedLaunch& L, cudaStream_t st) {
    switch (P.k.lap_order) {
        case WT_LAP_SEQ: return wt_launch_fused_nl_seq(fwd, P, L, st);
        case WT_LAP_SEQ | WT_LAP_UNIT: return wt_launch_fused_nl_seq_unit(fwd, P, L, st);
        case WT_LAP_PAIRED | WT_LAP_UNIT: return wt_launch_fused_nl_paired_unit(fwd, P, L, st);
    }
    return WT_ERR_INVALID;
}

int wt_launch_fused(bool fwd, const wt::FusedParams& P, const WtFusedLaunch& L, cudaStream_t st) {
    switch (P.k.lap_order) {
        case WT_LAP_SEQ: return wt_launch_fused_seq(fwd, P, L, st);
        case WT_LAP_SEQ | WT_LAP_UNIT: return wt_launch_fused_seq_unit(fwd, P, L, st);
        case WT_LAP_PAIRED | WT_LAP_UNIT: return wt_launch_fused_paired_unit(fwd, P, L, st);
    }
    return WT_ERR_INVALID;
}
#endif
