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
// Exchange.  Every step each thread writes its new values into a column-major
// shared-memory tile  F[col+1][OFF + row]  (the tile carries zero columns at
// y = -1 and y = ny, and one halo row above and below); the first and last
// rows of the CTA are also pushed into the neighbouring CTAs' halo rows with
// st.shared::cluster (DSMEM).  One barrier.cluster (release/acquire) per step
// publishes both; the tile is double buffered, so one barrier suffices.
// Up/down neighbours inside a strip come from registers, left/right columns
// and the strip ends from the tile (float4 loads, conflict-free because the
// column stride LD is 4 mod 8 floats).
//
// Adjoint.  The forward stores the pair (h_{t-1}, h_{t-2}) every `seg` steps.
// The adjoint walks the segments backwards: it reloads the checkpoint,
// recomputes the segment's forward steps to rebuild Lap(h_{t-1}) for each of
// its steps (the "stash"), then runs the segment's adjoint steps from the
// stash.  Adjoint state per cell (pending grad_y1/grad_y2 terms and the
// running dL/dc sum of this instance) stays in registers across segments.
#include "internal.cuh"

namespace wt {

constexpr int OFF = 4;       // first own row in a tile column (16-byte aligned)
constexpr int SRCMAX = 4;    // source entries one thread may own
constexpr int PRBMAX = 4;    // probe entries one thread may own

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

// Thread geometry shared by both kernels.
struct Geo {
    int inst, cta, col, strip, xl0, gx0;
    bool colv;          // column inside the grid
    uint32_t up_rank, dn_rank;
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
    g.colv = g.col < P.ny;
    g.has_up = g.cta > 0;
    g.has_dn = g.cta + 1 < P.C;
    g.up_rank = g.cta - 1;
    g.dn_rank = g.cta + 1;
    return g;
}

// Write the thread's M new values into tile `buf` and push the CTA boundary
// rows into the neighbours' halo rows.
template <int M>
WT_DEV void publish(const FusedParams& P, const Geo& g, float* buf, const float (&v)[M],
                    int S) {
    if (!g.colv) return;
    float* colp = buf + (size_t)(g.col + 1) * P.LD + OFF;
    sts_col<M>(colp + g.xl0, v);
    if (g.strip == 0 && g.has_up) {
        // my row 0 is the up-neighbour CTA's halo row R
        uint32_t a = map_shared_rank(colp + P.R, g.up_rank);
        st_cluster_f32(a, v[0]);
    }
    if (g.strip == S - 1 && g.has_dn) {
        // my row R-1 is the down-neighbour CTA's halo row -1
        uint32_t a = map_shared_rank(colp - 1, g.dn_rank);
        st_cluster_f32(a, v[M - 1]);
    }
}

// Laplacian of the thread's M cells from registers (center) + tile (rest).
template <int M, int ORDER>
WT_DEV void strip_lap(const FusedParams& P, const Geo& g, const float* buf, const float (&ctr)[M],
                      float (&L)[M]) {
    const float* colp = buf + (size_t)(g.col + 1) * P.LD + OFF + g.xl0;
    float lf[M], rt[M];
    lds_col<M>(lf, colp - P.LD);
    lds_col<M>(rt, colp + P.LD);
    const float up = colp[-1];
    const float dn = colp[M];
#pragma unroll
    for (int i = 0; i < M; ++i) {
        float u = i == 0 ? up : ctr[i - 1];
        float d = i == M - 1 ? dn : ctr[i + 1];
        L[i] = lap5<ORDER>(u, lf[i], ctr[i], rt[i], d, P.k.lap_w, P.k.lap_w4);
    }
}

WT_DEV void zero_smem(float* s, int n) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) s[i] = 0.f;
}

// Per-thread source list (table order) and probe list (descending order).
template <int M>
struct Taps {
    int ns, np;
    int s_i[SRCMAX], s_row[SRCMAX];
    int p_i[PRBMAX], p_kind[PRBMAX], p_col[PRBMAX];
};

template <int M>
WT_DEV void build_taps(const FusedParams& P, const Geo& g, Taps<M>& tp) {
    tp.ns = 0;
    tp.np = 0;
#pragma unroll
    for (int j = 0; j < SRCMAX; ++j) tp.s_i[j] = tp.s_row[j] = 0;
#pragma unroll
    for (int j = 0; j < PRBMAX; ++j) tp.p_i[j] = tp.p_kind[j] = tp.p_col[j] = 0;
    if (!g.colv) return;
    // (writes go through unrolled predicated stores so the lists stay in
    // registers instead of local memory)
    for (int e = 0; e < P.n_src; ++e) {
        int cell = __ldg(P.src_cell + e);
        int cx = cell / P.ny, cy = cell - cx * P.ny;
        int i = cx - g.gx0;
        if (cy == g.col && i >= 0 && i < M) {
            int row = __ldg(P.src_row + e);
            row = row < 0 ? g.inst : row;
            if (tp.ns >= SRCMAX) { atomicExch(P.err, WT_DEVERR_BOUNDS); continue; }
#pragma unroll
            for (int j = 0; j < SRCMAX; ++j)
                if (j == tp.ns) { tp.s_i[j] = i; tp.s_row[j] = row; }
            ++tp.ns;
        }
    }
    for (int e = 0; e < P.n_prb; ++e) {
        int cell = __ldg(P.prb_cell + e);
        int cx = cell / P.ny, cy = cell - cx * P.ny;
        int i = cx - g.gx0;
        if (cy == g.col && i >= 0 && i < M) {
            int kind = __ldg(P.prb_kind + e), col = __ldg(P.prb_col + e);
            if (tp.np >= PRBMAX) { atomicExch(P.err, WT_DEVERR_BOUNDS); continue; }
#pragma unroll
            for (int j = 0; j < PRBMAX; ++j)
                if (j == tp.np) { tp.p_i[j] = i; tp.p_kind[j] = kind; tp.p_col[j] = col; }
            ++tp.np;
        }
    }
}

// select v[i] for a runtime i without dynamic register indexing
template <int M>
WT_DEV float pick(const float (&v)[M], int i) {
    float r = 0.f;
#pragma unroll
    for (int j = 0; j < M; ++j) r = (j == i) ? v[j] : r;
    return r;
}
template <int M>
WT_DEV void add_at(float (&v)[M], int i, float a) {
#pragma unroll
    for (int j = 0; j < M; ++j)
        if (j == i) v[j] = fadd(v[j], a);
}

// One forward step for the thread's cells: Laplacian, update, sources.
template <int M, int ORDER>
WT_DEV void fwd_cells(const FusedParams& P, const Geo& g, const float* buf, const float (&A)[M],
                      const float (&Bc)[M], const float (&C2)[M], float (&y1)[M],
                      float (&y2)[M], float (&yn)[M], float (&L)[M], const Taps<M>& tp,
                      const float (&xv)[SRCMAX]) {
    strip_lap<M, ORDER>(P, g, buf, y1, L);
#pragma unroll
    for (int i = 0; i < M; ++i) yn[i] = leapfrog(A[i], Bc[i], C2[i], P.k.two_over, y1[i], y2[i], L[i]);
#pragma unroll
    for (int e = 0; e < SRCMAX; ++e)
        if (e < tp.ns) add_at<M>(yn, tp.s_i[e], xv[e]);
}

// ============================================================================
// Forward
template <int M, int ORDER>
__global__ void __launch_bounds__(512, 1) seq_fwd_fused_kernel(FusedParams P) {
    extern __shared__ __align__(16) float smem[];
    const Geo g = make_geo(P, M);
    const int S = P.R / M;
    const int tile = (P.ny + 2) * P.LD;
    float* F0 = smem;
    float* F1 = smem + tile;
    zero_smem(smem, 2 * tile);

    float A[M], Bc[M], C2[M], y1[M], y2[M];
#pragma unroll
    for (int i = 0; i < M; ++i) {
        A[i] = Bc[i] = C2[i] = 0.f;
        y1[i] = y2[i] = 0.f;
        int gx = g.gx0 + i;
        if (g.colv && gx < P.nx) {
            size_t cell = (size_t)gx * P.ny + g.col;
            FwdCoef f = fwd_coef(__ldg(P.b + cell), __ldg(P.c + cell), P.k);
            A[i] = f.A; Bc[i] = f.Bc; C2[i] = f.c2;
        }
    }
    Taps<M> tp;
    build_taps<M>(P, g, tp);
    float psum[PRBMAX], pcmp[PRBMAX];
#pragma unroll
    for (int e = 0; e < PRBMAX; ++e) psum[e] = pcmp[e] = 0.f;
    float xv[SRCMAX];
#pragma unroll
    for (int e = 0; e < SRCMAX; ++e) xv[e] = 0.f;
#pragma unroll
    for (int e = 0; e < SRCMAX; ++e)
        if (e < tp.ns) xv[e] = __ldg(P.x + (size_t)tp.s_row[e] * P.steps);

    const size_t plane = (size_t)P.nx * P.ny;
    const size_t bplane = (size_t)P.batch * plane;
    cluster_sync_all();

    for (int t = 0; t < P.steps; ++t) {
        const float* buf = (t & 1) ? F1 : F0;
        float* nbuf = (t & 1) ? F0 : F1;
        if (t > 0 && t % P.seg == 0 && g.colv) {
            // checkpoint (h_{t-1}, h_{t-2}) for the adjoint's segment t/seg
            float* ck = P.ckpt + (size_t)(t / P.seg) * 2 * bplane + (size_t)g.inst * plane;
#pragma unroll
            for (int i = 0; i < M; ++i) {
                int gx = g.gx0 + i;
                if (gx < P.nx) {
                    size_t cell = (size_t)gx * P.ny + g.col;
                    ck[cell] = y1[i];
                    ck[bplane + cell] = y2[i];
                }
            }
        }
        float yn[M], L[M];
        if (g.colv) {
            float xc[SRCMAX];
#pragma unroll
            for (int e = 0; e < SRCMAX; ++e) xc[e] = xv[e];
            // prefetch next step's inputs
            if (t + 1 < P.steps) {
#pragma unroll
                for (int e = 0; e < SRCMAX; ++e)
                    if (e < tp.ns) xv[e] = __ldg(P.x + (size_t)tp.s_row[e] * P.steps + t + 1);
            }
            fwd_cells<M, ORDER>(P, g, buf, A, Bc, C2, y1, y2, yn, L, tp, xc);
#pragma unroll
            for (int e = 0; e < PRBMAX; ++e) {
                if (e >= tp.np) break;
                float v = pick<M>(yn, tp.p_i[e]);
                float o = tp.p_kind[e] ? fmul(v, v) : v;
                size_t oi = ((size_t)g.inst * P.steps + t) * P.n_prb + tp.p_col[e];
                P.out[oi] = o;
                P.amp[oi] = v;
                // Kahan-compensated running time sum
                float yk = fsub(o, pcmp[e]);
                float tk = fadd(psum[e], yk);
                pcmp[e] = fsub(fsub(tk, psum[e]), yk);
                psum[e] = tk;
            }
            if (P.fields) {
                float* fo = P.fields + ((size_t)g.inst * P.steps + t) * plane;
#pragma unroll
                for (int i = 0; i < M; ++i) {
                    int gx = g.gx0 + i;
                    if (gx < P.nx) fo[(size_t)gx * P.ny + g.col] = yn[i];
                }
            }
            publish<M>(P, g, nbuf, yn, S);
#pragma unroll
            for (int i = 0; i < M; ++i) { y2[i] = y1[i]; y1[i] = yn[i]; }
        }
        cluster_sync_all();
    }
    if (P.probe_sum && g.colv) {
#pragma unroll
        for (int e = 0; e < PRBMAX; ++e)
            if (e < tp.np) P.probe_sum[(size_t)g.inst * P.n_prb + tp.p_col[e]] = psum[e];
    }
}

// ============================================================================
// Adjoint with segment recompute.
template <int M, int ORDER>
__global__ void __launch_bounds__(512, 1) seq_bwd_fused_kernel(FusedParams P) {
    extern __shared__ __align__(16) float smem[];
    const Geo g = make_geo(P, M);
    const int S = P.R / M;
    const int NT = blockDim.x;
    const int tile = (P.ny + 2) * P.LD;
    float* F0 = smem;
    float* F1 = smem + tile;
    // forward coefficients for the recompute live in shared memory,
    // layout [3][M][NT] (a warp reads 32 consecutive floats)
    float* KA = smem + 2 * tile;
    float* KB = KA + M * NT;
    float* KC2 = KB + M * NT;
    zero_smem(smem, 2 * tile);

    float X1[M], Kc[M], Kg[M], Ky2[M];
#pragma unroll
    for (int i = 0; i < M; ++i) {
        X1[i] = Kc[i] = Kg[i] = Ky2[i] = 0.f;
        float a = 0.f, bc = 0.f, c2 = 0.f;
        int gx = g.gx0 + i;
        if (g.colv && gx < P.nx) {
            size_t cell = (size_t)gx * P.ny + g.col;
            float bb = __ldg(P.b + cell), cc = __ldg(P.c + cell);
            FwdCoef f = fwd_coef(bb, cc, P.k);
            BwdCoef k = bwd_coef(bb, cc, P.k);
            a = f.A; bc = f.Bc; c2 = f.c2;
            X1[i] = k.X1; Kc[i] = k.Kc; Kg[i] = k.Kg; Ky2[i] = k.Ky2;
        }
        KA[i * NT + threadIdx.x] = a;
        KB[i * NT + threadIdx.x] = bc;
        KC2[i * NT + threadIdx.x] = c2;
    }
    Taps<M> tp;
    build_taps<M>(P, g, tp);

    const size_t plane = (size_t)P.nx * P.ny;
    const size_t bplane = (size_t)P.batch * plane;
    // stash of this thread: [seg][M] strided by NT
    float* stash = P.stash + ((size_t)(g.inst * P.C + g.cta) * P.seg) * M * NT + threadIdx.x;

    // adjoint state: gy1 pending from t+1, gy2 pending from t+1 and t+2
    float gy1[M], gy2a[M], gy2b[M], acc[M];
#pragma unroll
    for (int i = 0; i < M; ++i) gy1[i] = gy2a[i] = gy2b[i] = acc[i] = 0.f;
    bool have_gy1 = false, have_gy2b = false;   // gy2b: from t+2

    cluster_sync_all();
    const int nseg = (P.steps + P.seg - 1) / P.seg;
    // wsel: the tile to write next.  Invariant: its last reader finished
    // before the most recent cluster barrier, so writing it is race free.
    int wsel = 0;
    for (int sgi = nseg - 1; sgi >= 0; --sgi) {
        const int t0 = sgi * P.seg;
        const int t1 = min(P.steps, t0 + P.seg);
        // ---- recompute the segment's forward, stashing Lap(h_{t-1}) ----
        float y1[M], y2[M];
#pragma unroll
        for (int i = 0; i < M; ++i) y1[i] = y2[i] = 0.f;
        if (sgi > 0 && g.colv) {
            const float* ck = P.ckpt + (size_t)sgi * 2 * bplane + (size_t)g.inst * plane;
#pragma unroll
            for (int i = 0; i < M; ++i) {
                int gx = g.gx0 + i;
                if (gx < P.nx) {
                    size_t cell = (size_t)gx * P.ny + g.col;
                    y1[i] = __ldcg(ck + cell);
                    y2[i] = __ldcg(ck + bplane + cell);
                }
            }
        }
        publish<M>(P, g, wsel ? F1 : F0, y1, S);
        cluster_sync_all();
        int rsel = wsel;
        wsel ^= 1;
        float A[M], Bc[M], C2[M];
#pragma unroll
        for (int i = 0; i < M; ++i) {
            A[i] = KA[i * NT + threadIdx.x];
            Bc[i] = KB[i * NT + threadIdx.x];
            C2[i] = KC2[i * NT + threadIdx.x];
        }
        for (int t = t0; t < t1; ++t) {
            if (g.colv) {
                float xc[SRCMAX];
#pragma unroll
                for (int e = 0; e < SRCMAX; ++e)
                    xc[e] = e < tp.ns ? __ldg(P.x + (size_t)tp.s_row[e] * P.steps + t) : 0.f;
                float yn[M], L[M];
                fwd_cells<M, ORDER>(P, g, rsel ? F1 : F0, A, Bc, C2, y1, y2, yn, L, tp, xc);
                float* sp = stash + (size_t)(t - t0) * M * NT;
#pragma unroll
                for (int i = 0; i < M; ++i) sp[(size_t)i * NT] = L[i];
                if (t + 1 < t1) publish<M>(P, g, wsel ? F1 : F0, yn, S);
#pragma unroll
                for (int i = 0; i < M; ++i) { y2[i] = y1[i]; y1[i] = yn[i]; }
            }
            if (t + 1 < t1) {
                cluster_sync_all();
                rsel = wsel;
                wsel ^= 1;
            }
        }
        // ---- adjoint sweep over the segment ----
        for (int t = t1 - 1; t >= t0; --t) {
            float* buf = wsel ? F1 : F0;
            float lam[M];
#pragma unroll
            for (int i = 0; i < M; ++i) lam[i] = 0.f;
            if (g.colv) {
#pragma unroll
                for (int i = 0; i < M; ++i) {
                    float v = 0.f;
                    if (have_gy2b) v = gy2b[i];
                    if (have_gy1) v = have_gy2b ? fadd(v, gy1[i]) : gy1[i];
                    lam[i] = v;
                }
                // probe seeds, descending reference order (list order)
#pragma unroll
                for (int e = 0; e < PRBMAX; ++e) {
                    if (e >= tp.np) break;
                    size_t oi = ((size_t)g.inst * P.steps + t) * P.n_prb + tp.p_col[e];
                    float gv = __ldg(P.grad_out + oi);
                    float sd = tp.p_kind[e] ? fmul(gv, fmul(2.0f, __ldg(P.amp + oi))) : gv;
                    add_at<M>(lam, tp.p_i[e], sd);
                }
                if (P.grad_x) {
#pragma unroll
                    for (int e = 0; e < SRCMAX; ++e)
                        if (e < tp.ns && tp.s_row[e] == g.inst)
                            P.grad_x[(size_t)g.inst * P.steps + t] = pick<M>(lam, tp.s_i[e]);
                }
                float c2g[M];
#pragma unroll
                for (int i = 0; i < M; ++i) c2g[i] = fmul(Kg[i], lam[i]);
                publish<M>(P, g, buf, c2g, S);
            }
            cluster_sync_all();
            if (g.colv) {
                float c2g[M], lg[M];
#pragma unroll
                for (int i = 0; i < M; ++i) c2g[i] = fmul(Kg[i], lam[i]);
                strip_lap<M, ORDER>(P, g, buf, c2g, lg);
                const float* sp = stash + (size_t)(t - t0) * M * NT;
#pragma unroll
                for (int i = 0; i < M; ++i) {
                    float Ly = sp[(size_t)i * NT];
                    acc[i] = fadd(acc[i], fmul(fmul(X1[i], fmul(Kc[i], Ly)), lam[i]));
                    gy1[i] = fadd(fmul(P.k.dt2, lg[i]), fmul(fmul(2.0f, lam[i]), X1[i]));
                    gy2b[i] = gy2a[i];
                    gy2a[i] = fmul(Ky2[i], lam[i]);
                }
            }
            have_gy2b = have_gy1;   // gy2 from t+1 becomes "from t+2" at t-1
            have_gy1 = true;
            wsel ^= 1;
        }
    }
    if (g.colv) {
        float* o = P.gc_part + (size_t)g.inst * plane;
#pragma unroll
        for (int i = 0; i < M; ++i) {
            int gx = g.gx0 + i;
            if (gx < P.nx) o[(size_t)gx * P.ny + g.col] = acc[i];
        }
    }
    cluster_sync_all();
}

}  // namespace wt

// ---------------------------------------------------------------------------
// Host side: configuration and launch
#include <cstdio>

static int tile_ld(int rows) {
    int ld = rows + wt::OFF + 1;
    while (ld % 8 != 4) ++ld;
    return ld;
}

// Pick (C, M) for a grid: clusters of C CTAs, M cells per thread, at most
// 512 threads per CTA.  Returns 0 on success.
int wt_fused_plan(int nx, int ny, int cluster_req, WtFusedLaunch* L) {
    const int NCP = ((ny + 31) / 32) * 32;
    const int Ms[2] = {8, 4};
    const int Cs[5] = {4, 2, 8, 1, 16};
    for (int ci = 0; ci < 5; ++ci) {
        int C = Cs[ci];
        if (cluster_req > 0 && C != cluster_req) continue;
        if (C > 8) continue;
        for (int mi = 0; mi < 2; ++mi) {
            int M = Ms[mi];
            int rows = (nx + C - 1) / C;
            int R = ((rows + M - 1) / M) * M;
            if ((C - 1) * R >= nx) continue;   // an empty CTA
            int S = R / M;
            int threads = S * NCP;
            if (threads > 512) continue;
            int LD = tile_ld(R);
            size_t tile = (size_t)(ny + 2) * LD * sizeof(float);
            size_t fwd = 2 * tile;
            size_t bwd = 2 * tile + 3 * (size_t)M * threads * sizeof(float);
            if (bwd > 227 * 1024) continue;
            L->C = C; L->M = M; L->R = R; L->S = S; L->NCP = NCP; L->LD = LD;
            L->threads = threads; L->smem_fwd = fwd; L->smem_bwd = bwd;
            return 0;
        }
    }
    return WT_ERR_UNSUPPORTED;
}

template <int M, int ORDER>
static int launch_fused(bool fwd, const wt::FusedParams& P, const WtFusedLaunch& L,
                        cudaStream_t st) {
    void (*kern)(wt::FusedParams) = fwd ? wt::seq_fwd_fused_kernel<M, ORDER>
                                        : wt::seq_bwd_fused_kernel<M, ORDER>;
    size_t smem = fwd ? L.smem_fwd : L.smem_bwd;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return wt_cuda_status(e);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(L.C * P.batch, 1, 1);
    cfg.blockDim = dim3(L.threads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = L.C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, kern, P);
    wt_count_launches(1);
    return wt_cuda_status(e);
}

int wt_launch_fused(bool fwd, const wt::FusedParams& P, const WtFusedLaunch& L, cudaStream_t st) {
    if (P.k.lap_order == WT_LAP_SEQ) {
        if (L.M == 8) return launch_fused<8, WT_LAP_SEQ>(fwd, P, L, st);
        if (L.M == 4) return launch_fused<4, WT_LAP_SEQ>(fwd, P, L, st);
    } else {
        if (L.M == 8) return launch_fused<8, WT_LAP_PAIRED>(fwd, P, L, st);
        if (L.M == 4) return launch_fused<4, WT_LAP_PAIRED>(fwd, P, L, st);
    }
    return WT_ERR_UNSUPPORTED;
}
