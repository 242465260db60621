/*
 * ORACLE -- test infrastructure only.  A plain-C restatement of the float32
 * arithmetic of fancompute/wavetorch v0.2.1's time-stepping path, used by the
 * tests, the smoke check and the CPU baseline of the benchmark as the checker
 * and never as the product.  Pinned against golden vectors produced by the
 * reference itself (tests/golden/).
 *
 * Every function states the reference lines it restates.  Association orders:
 *   Laplacian     torch CPU conv2d (wavetorch/operators.py:5-11): oneDNN's
 *                 row-major fused multiply-add chain when batch > 1 or the grid
 *                 has > 20480 cells (ORD_SEQ), else the im2col+GEMM pairing
 *                 (u + l) + (-4c + (r + d)) (ORD_PAIRED, h == 1).
 *   update        wavetorch/cell.py:12-17, left to right; the nonlinear
 *                 cell's b and c (cell.py:8-9, :93-101) per cell and step.
 *   adjoint       wavetorch/cell.py:26-44, plus autograd's accumulation order:
 *                 the gradient reaching h_t is (grad_y2 from step t+2 +
 *                 grad_y1 from step t+1), then the probe terms in descending
 *                 probe order; per-step dL/dc is summed over the batch in
 *                 blocks of 16 (torch's CPU sum-to-shape), and the per-step
 *                 sums are added from the last step down.
 * Build: see oracle/Makefile (gcc, -ffp-contract=off, optional OpenMP).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORD_SEQ 0
#define ORD_PAIRED 1

typedef struct or_desc {
    int32_t batch, nx, ny, steps;
    float dt, h;
    int32_t order;
    int32_t n_src;
    const int32_t* src_cell;   /* table order */
    const int32_t* src_row;    /* -1 = own row */
    int32_t n_prb;
    const int32_t* prb_cell;   /* output column q */
    const int32_t* prb_kind;   /* 0 amplitude, 1 intensity */
    const int32_t* prb_order;  /* reference probe index */
} or_desc;

typedef struct scal {
    float inv_dt2, inv_dt, two_over, dt, dt2, w, w4;
} scal;

static scal make_scal(float dt, float h) {
    scal s;
    float dd = dt * dt;
    s.inv_dt2 = 1.0f / dd;          /* dt**-2  (pow -2 = 1/(x*x)) */
    s.inv_dt = 1.0f / dt;           /* dt**-1 */
    s.two_over = (1.0f / dd) * 2.0f;/* 2 / dt**2 = reciprocal(dt*dt) * 2 */
    s.dt = dt;
    s.dt2 = dd;                     /* dt**2 */
    float hh = h * h;
    s.w = 1.0f / hh;                /* h**-2 */
    s.w4 = s.w * -4.0f;
    return s;
}

/* 5-point Laplacian of field f at (i, j), zero outside (operators.py:5-11) */
static inline float lap_at(const float* f, int nx, int ny, int i, int j, const scal* s, int order) {
    float u = i > 0 ? f[(size_t)(i - 1) * ny + j] : 0.0f;
    float d = i + 1 < nx ? f[(size_t)(i + 1) * ny + j] : 0.0f;
    float l = j > 0 ? f[(size_t)i * ny + j - 1] : 0.0f;
    float r = j + 1 < ny ? f[(size_t)i * ny + j + 1] : 0.0f;
    float c = f[(size_t)i * ny + j];
    if (order == ORD_SEQ) {
        float acc = s->w * u;
        acc = fmaf(s->w, l, acc);
        acc = fmaf(s->w4, c, acc);
        acc = fmaf(s->w, r, acc);
        return fmaf(s->w, d, acc);
    }
    float wu = s->w * u, wl = s->w * l, wr = s->w * r, wd = s->w * d, wc = s->w4 * c;
    float ul = wu + wl;
    float rd = wr + wd;
    return ul + (wc + rd);
}

/* Laplacian of the field g = K * lam (K per cell) at (i, j) */
static inline float lap_scaled(const float* K, const float* lam, int nx, int ny, int i, int j,
                               const scal* s, int order) {
#define G(a, b) (K[(size_t)(a) * ny + (b)] * lam[(size_t)(a) * ny + (b)])
    float u = i > 0 ? G(i - 1, j) : 0.0f;
    float d = i + 1 < nx ? G(i + 1, j) : 0.0f;
    float l = j > 0 ? G(i, j - 1) : 0.0f;
    float r = j + 1 < ny ? G(i, j + 1) : 0.0f;
    float c = G(i, j);
#undef G
    if (order == ORD_SEQ) {
        float acc = s->w * u;
        acc = fmaf(s->w, l, acc);
        acc = fmaf(s->w4, c, acc);
        acc = fmaf(s->w, r, acc);
        return fmaf(s->w, d, acc);
    }
    float wu = s->w * u, wl = s->w * l, wr = s->w * r, wd = s->w * d, wc = s->w4 * c;
    return (wu + wl) + (wc + (wr + wd));
}

/* cell.py:12-17 for one cell */
static inline float update(float b, float c, float y1, float y2, float L, const scal* s) {
    float bd = b * s->inv_dt;
    float A = 1.0f / (s->inv_dt2 + bd);
    float Bc = s->inv_dt2 - bd;
    float c2 = c * c;
    float t1 = s->two_over * y1;
    float t2 = Bc * y2;
    float v = t1 - t2;
    float t3 = c2 * L;
    v = v + t3;
    return A * v;
}

/* ---- TimeStep (cell.py:20-44) ------------------------------------------ */
void or_step_fwd(int B, int nx, int ny, float dt, float h, int order, int coef_batched,
                 const float* b, const float* c, const float* y1, const float* y2, float* y) {
    scal s = make_scal(dt, h);
    size_t plane = (size_t)nx * ny;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < B; ++k)
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j) {
                size_t cell = (size_t)i * ny + j, ic = k * plane + cell;
                size_t co = coef_batched ? ic : cell;
                float L = lap_at(y1 + k * plane, nx, ny, i, j, &s, order);
                y[ic] = update(b[co], c[co], y1[ic], y2[ic], L, &s);
            }
}

/* torch CPU sum over the batch (blocks of 16, sequential) of v[k] */
static inline float batch_sum(const float* v, size_t stride, int B) {
    float acc = 0.0f, blk = 0.0f;
    for (int k = 0; k < B; ++k) {
        blk = blk + v[k * stride];
        if ((k & 15) == 15 || k == B - 1) {
            acc = k < 16 ? blk : acc + blk;
            blk = 0.0f;
        }
    }
    return acc;
}

void or_step_bwd(int B, int nx, int ny, float dt, float h, int order, int coef_batched,
                 const float* b, const float* c, const float* y1, const float* y2, const float* g,
                 float* gb, float* gc, float* gy1, float* gy2) {
    scal s = make_scal(dt, h);
    size_t plane = (size_t)nx * ny;
    float* tb = gb && !coef_batched ? (float*)malloc(sizeof(float) * B * plane) : NULL;
    float* tc = gc && !coef_batched ? (float*)malloc(sizeof(float) * B * plane) : NULL;
    /* Kg = X1 * c^2 per (instance, cell) for the grad_y1 Laplacian */
    float* Kg = (float*)malloc(sizeof(float) * (coef_batched ? B : 1) * plane);
    for (size_t q = 0; q < (coef_batched ? (size_t)B : 1) * plane; ++q) {
        float X1 = 1.0f / (b[q] * dt + 1.0f);
        Kg[q] = X1 * (c[q] * c[q]);
    }
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < B; ++k)
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j) {
                size_t cell = (size_t)i * ny + j, ic = k * plane + cell;
                size_t co = coef_batched ? ic : cell;
                float bb = b[co], cc = c[co], gv = g[ic];
                float bdt = bb * dt;
                float X1 = 1.0f / (bdt + 1.0f);
                float L = (gb || gc) ? lap_at(y1 + k * plane, nx, ny, i, j, &s, order) : 0.0f;
                if (gc) {
                    float t = (2.0f * cc) * s.dt2;
                    t = t * L;
                    t = X1 * t;
                    t = t * gv;
                    (coef_batched ? gc : tc)[ic] = t;
                }
                if (gb) {
                    float v = dt * bb + 1.0f;
                    float kb = -(1.0f / (v * v));
                    kb = kb * dt;
                    float in = ((cc * cc) * s.dt2) * L;
                    in = in + 2.0f * y1[ic];
                    in = in - 2.0f * y2[ic];
                    float t = (kb * in) * gv;
                    (coef_batched ? gb : tb)[ic] = t;
                }
                if (gy1) {
                    const float* K = Kg + (coef_batched ? k * plane : 0);
                    float lg = lap_scaled(K, g + k * plane, nx, ny, i, j, &s, order);
                    gy1[ic] = s.dt2 * lg + (2.0f * gv) * X1;
                }
                if (gy2) gy2[ic] = ((bdt - 1.0f) * X1) * gv;
            }
    if (!coef_batched) {
        for (size_t q = 0; q < plane; ++q) {
            if (gc) gc[q] = batch_sum(tc + q, plane, B);
            if (gb) gb[q] = batch_sum(tb + q, plane, B);
        }
    }
    free(tb);
    free(tc);
    free(Kg);
}

/* ---- the time loop, wavetorch/rnn.py:36-72 ------------------------------- */
/* hist: [B][T][nx][ny] (every field, needed by or_seq_bwd), out [B][T][n_prb] */
void or_seq_fwd(const or_desc* d, const float* b, const float* c, const float* x, float* out,
                float* hist) {
    const int B = d->batch, nx = d->nx, ny = d->ny, T = d->steps;
    scal s = make_scal(d->dt, d->h);
    const size_t plane = (size_t)nx * ny;
    const size_t hb = (size_t)T * plane;   /* history batch stride */
    /* factor the time-invariant coefficients exactly like update() */
    float* A = (float*)malloc(sizeof(float) * plane);
    float* Bc = (float*)malloc(sizeof(float) * plane);
    float* C2 = (float*)malloc(sizeof(float) * plane);
    for (size_t q = 0; q < plane; ++q) {
        float bd = b[q] * s.inv_dt;
        A[q] = 1.0f / (s.inv_dt2 + bd);
        Bc[q] = s.inv_dt2 - bd;
        C2[q] = c[q] * c[q];
    }
    float* zero = (float*)calloc(plane, sizeof(float));
    for (int t = 0; t < T; ++t) {
        /* every cell of every instance (rows in parallel too, for one large
         * instance), then each instance's sources and probes */
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k < B; ++k)
            for (int i = 0; i < nx; ++i) {
                const float* y1 = t >= 1 ? hist + k * hb + (size_t)(t - 1) * plane : zero;
                const float* y2 = t >= 2 ? hist + k * hb + (size_t)(t - 2) * plane : zero;
                float* y = hist + k * hb + (size_t)t * plane;
                for (int j = 0; j < ny; ++j) {
                    size_t q = (size_t)i * ny + j;
                    float L = lap_at(y1, nx, ny, i, j, &s, d->order);
                    float v = (s.two_over * y1[q]) - (Bc[q] * y2[q]);
                    v = v + C2[q] * L;
                    y[q] = A[q] * v;
                }
            }
        for (int k = 0; k < B; ++k) {
            float* y = hist + k * hb + (size_t)t * plane;
            for (int e = 0; e < d->n_src; ++e) {
                int row = d->src_row[e] < 0 ? k : d->src_row[e];
                y[d->src_cell[e]] = y[d->src_cell[e]] + x[(size_t)row * T + t];
            }
            for (int q = 0; q < d->n_prb; ++q) {
                float v = y[d->prb_cell[q]];
                out[((size_t)k * T + t) * d->n_prb + q] = d->prb_kind[q] ? v * v : v;
            }
        }
    }
    free(A); free(Bc); free(C2); free(zero);
}

/* adjoint of or_seq_fwd: grad_c [nx][ny]; grad_x [B][T] or NULL (own-row
 * sources only: dL/dx[k,t] = sum over that instance's source cells, added in
 * descending source order as autograd does) */
void or_seq_bwd(const or_desc* d, const float* b, const float* c, const float* hist,
                const float* grad_out, float* grad_c, float* grad_x) {
    const int B = d->batch, nx = d->nx, ny = d->ny, T = d->steps;
    scal s = make_scal(d->dt, d->h);
    const size_t plane = (size_t)nx * ny, bp = (size_t)B * plane, hb = (size_t)T * plane;
    float* X1 = (float*)malloc(sizeof(float) * plane);
    float* Kc = (float*)malloc(sizeof(float) * plane);
    float* Kg = (float*)malloc(sizeof(float) * plane);
    float* Ky2 = (float*)malloc(sizeof(float) * plane);
    for (size_t q = 0; q < plane; ++q) {
        float bdt = b[q] * s.dt;
        X1[q] = 1.0f / (bdt + 1.0f);
        Kc[q] = (2.0f * c[q]) * s.dt2;
        Kg[q] = X1[q] * (c[q] * c[q]);
        Ky2[q] = (bdt - 1.0f) * X1[q];
    }
    float* lam = (float*)malloc(sizeof(float) * 3 * bp);
    float* gct = (float*)malloc(sizeof(float) * bp);
    /* probe columns in descending reference order (stable) */
    int* pidx = (int*)malloc(sizeof(int) * (d->n_prb + 1));
    for (int q = 0; q < d->n_prb; ++q) pidx[q] = q;
    for (int a = 1; a < d->n_prb; ++a) {   /* insertion sort, stable */
        int v = pidx[a], j = a - 1;
        while (j >= 0 && d->prb_order[pidx[j]] < d->prb_order[v]) { pidx[j + 1] = pidx[j]; --j; }
        pidx[j + 1] = v;
    }
    for (int t = T - 1; t >= 0; --t) {
        float* L0 = lam + (size_t)(t % 3) * bp;
        const float* L1 = t + 1 < T ? lam + (size_t)((t + 1) % 3) * bp : NULL;
        const float* L2 = t + 2 < T ? lam + (size_t)((t + 2) % 3) * bp : NULL;
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k < B; ++k)
            for (int i = 0; i < nx; ++i) {
                float* l0 = L0 + k * plane;
                for (int j = 0; j < ny; ++j) {
                    size_t q = (size_t)i * ny + j;
                    float v = 0.0f;
                    if (L2) v = Ky2[q] * L2[k * plane + q];
                    if (L1) {
                        float lg = lap_scaled(Kg, L1 + k * plane, nx, ny, i, j, &s, d->order);
                        float gy1 = s.dt2 * lg + (2.0f * L1[k * plane + q]) * X1[q];
                        v = L2 ? v + gy1 : gy1;
                    }
                    l0[q] = v;
                }
            }
        for (int k = 0; k < B; ++k) {
            float* l0 = L0 + k * plane;
            for (int a = 0; a < d->n_prb; ++a) {
                int q = pidx[a];
                size_t o = ((size_t)k * T + t) * d->n_prb + q;
                float gv = grad_out[o];
                float amp = hist[k * hb + (size_t)t * plane + d->prb_cell[q]];
                float sd = d->prb_kind[q] ? gv * (2.0f * amp) : gv;
                l0[d->prb_cell[q]] = l0[d->prb_cell[q]] + sd;
            }
            if (grad_x) {
                float acc = 0.0f;
                int first = 1;
                for (int e = d->n_src - 1; e >= 0; --e) {
                    if (d->src_row[e] >= 0) continue;
                    float v = l0[d->src_cell[e]];
                    acc = first ? v : acc + v;
                    first = 0;
                }
                grad_x[(size_t)k * T + t] = acc;
            }
        }
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k < B; ++k)
            for (int i = 0; i < nx; ++i) {
                const float* l0 = L0 + k * plane;
                const float* hp = t >= 1 ? hist + k * hb + (size_t)(t - 1) * plane : NULL;
                for (int j = 0; j < ny; ++j) {
                    size_t q = (size_t)i * ny + j;
                    float L = hp ? lap_at(hp, nx, ny, i, j, &s, d->order) : 0.0f;
                    float tt = Kc[q] * L;
                    tt = X1[q] * tt;
                    gct[k * plane + q] = tt * l0[q];
                }
            }
#pragma omp parallel for schedule(static)
        for (long q = 0; q < (long)plane; ++q) {
            float sum = batch_sum(gct + q, plane, B);
            grad_c[q] = (t == T - 1) ? sum : grad_c[q] + sum;
        }
    }
    free(X1); free(Kc); free(Kg); free(Ky2); free(lam); free(gct); free(pidx);
}

/* ---- nonlinear cell, wavetorch/cell.py:8-9, :79-107 ---------------------
 * Per step, from h1 = h_{t-1} (the post-source field):
 *   b = b_pml + rho * (b0 / (1 + |h1 / uth|^2))      (when b0 > 0)
 *   c = c_lin + (rho * c_nl) * h1^2                  (when c_nl != 0)
 * then TimeStep with these per-instance b, c.  rho is the raw density
 * parameter (wavetorch/rnn.py:47, geom.py:185-205), c_lin its projected
 * speed. */
typedef struct or_nl {
    float b0, uth, cnl;
} or_nl;

typedef struct nl_cell {
    float b, c, sat, q, a, D;    /* b, c of the step; sat, |h1/uth| pieces */
} nl_cell;

static inline nl_cell nl_bc(const or_nl* n, float bp, float cl, float rho, float h1) {
    nl_cell r;
    r.b = bp; r.c = cl; r.sat = 0.0f; r.q = 0.0f; r.a = 0.0f; r.D = 1.0f;
    if (n->b0 > 0.0f) {
        r.q = h1 / n->uth;
        r.a = fabsf(r.q);
        r.D = 1.0f + r.a * r.a;
        r.sat = n->b0 / r.D;
        r.b = bp + rho * r.sat;
    }
    if (n->cnl != 0.0f) r.c = cl + (rho * n->cnl) * (h1 * h1);
    return r;
}

/* forward: as or_seq_fwd with b, c formed per cell and step */
void or_seq_fwd_nl(const or_desc* d, const or_nl* n, const float* bp, const float* cl,
                   const float* rho, const float* x, float* out, float* hist) {
    const int B = d->batch, nx = d->nx, ny = d->ny, T = d->steps;
    scal s = make_scal(d->dt, d->h);
    const size_t plane = (size_t)nx * ny;
    const size_t hb = (size_t)T * plane;
    float* zero = (float*)calloc(plane, sizeof(float));
    for (int t = 0; t < T; ++t) {
#pragma omp parallel for schedule(static)
        for (int k = 0; k < B; ++k) {
            const float* y1 = t >= 1 ? hist + k * hb + (size_t)(t - 1) * plane : zero;
            const float* y2 = t >= 2 ? hist + k * hb + (size_t)(t - 2) * plane : zero;
            float* y = hist + k * hb + (size_t)t * plane;
            for (int i = 0; i < nx; ++i)
                for (int j = 0; j < ny; ++j) {
                    size_t q = (size_t)i * ny + j;
                    nl_cell m = nl_bc(n, bp[q], cl[q], rho[q], y1[q]);
                    float L = lap_at(y1, nx, ny, i, j, &s, d->order);
                    y[q] = update(m.b, m.c, y1[q], y2[q], L, &s);
                }
            for (int e = 0; e < d->n_src; ++e) {
                int row = d->src_row[e] < 0 ? k : d->src_row[e];
                y[d->src_cell[e]] = y[d->src_cell[e]] + x[(size_t)row * T + t];
            }
            for (int q = 0; q < d->n_prb; ++q) {
                float v = y[d->prb_cell[q]];
                out[((size_t)k * T + t) * d->n_prb + q] = d->prb_kind[q] ? v * v : v;
            }
        }
    }
    free(zero);
}

/* Adjoint of or_seq_fwd_nl in the order autograd runs the reference's graph
 * (highest sequence number first).  Step s's nodes run after those of every
 * later step: TimeStep_s, then the Kerr branch (AddBackward, MulBackward,
 * PowBackward(h1, 2), MulBackward(rho, c_nl)), then the damping branch
 * (AddBackward, MulBackward(rho, sat), DivBackward(b0, D), AddBackward,
 * PowBackward(a, 2), AbsBackward, DivBackward(h1, uth)), then the probes of
 * step s-1.  So the gradient of h_{s-1} is
 *   (((grad_y2 of step s+1 + grad_y1 of step s) + Kerr term) + damping term)
 * plus the probe terms in descending probe order; the density's gradient
 * takes, per step from the last, the Kerr term then the damping term (each
 * summed over the batch first, as sum_to does), and c_lin's the batch sum of
 * grad_c.  Formulas: TimeStep.backward (cell.py:26-44); torch's derivatives
 * of mul, div (other: -grad * ((self / other) / other)), pow (grad * (2 x)),
 * abs (grad * sgn).  Outputs: grad_c (dL/dc_lin) and grad_rho (the direct
 * part; the projection's part is added by the caller, last, as autograd
 * does). */
void or_seq_bwd_nl(const or_desc* d, const or_nl* n, const float* bp, const float* cl,
                   const float* rho, const float* hist, const float* grad_out, float* grad_c,
                   float* grad_rho) {
    const int B = d->batch, nx = d->nx, ny = d->ny, T = d->steps;
    scal s = make_scal(d->dt, d->h);
    const float dt = s.dt;
    const size_t plane = (size_t)nx * ny, bp_ = (size_t)B * plane, hb = (size_t)T * plane;
    float* lam = (float*)malloc(sizeof(float) * 3 * bp_);     /* lambda_t, ring of 3 */
    int set[3] = {0, 0, 0};                                     /* a gradient has arrived */
    float* Kg = (float*)malloc(sizeof(float) * bp_);            /* X1 c^2 of the step */
    float* gcs = (float*)malloc(sizeof(float) * bp_);           /* grad_c of the step */
    float* gkr = (float*)malloc(sizeof(float) * bp_);           /* grad_c * h1^2 */
    float* gbs = (float*)malloc(sizeof(float) * bp_);           /* grad_b * sat */
    float* zero = (float*)calloc(plane, sizeof(float));
    int* pidx = (int*)malloc(sizeof(int) * (d->n_prb + 1));
    for (int q = 0; q < d->n_prb; ++q) pidx[q] = q;
    for (int a = 1; a < d->n_prb; ++a) {
        int v = pidx[a], j = a - 1;
        while (j >= 0 && d->prb_order[pidx[j]] < d->prb_order[v]) { pidx[j + 1] = pidx[j]; --j; }
        pidx[j + 1] = v;
    }
    int first_rho = 1;
    for (int t = T - 1; t >= 0; --t) {
        float* L0 = lam + (size_t)(t % 3) * bp_;
        /* probe terms of step t into lambda_t */
        if (!set[t % 3]) memset(L0, 0, sizeof(float) * bp_);
        for (int k = 0; k < B; ++k)
            for (int a = 0; a < d->n_prb; ++a) {
                int q = pidx[a];
                size_t o = ((size_t)k * T + t) * d->n_prb + q;
                float gv = grad_out[o];
                float amp = hist[k * hb + (size_t)t * plane + d->prb_cell[q]];
                float sd = d->prb_kind[q] ? gv * (2.0f * amp) : gv;
                float* cell = L0 + k * plane + d->prb_cell[q];
                *cell = *cell + sd;   /* IndexBackward: zeros with the value added */
            }
        if (d->n_prb > 0) set[t % 3] = 1;
        /* step t's nodes: coefficients from h1 = h_{t-1}, h2 = h_{t-2} */
        float* L1 = lam + (size_t)((t + 2) % 3) * bp_;   /* lambda_{t-1} */
        float* L2 = lam + (size_t)((t + 1) % 3) * bp_;   /* lambda_{t-2} */
        const int has1 = t >= 1, has2 = t >= 2;
#pragma omp parallel for schedule(static)
        for (int k = 0; k < B; ++k) {
            const float* h1 = has1 ? hist + k * hb + (size_t)(t - 1) * plane : zero;
            const float* h2 = has2 ? hist + k * hb + (size_t)(t - 2) * plane : zero;
            const float* g = L0 + k * plane;
            for (size_t q = 0; q < plane; ++q) {
                nl_cell m = nl_bc(n, bp[q], cl[q], rho[q], h1[q]);
                float X1 = 1.0f / (m.b * dt + 1.0f);
                Kg[k * plane + q] = X1 * (m.c * m.c);
            }
            for (int i = 0; i < nx; ++i)
                for (int j = 0; j < ny; ++j) {
                    size_t q = (size_t)i * ny + j, ic = k * plane + q;
                    nl_cell m = nl_bc(n, bp[q], cl[q], rho[q], h1[q]);
                    float gv = set[t % 3] ? g[q] : 0.0f;
                    float bdt = m.b * dt;
                    float X1 = 1.0f / (bdt + 1.0f);
                    float L = lap_at(h1, nx, ny, i, j, &s, d->order);
                    float gc = (2.0f * m.c) * s.dt2;                  /* grad_c */
                    gc = gc * L;
                    gc = X1 * gc;
                    gc = gc * gv;
                    gcs[ic] = gc;
                    float gb = 0.0f;                                  /* grad_b */
                    if (n->b0 > 0.0f) {
                        float v = dt * m.b + 1.0f;
                        float kb = -(1.0f / (v * v));
                        kb = kb * dt;
                        float in = ((m.c * m.c) * s.dt2) * L;
                        in = in + 2.0f * h1[q];
                        in = in - 2.0f * h2[q];
                        gb = (kb * in) * gv;
                    }
                    gkr[ic] = gc * (h1[q] * h1[q]);
                    gbs[ic] = gb * m.sat;
                    if (has1) {
                        float lg = lap_scaled(Kg + k * plane, g, nx, ny, i, j, &s, d->order);
                        float v = s.dt2 * lg + (2.0f * gv) * X1;       /* grad_y1 */
                        float* l1 = L1 + ic;
                        v = set[(t + 2) % 3] ? *l1 + v : v;
                        if (n->cnl != 0.0f)                            /* Kerr term */
                            v = v + (gc * (rho[q] * n->cnl)) * (2.0f * h1[q]);
                        if (n->b0 > 0.0f) {                            /* damping term */
                            float gsat = gb * rho[q];
                            float gD = -gsat * ((n->b0 / m.D) / m.D);
                            float ga = gD * (2.0f * m.a);
                            float sg = m.q > 0.0f ? 1.0f : (m.q < 0.0f ? -1.0f : 0.0f);
                            v = v + (ga * sg) / n->uth;
                        }
                        *l1 = v;
                    }
                    if (has2) L2[ic] = ((bdt - 1.0f) * X1) * gv;     /* grad_y2, first arrival */
                }
        }
        if (has1) set[(t + 2) % 3] = 1;
        if (has2) set[(t + 1) % 3] = 1;
        set[t % 3] = 0;   /* the ring slot is lambda_{t-3} from here on */
#pragma omp parallel for schedule(static)
        for (long q = 0; q < (long)plane; ++q) {
            float sc = batch_sum(gcs + q, plane, B);
            grad_c[q] = (t == T - 1) ? sc : grad_c[q] + sc;
            float r = first_rho ? 0.0f : grad_rho[q];
            int have = !first_rho;
            if (n->cnl != 0.0f) {
                float v = batch_sum(gkr + q, plane, B) * n->cnl;
                r = have ? r + v : v;
                have = 1;
            }
            if (n->b0 > 0.0f) {
                float v = batch_sum(gbs + q, plane, B);
                r = have ? r + v : v;
                have = 1;
            }
            grad_rho[q] = have ? r : 0.0f;
        }
        if (n->cnl != 0.0f || n->b0 > 0.0f) first_rho = 0;
    }
    free(lam); free(Kg); free(gcs); free(gkr); free(gbs); free(zero); free(pidx);
}

/* ---- free-form geometry, wavetorch/geom.py:207-233 ---------------------- */
/* blur: row-major fused multiply-add chain (oneDNN order) */
static void blur(int nx, int ny, int rad, const float* w, const float* in, float* out) {
    int K = 2 * rad + 1;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j) {
            float acc = 0.0f;
            for (int kh = 0; kh < K; ++kh)
                for (int kw = 0; kw < K; ++kw) {
                    int si = i + kh - rad, sj = j + kw - rad;
                    float v = (si >= 0 && si < nx && sj >= 0 && sj < ny) ? in[(size_t)si * ny + sj] : 0.0f;
                    acc = fmaf(w[kh * K + kw], v, acc);
                }
            out[(size_t)i * ny + j] = acc;
        }
}

/* transposed blur (conv2d input gradient, col2im order) */
static void blur_t(int nx, int ny, int rad, const float* w, const float* in, float* out) {
    int K = 2 * rad + 1;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j) {
            float acc = 0.0f;
            for (int kh = 0; kh < K; ++kh)
                for (int kw = 0; kw < K; ++kw) {
                    int si = i - kh + rad, sj = j - kw + rad;
                    float v = (si >= 0 && si < nx && sj >= 0 && sj < ny) ? in[(size_t)si * ny + sj] : 0.0f;
                    float p = w[kh * K + kw] * v;
                    acc = acc + p;
                }
            out[(size_t)i * ny + j] = acc;
        }
}

/* c = c0 + (c1-c0) P(blur^n(rho)); th (nullable) receives tanh(beta (r - eta)) */
void or_rho_to_c(int nx, int ny, int rad, int blur_n, float eta, float beta, float c0, float c1,
                 const float* w, const float* rho, float* c, float* th) {
    size_t n = (size_t)nx * ny;
    float* a = (float*)malloc(sizeof(float) * n);
    float* t = (float*)malloc(sizeof(float) * n);
    memcpy(a, rho, sizeof(float) * n);
    for (int p = 0; p < blur_n; ++p) {
        blur(nx, ny, rad, w, a, t);
        memcpy(a, t, sizeof(float) * n);
    }
    double be = (double)beta * (double)eta, b1 = (double)beta * (1.0 - (double)eta);
    float tbe = (float)tanh(be);
    float den = (float)(tanh(be) + tanh(b1));
    float dc = (float)((double)c1 - (double)c0);
    for (size_t q = 0; q < n; ++q) {
        float z = beta * (a[q] - eta);
        float tz = (float)tanh((double)z);   /* rounded once, like the GPU path */
        if (th) th[q] = tz;
        float P = (tz + tbe) / den;
        c[q] = c0 + dc * P;
    }
    free(a); free(t);
}

void or_rho_to_c_bwd(int nx, int ny, int rad, int blur_n, float eta, float beta, float c0,
                     float c1, const float* w, const float* th, const float* gc, float* grho) {
    size_t n = (size_t)nx * ny;
    (void)eta;
    double be = (double)beta * (double)eta, b1 = (double)beta * (1.0 - (double)eta);
    float den = (float)(tanh(be) + tanh(b1));
    float dc = (float)((double)c1 - (double)c0);
    float* a = (float*)malloc(sizeof(float) * n);
    float* t = (float*)malloc(sizeof(float) * n);
    for (size_t q = 0; q < n; ++q) {
        float gp = (gc[q] * dc) / den;
        float gz = gp * (1.0f - th[q] * th[q]);
        a[q] = gz * beta;
    }
    for (int p = 0; p < blur_n; ++p) {
        blur_t(nx, ny, rad, w, a, t);
        memcpy(a, t, sizeof(float) * n);
    }
    memcpy(grho, a, sizeof(float) * n);
    free(a); free(t);
}

/* ---- hole geometry (wavetorch/geom.py:109-132) ----------------------------
 * s[i][j] = sum_k exp(-sqrt((i - x_k)^2 + (j - y_k)^2) / r_k), the holes added
 * in index order to a zero field (geom.py:119-123); rho = P(s) and
 * c = c0 + (c1 - c0) rho (geom.py:125-132).  exp and tanh are evaluated in
 * double and rounded once to float.  rho, c, th nullable. */
static float hole_exp(float fi, float fj, float xk, float yk, float rk, float* dist, float* dx,
                      float* dy) {
    float a = fi - xk, b = fj - yk;
    float d = sqrtf(a * a + b * b);
    *dist = d; *dx = a; *dy = b;
    return (float)exp((double)(-d / rk));
}

void or_holey(int nx, int ny, int nh, float eta, float beta, float c0, float c1, const float* x,
              const float* y, const float* r, float* rho, float* c, float* th) {
    double be = (double)beta * (double)eta, b1 = (double)beta * (1.0 - (double)eta);
    float tbe = (float)tanh(be);
    float den = (float)(tanh(be) + tanh(b1));
    float dc = (float)((double)c1 - (double)c0);
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j) {
            float s = 0.0f, d, a, b;
            for (int k = 0; k < nh; ++k) s = s + hole_exp((float)i, (float)j, x[k], y[k], r[k], &d, &a, &b);
            float tz = (float)tanh((double)(beta * (s - eta)));
            float P = (tz + tbe) / den;
            size_t q = (size_t)i * ny + j;
            if (th) th[q] = tz;
            if (rho) rho[q] = P;
            if (c) c[q] = c0 + dc * P;
        }
}

/* Gradients with respect to the holes' centres and radii, the reference's
 * autograd chain per cell (MulBackward, DivBackward, TanhBackward,
 * ExpBackward, DivBackward for both operands, NegBackward, SqrtBackward,
 * PowBackward, SubBackward) in float32; the sum over cells in double.  grho
 * and gc nullable (zero). */
void or_holey_bwd(int nx, int ny, int nh, float eta, float beta, float c0, float c1,
                  const float* x, const float* y, const float* r, const float* th,
                  const float* grho, const float* gc, float* gx, float* gy, float* gr) {
    double be = (double)beta * (double)eta, b1 = (double)beta * (1.0 - (double)eta);
    float den = (float)(tanh(be) + tanh(b1));
    float dc = (float)((double)c1 - (double)c0);
    for (int k = 0; k < nh; ++k) {
        double ax = 0.0, ay = 0.0, ar = 0.0;
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j) {
                size_t q = (size_t)i * ny + j;
                float gp = (grho ? grho[q] : 0.0f) + (gc ? gc[q] * dc : 0.0f);
                float gs = ((gp / den) * (1.0f - th[q] * th[q])) * beta;
                float d, a, b;
                float e = hole_exp((float)i, (float)j, x[k], y[k], r[k], &d, &a, &b);
                float ge = gs * e;
                float gq = ge / r[k];
                float grk = -ge * ((-d / r[k]) / r[k]);
                float gd2 = -gq / (2.0f * d);
                ax += (double)(-(gd2 * (2.0f * a)));
                ay += (double)(-(gd2 * (2.0f * b)));
                ar += (double)grk;
            }
        gx[k] = (float)ax;
        gy[k] = (float)ay;
        gr[k] = (float)ar;
    }
}

int or_num_threads(void) {
#ifdef _OPENMP
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();
#else
    return 1;
#endif
}
