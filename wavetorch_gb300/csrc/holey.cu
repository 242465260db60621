// Hole geometry (wavetorch/geom.py:88-132) and its adjoint:
//   s[i][j] = sum_k exp(-sqrt((i - x_k)^2 + (j - y_k)^2) / r_k)
//   rho = P(s),  c = c0 + (c1 - c0) * rho
// with P the free-form geometry's projection.  The holes are added in index
// order to a zero field, as the reference's loop does (geom.py:119-123).
// exp and tanh are evaluated in double and rounded once to float; the
// reference's float32 exp and tanh are within an ulp of that.
//
// The adjoint forms each cell's contribution in float32 in the order of the
// reference's autograd chain and sums the cells in double: each block writes
// one partial per hole and component, a second kernel adds the partials in
// block order, so the result does not depend on scheduling.
#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace wt {

struct HoleyK {
    int nx, ny, nh;
    float eta, beta;
    float tanh_be;     // (float) tanh(beta*eta), formed in double like numpy
    float den;         // (float) (tanh(beta*eta) + tanh(beta*(1-eta)))
    float c0, dc;      // c0 and (float)(c1 - c0) formed in double
};

constexpr int HOLEY_THREADS = 256;
constexpr int HOLEY_MAX_BLOCKS = 4 * 152;

// exp(-|(fi, fj) - (xk, yk)| / rk) with the distance and its components.
WT_DEV float hole_exp(float fi, float fj, float xk, float yk, float rk, float& dist, float& dx,
                      float& dy) {
    dx = fsub(fi, xk);
    dy = fsub(fj, yk);
    dist = __fsqrt_rn(fadd(fmul(dx, dx), fmul(dy, dy)));
    return (float)exp((double)fdiv(-dist, rk));
}

__global__ void __launch_bounds__(HOLEY_THREADS)
holey_fwd_kernel(HoleyK g, const float* __restrict__ hx, const float* __restrict__ hy,
                 const float* __restrict__ hr, float* __restrict__ rho, float* __restrict__ c,
                 float* __restrict__ th_out) {
    const size_t n = (size_t)g.nx * g.ny;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
        const float fi = (float)(int)(q / g.ny), fj = (float)(int)(q % g.ny);
        float s = 0.f, d, a, b;
        for (int k = 0; k < g.nh; ++k)
            s = fadd(s, hole_exp(fi, fj, __ldg(hx + k), __ldg(hy + k), __ldg(hr + k), d, a, b));
        const float th = (float)tanh((double)fmul(g.beta, fsub(s, g.eta)));
        th_out[q] = th;
        const float P = fdiv(fadd(th, g.tanh_be), g.den);
        if (rho) rho[q] = P;
        if (c) c[q] = fadd(g.c0, fmul(g.dc, P));
    }
}

// Block sum of three doubles; thread 0 receives the totals (warps added in
// warp order).  `red` holds 3 x (blockDim.x / 32) doubles.
WT_DEV void block_sum3(double& a, double& b, double& c, double* red) {
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[w] = a;
        red[nw + w] = b;
        red[2 * nw + w] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        a = b = c = 0.0;
        for (int i = 0; i < nw; ++i) {
            a += red[i];
            b += red[nw + i];
            c += red[2 * nw + i];
        }
    }
    __syncthreads();
}

// partial[(block * nh + k) * 3 + {0,1,2}] = this block's sums of the cells'
// contributions to dL/dx_k, dL/dy_k, dL/dr_k.
__global__ void __launch_bounds__(HOLEY_THREADS)
holey_bwd_kernel(HoleyK g, const float* __restrict__ hx, const float* __restrict__ hy,
                 const float* __restrict__ hr, const float* __restrict__ grho,
                 const float* __restrict__ gc, const float* __restrict__ th,
                 double* __restrict__ partial) {
    __shared__ double red[3 * (HOLEY_THREADS / 32)];
    const size_t n = (size_t)g.nx * g.ny;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (int k = 0; k < g.nh; ++k) {
        const float xk = __ldg(hx + k), yk = __ldg(hy + k), rk = __ldg(hr + k);
        double ax = 0.0, ay = 0.0, ar = 0.0;
        for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
            // MulBackward (c1 - c0), DivBackward (den), TanhBackward, MulBackward (beta)
            const float gp = fadd(grho ? __ldg(grho + q) : 0.f, gc ? fmul(__ldg(gc + q), g.dc) : 0.f);
            const float t = __ldg(th + q);
            const float gs = fmul(fmul(fdiv(gp, g.den), fsub(1.0f, fmul(t, t))), g.beta);
            const float fi = (float)(int)(q / g.ny), fj = (float)(int)(q % g.ny);
            float d, a, b;
            const float e = hole_exp(fi, fj, xk, yk, rk, d, a, b);
            const float ge = fmul(gs, e);                               // ExpBackward
            const float gq = fdiv(ge, rk);                              // DivBackward, self
            const float grk = fmul(-ge, fdiv(fdiv(-d, rk), rk));        // DivBackward, other
            const float gd2 = fdiv(-gq, fmul(2.0f, d));                 // NegBackward, SqrtBackward
            ax += (double)(-fmul(gd2, fmul(2.0f, a)));                  // PowBackward, SubBackward
            ay += (double)(-fmul(gd2, fmul(2.0f, b)));
            ar += (double)grk;
        }
        block_sum3(ax, ay, ar, red);
        if (threadIdx.x == 0) {
            double* p = partial + ((size_t)blockIdx.x * g.nh + k) * 3;
            p[0] = ax;
            p[1] = ay;
            p[2] = ar;
        }
    }
}

__global__ void holey_reduce_kernel(int nblk, int nh, const double* __restrict__ partial,
                                    float* __restrict__ gx, float* __restrict__ gy,
                                    float* __restrict__ gr) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * nh) return;
    const int k = t / 3, comp = t % 3;
    double s = 0.0;
    for (int b = 0; b < nblk; ++b) s += partial[((size_t)b * nh + k) * 3 + comp];
    float* out = comp == 0 ? gx : (comp == 1 ? gy : gr);
    out[k] = (float)s;
}

}  // namespace wt

static int make_holeyk(const wt_holey_desc* d, wt::HoleyK* g) {
    if (!d || d->nx <= 0 || d->ny <= 0 || d->n_holes < 0) return WT_ERR_INVALID;
    g->nx = d->nx;
    g->ny = d->ny;
    g->nh = d->n_holes;
    g->eta = d->eta;
    g->beta = d->beta;
    const double be = (double)d->beta * (double)d->eta;
    const double b1 = (double)d->beta * (1.0 - (double)d->eta);
    g->tanh_be = (float)std::tanh(be);
    g->den = (float)(std::tanh(be) + std::tanh(b1));
    g->c0 = d->c0;
    g->dc = (float)((double)d->c1 - (double)d->c0);
    return WT_OK;
}

static size_t holey_cells(const wt::HoleyK& g) { return (size_t)g.nx * g.ny; }
static int holey_blocks(size_t n) {
    return (int)std::min<size_t>((n + wt::HOLEY_THREADS - 1) / wt::HOLEY_THREADS, wt::HOLEY_MAX_BLOCKS);
}
// tanh values first, the adjoint's partial sums after them (256-byte aligned)
static size_t holey_partial_offset(size_t n) { return (n * sizeof(float) + 255) & ~(size_t)255; }

extern "C" int wt_holey_work_bytes(const wt_holey_desc* d, size_t* bytes) {
    wt::HoleyK g;
    int st = make_holeyk(d, &g);
    if (st) return st;
    if (!bytes) return WT_ERR_INVALID;
    const size_t n = holey_cells(g);
    *bytes = holey_partial_offset(n) + (size_t)holey_blocks(n) * g.nh * 3 * sizeof(double);
    return WT_OK;
}

extern "C" int wt_holey_fwd(const wt_holey_desc* d, const float* x, const float* y, const float* r,
                            float* rho, float* c, float* work, wt_stream_t stream) {
    wt::HoleyK g;
    int st = make_holeyk(d, &g);
    if (st) return st;
    if (!work || (g.nh > 0 && (!x || !y || !r))) return WT_ERR_INVALID;
    const size_t n = holey_cells(g);
    wt::holey_fwd_kernel<<<holey_blocks(n), wt::HOLEY_THREADS, 0, (cudaStream_t)stream>>>(
        g, x, y, r, rho, c, work);
    wt_count_launches(1);
    return wt_cuda_status(cudaGetLastError());
}

extern "C" int wt_holey_bwd(const wt_holey_desc* d, const float* x, const float* y, const float* r,
                            const float* grad_rho, const float* grad_c, float* grad_x,
                            float* grad_y, float* grad_r, float* work, wt_stream_t stream) {
    wt::HoleyK g;
    int st = make_holeyk(d, &g);
    if (st) return st;
    if (!work || (!grad_rho && !grad_c)) return WT_ERR_INVALID;
    if (reinterpret_cast<uintptr_t>(work) % alignof(double)) return WT_ERR_INVALID;
    if (g.nh == 0) return WT_OK;
    if (!x || !y || !r || !grad_x || !grad_y || !grad_r) return WT_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = holey_cells(g);
    const int nblk = holey_blocks(n);
    double* partial = reinterpret_cast<double*>(reinterpret_cast<char*>(work) + holey_partial_offset(n));
    wt::holey_bwd_kernel<<<nblk, wt::HOLEY_THREADS, 0, s>>>(g, x, y, r, grad_rho, grad_c, work,
                                                            partial);
    wt::holey_reduce_kernel<<<(3 * g.nh + 127) / 128, 128, 0, s>>>(nblk, g.nh, partial, grad_x,
                                                                   grad_y, grad_r);
    wt_count_launches(2);
    return wt_cuda_status(cudaGetLastError());
}
