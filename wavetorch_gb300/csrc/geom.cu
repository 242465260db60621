// Free-form geometry parameterisation rho -> c and its adjoint
// (wavetorch/geom.py:207-233):
//   c = c0 + (c1 - c0) * P(blur^n(rho))
//   P(r) = (tanh(beta*eta) + tanh(beta*(r - eta))) / (tanh(beta*eta) + tanh(beta*(1 - eta)))
// blur = zero-padded 2-D convolution with the geometry's (2R+1)^2 kernel.
//
// The blur accumulates its taps row-major with fused multiply-adds, the order
// oneDNN uses for this single-channel convolution (bit-identical to the
// reference for grids above 20480 cells; below that the reference's
// im2col+GEMM path rounds differently by at most one ulp of the blurred
// density).  tanh is evaluated in double precision and rounded to float.
#include "common.cuh"

namespace wt {

struct GeomK {
    int nx, ny, rad;
    float eta, beta;
    float tanh_be;     // (float) tanh(beta*eta), formed in double like numpy
    float den;         // (float) (tanh(beta*eta) + tanh(beta*(1-eta)))
    float c0, dc;      // c0 and (float)(c1 - c0) formed in double
};

__global__ void blur_fwd_kernel(GeomK g, const float* __restrict__ in, const float* __restrict__ w,
                                float* __restrict__ out) {
    int y = blockIdx.x * blockDim.x + threadIdx.x;
    int x = blockIdx.y;
    if (y >= g.ny) return;
    const int K = 2 * g.rad + 1;
    float acc = 0.f;
    for (int kh = 0; kh < K; ++kh) {
        int sx = x + kh - g.rad;
        for (int kw = 0; kw < K; ++kw) {
            int sy = y + kw - g.rad;
            float v = (sx >= 0 && sx < g.nx && sy >= 0 && sy < g.ny) ? __ldg(in + (size_t)sx * g.ny + sy) : 0.f;
            acc = ffma(__ldg(w + kh * K + kw), v, acc);
        }
    }
    out[(size_t)x * g.ny + y] = acc;
}

// Transposed blur (the input-gradient of conv2d): im2col/col2im order, taps
// (kh, kw) row-major, each product rounded, sums accumulated from zero.
__global__ void blur_bwd_kernel(GeomK g, const float* __restrict__ gin, const float* __restrict__ w,
                                float* __restrict__ gout) {
    int y = blockIdx.x * blockDim.x + threadIdx.x;
    int x = blockIdx.y;
    if (y >= g.ny) return;
    const int K = 2 * g.rad + 1;
    float acc = 0.f;
    for (int kh = 0; kh < K; ++kh) {
        int sx = x - kh + g.rad;
        for (int kw = 0; kw < K; ++kw) {
            int sy = y - kw + g.rad;
            float v = (sx >= 0 && sx < g.nx && sy >= 0 && sy < g.ny) ? __ldg(gin + (size_t)sx * g.ny + sy) : 0.f;
            acc = fadd(acc, fmul(__ldg(w + kh * K + kw), v));
        }
    }
    gout[(size_t)x * g.ny + y] = acc;
}

// Projection and affine map to c; keeps tanh(beta*(r-eta)) for the adjoint.
__global__ void project_fwd_kernel(GeomK g, const float* __restrict__ r, float* __restrict__ th_out,
                                   float* __restrict__ c) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)g.nx * g.ny) return;
    float z = fmul(g.beta, fsub(__ldg(r + i), g.eta));
    // tanh evaluated in double and rounded once: agrees with the reference's
    // float32 tanh (a < 1 ulp vectorised implementation) in all but a few
    // arguments per thousand, where tanhf would differ in about a third
    float th = (float)tanh((double)z);
    th_out[i] = th;
    float P = fdiv(fadd(th, g.tanh_be), g.den);
    c[i] = fadd(g.c0, fmul(g.dc, P));
}

// Adjoint of the projection and affine map: autograd's chain
//   MulBackward (dc) -> DivBackward (den) -> TanhBackward (1 - th^2) -> MulBackward (beta)
__global__ void project_bwd_kernel(GeomK g, const float* __restrict__ gc, const float* __restrict__ th,
                                   float* __restrict__ gr) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)g.nx * g.ny) return;
    float t = __ldg(th + i);
    float gp = fdiv(fmul(__ldg(gc + i), g.dc), g.den);
    float gz = fmul(gp, fsub(1.0f, fmul(t, t)));
    gr[i] = fmul(gz, g.beta);
}

}  // namespace wt

#include <cmath>

static int make_geomk(const wt_geom_desc* d, wt::GeomK* g) {
    if (!d || d->nx <= 0 || d->ny <= 0 || d->blur_radius < 0 || d->blur_n < 0) return WT_ERR_INVALID;
    g->nx = d->nx;
    g->ny = d->ny;
    g->rad = d->blur_radius;
    g->eta = d->eta;
    g->beta = d->beta;
    double be = (double)d->beta * (double)d->eta;
    double b1 = (double)d->beta * (1.0 - (double)d->eta);
    g->tanh_be = (float)std::tanh(be);
    g->den = (float)(std::tanh(be) + std::tanh(b1));
    g->c0 = d->c0;
    g->dc = (float)((double)d->c1 - (double)d->c0);
    return WT_OK;
}

extern "C" int wt_rho_to_c_work_bytes(const wt_geom_desc* d, size_t* bytes) {
    if (!d || !bytes || d->nx <= 0 || d->ny <= 0 || d->blur_n < 0) return WT_ERR_INVALID;
    *bytes = (size_t)2 * d->nx * d->ny * sizeof(float);
    return WT_OK;
}

extern "C" int wt_rho_to_c_fwd(const wt_geom_desc* d, const float* rho, const float* blur_kernel,
                               float* c, float* work, wt_stream_t stream) {
    wt::GeomK g;
    int st = make_geomk(d, &g);
    if (st) return st;
    if (!rho || !c || !work || (d->blur_n > 0 && !blur_kernel)) return WT_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)g.nx * g.ny;
    float* th = work;          // tanh values
    float* tmp = work + n;     // blurred density
    dim3 blk(128), grd((g.ny + 127) / 128, g.nx);
    // blur passes ping-pong between tmp and c (c is overwritten last)
    const float* src = rho;
    for (int p = 0; p < d->blur_n; ++p) {
        float* dst = (p % 2 == 0) ? tmp : c;
        wt::blur_fwd_kernel<<<grd, blk, 0, s>>>(g, src, blur_kernel, dst);
        wt_count_launches(1);
        src = dst;
    }
    if (d->blur_n > 0 && src == c) {
        cudaError_t e = cudaMemcpyAsync(tmp, c, n * sizeof(float), cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return wt_cuda_status(e);
        src = tmp;
    }
    wt::project_fwd_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, src, th, c);
    wt_count_launches(1);
    return wt_cuda_status(cudaGetLastError());
}

extern "C" int wt_rho_to_c_bwd(const wt_geom_desc* d, const float* rho, const float* blur_kernel,
                               const float* grad_c, float* grad_rho, float* work,
                               wt_stream_t stream) {
    (void)rho;
    wt::GeomK g;
    int st = make_geomk(d, &g);
    if (st) return st;
    if (!grad_c || !grad_rho || !work || (d->blur_n > 0 && !blur_kernel)) return WT_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)g.nx * g.ny;
    const float* th = work;
    float* tmp = work + n;     // the forward's blurred density is no longer needed
    dim3 blk(128), grd((g.ny + 127) / 128, g.nx);
    // projection adjoint into grad_rho (or tmp when passes follow)
    float* dst0 = d->blur_n % 2 == 1 ? tmp : grad_rho;
    wt::project_bwd_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, grad_c, th, dst0);
    wt_count_launches(1);
    const float* src = dst0;
    for (int p = 0; p < d->blur_n; ++p) {
        float* dst = (src == tmp) ? grad_rho : tmp;
        wt::blur_bwd_kernel<<<grd, blk, 0, s>>>(g, src, blur_kernel, dst);
        wt_count_launches(1);
        src = dst;
    }
    // with blur_n passes the result alternates; it always ends in grad_rho:
    // odd n starts in tmp and ends in grad_rho, even n starts and ends in grad_rho.
    return wt_cuda_status(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// wt_rho_to_c_fwd_noalloc: the same forward with its scratch (tanh values and
// blurred density, 2 floats per cell) in this file-scope array instead of a
// caller-owned buffer.  Each device has its own copy.  Its address on the
// current device is looked up on every call (cudaGetSymbolAddress allocates
// nothing), so no cached address can outlive a device reset or a re-created
// primary context.
static __device__ __align__(256) float g_rho_to_c_scratch[2 * (size_t)WT_RHO_TO_C_NOALLOC_MAX_CELLS];

// Address of the current device's scratch array.
static int noalloc_scratch(float** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_rho_to_c_scratch);
    if (e != cudaSuccess) return wt_cuda_status(e);
    *out = static_cast<float*>(p);
    return WT_OK;
}

extern "C" int wt_rho_to_c_fwd_noalloc(const wt_geom_desc* d, const float* rho,
                                       const float* blur_kernel, float* c, wt_stream_t stream) {
    if (!d || d->nx <= 0 || d->ny <= 0) return WT_ERR_INVALID;
    if ((size_t)d->nx * (size_t)d->ny > (size_t)WT_RHO_TO_C_NOALLOC_MAX_CELLS)
        return WT_ERR_UNSUPPORTED;
    if (!rho || !c || (d->blur_n > 0 && !blur_kernel)) return WT_ERR_INVALID;
    float* work = nullptr;
    int st = noalloc_scratch(&work);
    if (st) return st;
    return wt_rho_to_c_fwd(d, rho, blur_kernel, c, work, stream);
}
