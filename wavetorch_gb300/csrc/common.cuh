// Shared device helpers for the wavetorch_gb300 kernels (sm_103a).
//
// All parity-relevant float arithmetic goes through the explicit round-to-
// nearest intrinsics below, so the compiler can never contract a multiply and
// an add into one FMA where the reference rounds twice.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/wavetorch_gb300.h"

#define WT_DEV __device__ __forceinline__

WT_DEV float fmul(float a, float b) { return __fmul_rn(a, b); }
WT_DEV float fadd(float a, float b) { return __fadd_rn(a, b); }
WT_DEV float fsub(float a, float b) { return __fsub_rn(a, b); }
WT_DEV float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
WT_DEV float fdiv(float a, float b) { return __fdiv_rn(a, b); }

// Per-launch scalars of the leapfrog update, formed on the host exactly as the
// reference forms them from its float32 0-d tensors (wavetorch/cell.py:12-17,
// :33-42; wavetorch/operators.py:7).
struct StepScalars {
    float inv_dt2;   // dt**-2        = 1/(dt*dt)
    float inv_dt;    // dt**-1        = 1/dt
    float two_over;  // 2 / dt**2     = reciprocal(dt*dt) * 2
    float dt;        // dt
    float dt2;       // dt**2         = dt*dt
    float lap_w;     // h**-2         = 1/(h*h)
    float lap_w4;    // h**-2 * -4
    int lap_order;   // WT_LAP_SEQ / WT_LAP_PAIRED, | WT_LAP_UNIT when lap_w == 1
};

// Internal Laplacian orders: WT_LAP_SEQ / WT_LAP_PAIRED plus this flag when
// the tap weight h**-2 is exactly 1 (h == 1).  Then w*v == v exactly and
// fma(1, v, a) rounds as v + a, so the unit-weight forms drop the
// multiplications by w and give the same bits with fewer instructions.
constexpr int WT_LAP_UNIT = 2;

// 5-point Laplacian with the association order of the reference's conv2d.
// u = (x-1,y), l = (x,y-1), c = (x,y), r = (x,y+1), d = (x+1,y).
template <int ORDER>
WT_DEV float lap5(float u, float l, float c, float r, float d, float w, float w4) {
    if constexpr (ORDER == (WT_LAP_SEQ | WT_LAP_UNIT)) {
        float acc = fadd(u, l);
        acc = ffma(w4, c, acc);
        acc = fadd(acc, r);
        return fadd(acc, d);
    } else if constexpr (ORDER == (WT_LAP_PAIRED | WT_LAP_UNIT)) {
        const float ul = fadd(u, l);
        const float rd = fadd(r, d);
        return fadd(ul, fadd(fmul(w4, c), rd));
    } else if constexpr (ORDER == WT_LAP_SEQ) {
        float acc = fmul(w, u);
        acc = ffma(w, l, acc);
        acc = ffma(w4, c, acc);
        acc = ffma(w, r, acc);
        return ffma(w, d, acc);
    } else {
        // im2col+GEMM order of the reference's B=1 small-grid path (taps are
        // exact for h == 1, the only case the host selects it for)
        float ul = fadd(fmul(w, u), fmul(w, l));
        float rd = fadd(fmul(w, r), fmul(w, d));
        return fadd(ul, fadd(fmul(w4, c), rd));
    }
}

// Leapfrog update in the reference's order (wavetorch/cell.py:13-16):
//   A * ( (two_over*y1 - Bc*y2) + c2*L )
WT_DEV float leapfrog(float A, float Bc, float c2, float two_over, float y1, float y2, float L) {
    float s = fsub(fmul(two_over, y1), fmul(Bc, y2));
    s = fadd(s, fmul(c2, L));
    return fmul(A, s);
}

// Time-invariant coefficient fields of one cell (b, c -> A, Bc, c2, ...),
// formed as the reference forms them every step.
struct FwdCoef { float A, Bc, c2; };
WT_DEV FwdCoef fwd_coef(float b, float c, const StepScalars& s) {
    float bd = fmul(b, s.inv_dt);                 // b * dt**-1
    FwdCoef k;
    k.A = fdiv(1.0f, fadd(s.inv_dt2, bd));        // (dt**-2 + b*dt**-1).pow(-1)
    k.Bc = fsub(s.inv_dt2, bd);                   // dt**-2 - b*dt**-1
    k.c2 = fmul(c, c);                            // c.pow(2)
    return k;
}

// Adjoint coefficients (wavetorch/cell.py:33-42):
//   X1  = (b*dt + 1).pow(-1)
//   Kc  = 2*c*dt**2                (grad_c = (X1 * (Kc * Lap(y1))) * g)
//   Kg  = X1 * c.pow(2)            (c2_grad = Kg * g)
//   Ky2 = (b*dt - 1) * X1          (grad_y2 = Ky2 * g)
//   Kb0 = -(dt*b + 1).pow(-2)      (grad_b = ((Kb0*dt) * (...)) * g)
struct BwdCoef { float X1, Kc, Kg, Ky2; };
WT_DEV BwdCoef bwd_coef(float b, float c, const StepScalars& s) {
    float bdt = fmul(b, s.dt);
    BwdCoef k;
    k.X1 = fdiv(1.0f, fadd(bdt, 1.0f));
    k.Kc = fmul(fmul(2.0f, c), s.dt2);
    k.Kg = fmul(k.X1, fmul(c, c));
    k.Ky2 = fmul(fsub(bdt, 1.0f), k.X1);
    return k;
}

// ---- error reporting from device code ------------------------------------
// Kernels never trap: a bounded wait that gives up, or an index check that
// fails, records a code in this word and the kernel returns.  The host reads
// it back after the launch.
#define WT_DEVERR_NONE 0
#define WT_DEVERR_TIMEOUT 1
#define WT_DEVERR_BOUNDS 2

// ---- thread-block cluster helpers (inline PTX) ----------------------------
WT_DEV uint32_t cluster_ctarank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// Map a local shared-memory address to the same offset in CTA `rank` of the
// cluster (a 32-bit shared::cluster address).
WT_DEV uint32_t map_shared_rank(const void* local_smem, uint32_t rank) {
    uint32_t a = (uint32_t)__cvta_generic_to_shared(local_smem);
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
WT_DEV void cluster_arrive_release() {
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
WT_DEV void cluster_wait_acquire() {
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
WT_DEV void cluster_sync_all() {
    cluster_arrive_release();
    cluster_wait_acquire();
}

// ---- mbarrier / asynchronous DSMEM store helpers (inline PTX, sm_90+) ------
WT_DEV uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
WT_DEV void mbar_init(uint32_t addr, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(addr), "r"(count) : "memory");
}
WT_DEV void fence_mbarrier_init_cluster() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// One local arrival that also raises the phase's expected transaction bytes.
WT_DEV void mbar_arrive_expect_tx(uint32_t addr, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\t"
                 "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(addr),
                 "r"(bytes)
                 : "memory");
}
// Probe of phase completion with acquire semantics at CTA scope: enough for
// data a bulk copy wrote into this CTA's own shared memory.
WT_DEV bool mbar_try_wait_parity_cta(uint32_t addr, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(addr), "r"(parity)
                 : "memory");
    return ok != 0;
}
// Relaxed 8-byte store into another CTA's shared memory (shared::cluster
// address) and relaxed 8-byte load from this CTA's shared memory; aligned
// 8-byte accesses are single-copy atomic, so a {value, tag} word is never torn.
WT_DEV void st_cluster_u64(uint32_t remote, unsigned long long v) {
    asm volatile("st.relaxed.cluster.shared::cluster.b64 [%0], %1;" ::"r"(remote), "l"(v) : "memory");
}
WT_DEV unsigned long long ld_cluster_u64(uint32_t local) {
    unsigned long long v;
    asm volatile("ld.relaxed.cluster.shared::cta.b64 %0, [%1];" : "=l"(v) : "r"(local) : "memory");
    return v;
}
// Order this thread's earlier generic-proxy shared-memory accesses before
// later asynchronous-proxy (bulk copy) accesses to the same memory.
WT_DEV void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// Bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned)
// from global memory into this CTA's shared memory; completion is counted
// as transaction bytes on the mbarrier at `mbar`.
WT_DEV void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(mbar)
        : "memory");
}
WT_DEV uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Host-side helpers shared by the translation units (defined in api.cu).
StepScalars wt_make_scalars(const wt_scalars* s);
int wt_cuda_status(cudaError_t e);
// Count `n` kernel launches (wt_kernel_launches).
void wt_count_launches(unsigned n);
