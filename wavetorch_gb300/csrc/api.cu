// extern "C" entry points declared in include/wavetorch_gb300.h: argument
// validation, workspace layout, host-side tables and kernel launches.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "internal.cuh"
#include "../../include/wavetorch_gb300_testing.h"

// ---------------------------------------------------------------------------
static thread_local char g_last_err[256] = "";

int wt_cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return WT_OK;
    std::snprintf(g_last_err, sizeof(g_last_err), "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
    return WT_ERR_CUDA;
}

StepScalars wt_make_scalars(const wt_scalars* s) {
    // float32 arithmetic in the reference's order (torch pow(-2) on a float
    // tensor is 1/(x*x), pow(-1) is 1/x, `2 / t` is reciprocal(t) * 2)
    StepScalars k;
    const float dt = s->dt, h = s->h;
    const float dtdt = dt * dt;
    k.inv_dt2 = 1.0f / dtdt;
    k.inv_dt = 1.0f / dt;
    k.two_over = (1.0f / dtdt) * 2.0f;
    k.dt = dt;
    k.dt2 = dtdt;
    const float hh = h * h;
    k.lap_w = 1.0f / hh;
    k.lap_w4 = k.lap_w * -4.0f;
    k.lap_order = s->lap_order | (k.lap_w == 1.0f ? WT_LAP_UNIT : 0);
    return k;
}

// WT_LAP_PAIRED is the order of the reference's im2col path, which it takes
// for h == 1 only (h**-2 must be exactly 1: the kernels then add the taps
// without multiplying them).
static bool scalars_ok(const wt_scalars* s) {
    return s && std::isfinite(s->dt) && s->dt > 0.f && std::isfinite(s->h) && s->h > 0.f &&
           (s->lap_order == WT_LAP_SEQ ||
            (s->lap_order == WT_LAP_PAIRED && 1.0f / (s->h * s->h) == 1.0f));
}

extern "C" const char* wt_version(void) { return "wavetorch_gb300 0.1.0 sm_103a"; }

extern "C" const char* wt_status_string(int status) {
    switch (status) {
        case WT_OK: return "ok";
        case WT_ERR_INVALID: return "invalid argument";
        case WT_ERR_CUDA: return "CUDA runtime error";
        case WT_ERR_TIMEOUT: return "device-side wait timed out";
        case WT_ERR_UNSUPPORTED: return "unsupported configuration";
        default: return "unknown status";
    }
}

extern "C" const char* wt_last_error(void) { return g_last_err; }

#include <atomic>
static std::atomic<uint64_t> g_launches{0};
void wt_count_launches(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
extern "C" uint64_t wt_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

// ---------------------------------------------------------------------------
// 1. single step
extern "C" int wt_step_fwd(const wt_scalars* s, int32_t batch, int32_t nx, int32_t ny,
                           int32_t coef_batched, const float* b, const float* c,
                           const float* y1, const float* y2, float* y, wt_stream_t stream) {
    if (!scalars_ok(s) || batch <= 0 || nx <= 0 || ny <= 0 || !b || !c || !y1 || !y2 || !y)
        return WT_ERR_INVALID;
    if (y == y1 || y == y2) return WT_ERR_INVALID;   // the stencil reads y1 halos
    const size_t plane = (size_t)nx * ny;
    return wt_launch_step_fwd(wt_make_scalars(s), batch, nx, ny, coef_batched ? 1 : 0, b, c, y1,
                              plane, y2, plane, y, plane, nullptr, (cudaStream_t)stream);
}

extern "C" int wt_step_bwd(const wt_scalars* s, int32_t batch, int32_t nx, int32_t ny,
                           int32_t coef_batched, const float* b, const float* c,
                           const float* y1, const float* y2, const float* grad_y,
                           float* grad_b, float* grad_c, float* grad_y1, float* grad_y2,
                           wt_stream_t stream) {
    if (!scalars_ok(s) || batch <= 0 || nx <= 0 || ny <= 0 || !b || !c || !y1 || !y2 || !grad_y)
        return WT_ERR_INVALID;
    if (!grad_b && !grad_c && !grad_y1 && !grad_y2) return WT_OK;
    return wt_launch_step_bwd(wt_make_scalars(s), batch, nx, ny, coef_batched ? 1 : 0, b, c, y1,
                              y2, grad_y, grad_b, grad_c, grad_y1, grad_y2, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// 2. sequences: workspace plan
namespace {

constexpr size_t ALIGN = 256;
// Automatic choice of the fused adjoint's mode: the tape (every step's
// Laplacian, T x batch x nx x pitch floats) when it takes at most this many
// bytes, else checkpoints with segment recompute.
constexpr size_t WT_TAPE_AUTO_MAX_BYTES = (size_t)16 << 30;
// The same choice in the band layout (grids larger than a cluster holds,
// whose tapes are large: 31 GiB at 1024 x 1024, T=8000).
constexpr size_t WT_BAND_TAPE_AUTO_MAX_BYTES = (size_t)64 << 30;
size_t up(size_t v) { return (v + ALIGN - 1) / ALIGN * ALIGN; }

struct SeqPlan {
    int B, nx, ny, T, ns, np, form, coef_batched;
    size_t plane;
    // int tables
    size_t o_srcmap, o_srcnext, o_srcrow, o_srccell;
    size_t o_prbmap, o_prbnext, o_prbkind;          // entry index == output column
    size_t o_fcell, o_fkind, o_fcol;                // probes, descending reference order
    size_t o_err;
    size_t o_tileflag;                              // plain: tiles of the vector kernels
    int tiles_x, tiles_y;
    size_t tables_end;
    // float areas
    size_t o_amp;
    size_t o_hist, o_zero, o_lam, o_gc, o_kco;      // plain
    size_t o_fco;                                   // plain: the forward's coefficient planes
    size_t o_ckpt, o_stash, o_gcpart, o_lap, o_grho; // fused
    size_t o_halo;                                  // fused, band layout
    size_t o_bstate;                                // band layout from checkpoints:
                                                    // the adjoint's saved state
    size_t o_rfirst, o_ritems;                      // band layout in rounds: the work list
    int rctas;                                      // CTAs of the rounds (0: one launch of
                                                    // batch x bands CTAs)
    size_t total;
    int seg, nseg;
    bool tape;                                      // fused: tape mode
    bool band;                                      // fused: band layout
    WtFusedLaunch L;
    WtBandLaunch BL;
};

// SMs of the band layout: the descriptor's count, else the current device's
// (0 when there is no device).
int band_sms(const wt_seq_desc* d) {
    if (d->sm_count > 0) return d->sm_count;
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();   // leave no sticky error behind
        return 0;
    }
    return n;
}

// Workspace of the band layout after the shared tables (offset o): the tape
// (every step's Laplacian, [step][batch][band][M][threads]) or, from
// checkpoints, the pairs (h_{t-1}, h_{t-2}) every `seg` steps
// ([nseg][2][batch][nx][ny]), one segment's stash of Laplacians (the tape's
// layout, seg steps deep) and the adjoint's state between its segment
// launches ([batch][band][3][M][threads]); then the exchange words and the
// per-instance dL/dc.  Sources and probes: at most two of each per thread.
int plan_band(const wt_seq_desc* d, SeqPlan& P, size_t o) {
    const WtBandLaunch& B = P.BL;
    const size_t F = sizeof(float);
    const size_t slice = (size_t)P.B * B.PR * B.threads * B.M * F;   // one step of tape
    P.band = true;
    P.tape = d->segment == -1 ||
             (d->segment == 0 && (size_t)P.T * slice <= WT_BAND_TAPE_AUTO_MAX_BYTES);
    if (P.tape) {
        P.seg = P.T;
        P.nseg = 1;
        P.o_lap = o; o = up(o + (size_t)P.T * slice);
    } else {
        P.seg = d->segment > 0 ? std::min(d->segment, P.T)
                               : std::max(1, (int)std::ceil(std::sqrt((double)P.T)));
        P.nseg = (P.T + P.seg - 1) / P.seg;
        P.o_ckpt = o; o = up(o + (size_t)P.nseg * 2 * P.B * P.plane * F);
        P.o_stash = o; o = up(o + (size_t)P.seg * slice);
        P.o_bstate = o; o = up(o + 3 * slice);
    }
    P.o_halo = o; o = up(o + wt_band_halo_bytes(P.B, B));
    P.o_gcpart = o; o = up(o + (size_t)P.B * P.plane * F);
    std::vector<int> cnt((size_t)B.PR * B.S * B.NCP, 0);
    auto key = [&](int cell) {
        const int gx = cell / P.ny, gy = cell % P.ny;
        return ((size_t)(gx / B.R) * B.S + (gx % B.R) / B.M) * B.NCP + gy;
    };
    for (int i = 0; i < P.ns; ++i)
        if (++cnt[key(d->sources_host[i].cell)] > 2) return WT_ERR_UNSUPPORTED;
    std::fill(cnt.begin(), cnt.end(), 0);
    for (int i = 0; i < P.np; ++i)
        if (++cnt[key(d->probes_host[i].cell)] > 2) return WT_ERR_UNSUPPORTED;
    P.total = o;
    return WT_OK;
}

// The band layout in rounds: instance i's band p is work item (i, p) on CTA
// (i * PR + p) % ctas, each CTA taking its items in instance order, so the
// bands of one instance run at once and the instances follow one another
// (the kernels' band bodies as a work list; see band_list_kernel).  The
// lists go into the int tables, which upload_tables writes.
int plan_rounds(const wt_seq_desc* d, SeqPlan& P, size_t o, int sms) {
    int st = plan_band(d, P, o);
    if (st) return st;
    P.rctas = std::min(sms, P.B * P.BL.PR);
    P.o_rfirst = up(P.total);
    P.o_ritems = up(P.o_rfirst + (size_t)(P.rctas + 1) * sizeof(int));
    P.total = up(P.o_ritems + (size_t)2 * P.B * P.BL.PR * sizeof(int));
    return WT_OK;
}

// Write the rounds' work list (first[ctas + 1], items (instance, band)) into
// the workspace with the scatter kernel (no host wait; capturable).
int upload_rounds(const SeqPlan& P, void* ws, cudaStream_t st) {
    const int PR = P.BL.PR, C = P.rctas, n = P.B * PR;
    std::vector<int> first(C + 1, 0), items(2 * (size_t)n);
    for (int k = 0; k < n; ++k) ++first[k % C + 1];
    for (int c = 0; c < C; ++c) first[c + 1] += first[c];
    std::vector<int> fill(first.begin(), first.end() - 1);
    for (int k = 0; k < n; ++k) {          // item k = (k / PR, k % PR), in instance order
        const int at_ = fill[k % C]++;
        items[2 * (size_t)at_] = k / PR;
        items[2 * (size_t)at_ + 1] = k % PR;
    }
    static thread_local wt::IntScatter sc;
    int* base = reinterpret_cast<int*>(static_cast<char*>(ws));
    auto flush = [&]() -> int {
        int rc = sc.n ? wt_launch_scatter_ints(base, sc, st) : WT_OK;
        sc.n = 0;
        return rc;
    };
    sc.n = 0;
    auto put = [&](size_t off_bytes, const std::vector<int>& v) -> int {
        for (size_t i = 0; i < v.size(); ++i) {
            if (sc.n == wt::INT_SCATTER_CAP) { int rc = flush(); if (rc) return rc; }
            sc.idx[sc.n] = (int)(off_bytes / sizeof(int) + i);
            sc.val[sc.n++] = v[i];
        }
        return WT_OK;
    };
    int rc = put(P.o_rfirst, first);
    if (!rc) rc = put(P.o_ritems, items);
    if (!rc) rc = flush();
    return rc;
}

int make_plan(const wt_seq_desc* d, SeqPlan* p, bool nl = false) {
    if (!d || d->batch <= 0 || d->nx <= 0 || d->ny <= 0 || d->steps <= 0) return WT_ERR_INVALID;
    if (d->n_sources < 0 || d->n_probes < 0) return WT_ERR_INVALID;
    if ((d->n_sources > 0 && !d->sources_host) || (d->n_probes > 0 && !d->probes_host))
        return WT_ERR_INVALID;
    if (d->form != WT_FORM_PLAIN && d->form != WT_FORM_FUSED) return WT_ERR_INVALID;
    if (d->coef_batched != 0 && d->coef_batched != 1) return WT_ERR_INVALID;
    if (d->sm_count < 0) return WT_ERR_INVALID;
    if (d->coef_batched && d->form != WT_FORM_FUSED) return WT_ERR_UNSUPPORTED;
    const long long cells = (long long)d->nx * d->ny;
    if (cells > (1LL << 30)) return WT_ERR_INVALID;
    for (int i = 0; i < d->n_sources; ++i) {
        const wt_source_entry& e = d->sources_host[i];
        if (e.cell < 0 || e.cell >= cells || e.in_row < -1 || e.in_row >= d->batch) return WT_ERR_INVALID;
    }
    for (int i = 0; i < d->n_probes; ++i) {
        const wt_probe_entry& e = d->probes_host[i];
        if (e.cell < 0 || e.cell >= cells || (e.kind != 0 && e.kind != 1)) return WT_ERR_INVALID;
    }
    SeqPlan& P = *p;
    std::memset(&P, 0, sizeof(P));
    P.B = d->batch; P.nx = d->nx; P.ny = d->ny; P.T = d->steps;
    P.ns = d->n_sources; P.np = d->n_probes; P.form = d->form;
    P.coef_batched = d->coef_batched;
    P.plane = (size_t)cells;
    const size_t I = sizeof(int), F = sizeof(float);
    size_t o = 0;
    P.o_srcmap = o; o = up(o + P.plane * I);
    P.o_srcnext = o; o = up(o + (P.ns + 1) * I);
    P.o_srcrow = o; o = up(o + (P.ns + 1) * I);
    P.o_srccell = o; o = up(o + (P.ns + 1) * I);
    P.o_prbmap = o; o = up(o + P.plane * I);
    P.o_prbnext = o; o = up(o + (P.np + 1) * I);
    P.o_prbkind = o; o = up(o + (P.np + 1) * I);
    P.o_fcell = o; o = up(o + (P.np + 1) * I);
    P.o_fkind = o; o = up(o + (P.np + 1) * I);
    P.o_fcol = o; o = up(o + (P.np + 1) * I);
    P.o_err = o; o = up(o + I);
    P.tiles_x = (P.nx + wt::STEP4_TX - 1) / wt::STEP4_TX;
    P.tiles_y = (P.ny + wt::STEP4_TY - 1) / wt::STEP4_TY;
    P.o_tileflag = o; o = up(o + (size_t)P.tiles_x * P.tiles_y * I);
    P.tables_end = o;
    const size_t bp = (size_t)P.B * P.plane;
    P.o_amp = o; o = up(o + (size_t)P.B * P.T * (P.np + 1) * F);
    if (P.form == WT_FORM_PLAIN) {
        P.o_hist = o; o = up(o + (size_t)P.T * bp * F);
        P.o_zero = o; o = up(o + P.plane * F);
        P.o_lam = o; o = up(o + 3 * bp * F);
        P.o_gc = o; o = up(o + bp * F);
        P.o_kco = o; o = up(o + 4 * P.plane * F);
        P.o_fco = o; o = up(o + 3 * P.plane * F);
    } else {
        if (d->segment < -2 || d->cluster < -1) return WT_ERR_INVALID;
        // cluster -1 asks for the band layout; 0 takes a cluster when one
        // holds the instance, else bands
        int st = d->cluster == -1 ? (int)WT_ERR_UNSUPPORTED
                                  : wt_fused_plan(P.nx, P.ny, P.T, P.np, d->cluster, d->segment, &P.L);
        if (st == WT_ERR_UNSUPPORTED && !nl && d->cluster <= 0 && !d->output_fields) {
            // too large for one cluster: bands of rows, one CTA per band
            const int sms = band_sms(d);
            if (sms > 0 && wt_band_plan(P.B, P.nx, P.ny, P.np, sms, &P.BL) == WT_OK)
                return plan_band(d, P, o);
            // more bands than SMs for the whole batch: one instance's bands on
            // the SMs, the instances in rounds (a work list, see plan_rounds)
            if (sms > 0 && P.B > 1 && wt_band_plan(1, P.nx, P.ny, P.np, sms, &P.BL) == WT_OK)
                return plan_rounds(d, P, o, sms);
        }
        if (st) return st;
        const size_t tape_bytes = (size_t)(nl ? 2 : 1) * P.T * P.B * P.L.C * P.L.threads * P.L.M * F;
        if (nl) {
            // the nonlinear adjoint runs from a two-part tape only (it reads
            // the field of the next slot as well, so at least 3 slots)
            if (d->segment > 0 || d->segment == -2 || d->output_fields || P.L.nbuf_nl < 3)
                return WT_ERR_UNSUPPORTED;
            P.L.nbuf = P.L.nbuf_nl;
            P.tape = true;
        } else {
            // automatic mode: no tape next to field outputs (the caller
            // already receives every field; checkpoints cost 2/seg of them)
            P.tape = P.L.nbuf >= 2 &&
                     (d->segment == -1 || (d->segment == 0 && !d->output_fields &&
                                           tape_bytes <= WT_TAPE_AUTO_MAX_BYTES));
        }
        if (d->segment == -1 && !P.tape) return WT_ERR_UNSUPPORTED;
        if (P.tape) {
            // the forward runs on the adjoint's strips so that the tape's
            // per-thread layout is the same on both sides
            P.L.fM = P.L.M; P.L.fR = P.L.R; P.L.fS = P.L.S; P.L.fLD = P.L.LD;
            P.L.fthreads = P.L.threads;
            P.L.smem_fwd = P.L.smem_fwd_tape;
            P.seg = P.T;      // no checkpoints
            P.nseg = 1;
            P.o_lap = o; o = up(o + tape_bytes);
        } else {
            const size_t per_step = (size_t)P.B * P.L.C * P.L.M * P.L.threads * F;
            // the recompute beside the adjoint where its kernel fits (a
            // sqrt(T) interval unless asked; the stash holds two segments in
            // global memory), else the recompute before each segment's
            // adjoint steps
            WtFusedLaunch W = P.L;
            W.seg = d->segment > 0 ? std::min(d->segment, P.T)
                                   : std::max(1, (int)std::ceil(std::sqrt((double)P.T)));
            if (wt_ws_plan(P.B, P.ny, P.np, &W) == WT_OK) {
                P.L = W;
                P.L.ws = 1;
                P.L.stash_smem = 0;
            }
            P.seg = P.L.seg;
            P.nseg = (P.T + P.seg - 1) / P.seg;
            P.o_ckpt = o; o = up(o + (size_t)P.nseg * 2 * bp * F);
            P.o_stash = o;
            o = up(o + (P.L.ws ? 2 * (size_t)P.seg * per_step
                               : P.L.stash_smem ? 0 : (size_t)P.seg * per_step));
        }
        P.o_gcpart = o; o = up(o + bp * F);
        if (nl) { P.o_grho = o; o = up(o + bp * F); }
        // per-thread tap capacity of both fused kernels (4 sources, 4 probes)
        for (int layout = 0; layout < 2; ++layout) {
            const int R = layout ? P.L.fR : P.L.R, M = layout ? P.L.fM : P.L.M;
            const int S = R / M;
            std::vector<int> cnt((size_t)P.L.C * S * P.L.NCP, 0);
            auto key = [&](int cell) {
                int gx = cell / P.ny, gy = cell % P.ny;
                int cta = gx / R, strip = (gx % R) / M;
                return ((size_t)cta * S + strip) * P.L.NCP + gy;
            };
            for (int i = 0; i < P.ns; ++i)
                if (++cnt[key(d->sources_host[i].cell)] > 4) return WT_ERR_UNSUPPORTED;
            std::fill(cnt.begin(), cnt.end(), 0);
            for (int i = 0; i < P.np; ++i)
                if (++cnt[key(d->probes_host[i].cell)] > 4) return WT_ERR_UNSUPPORTED;
        }
    }
    P.total = o;
    return WT_OK;
}

template <class T>
T* at(void* ws, size_t off) { return reinterpret_cast<T*>(static_cast<char*>(ws) + off); }

// Build and upload the lookup tables (sources in table order; probes linked
// per cell in descending reference order).
int upload_tables(const wt_seq_desc* d, const SeqPlan& P, void* ws, cudaStream_t st) {
    std::vector<int> h(P.tables_end / sizeof(int), 0);
    auto H = [&](size_t off) { return h.data() + off / sizeof(int); };
    std::fill(H(P.o_srcmap), H(P.o_srcmap) + P.plane, -1);
    std::fill(H(P.o_prbmap), H(P.o_prbmap) + P.plane, -1);
    // sources: per-cell chains in table order
    std::vector<int> tail(P.plane, -1);
    for (int i = 0; i < P.ns; ++i) {
        const wt_source_entry& e = d->sources_host[i];
        H(P.o_srcnext)[i] = -1;
        H(P.o_srcrow)[i] = e.in_row;
        H(P.o_srccell)[i] = e.cell;
        if (tail[e.cell] < 0) H(P.o_srcmap)[e.cell] = i;
        else H(P.o_srcnext)[tail[e.cell]] = i;
        tail[e.cell] = i;
    }
    // probes: descending `order` (stable), chains per cell in that order
    std::vector<int> idx(P.np);
    for (int i = 0; i < P.np; ++i) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
        return d->probes_host[a].order > d->probes_host[b].order;
    });
    std::fill(tail.begin(), tail.end(), -1);
    for (int j = 0; j < P.np; ++j) {
        int i = idx[j];
        const wt_probe_entry& e = d->probes_host[i];
        H(P.o_prbnext)[i] = -1;
        H(P.o_prbkind)[i] = e.kind;
        if (tail[e.cell] < 0) H(P.o_prbmap)[e.cell] = i;
        else H(P.o_prbnext)[tail[e.cell]] = i;
        tail[e.cell] = i;
        H(P.o_fcell)[j] = e.cell;
        H(P.o_fkind)[j] = e.kind;
        H(P.o_fcol)[j] = i;
    }
    H(P.o_err)[0] = 0;
    // tiles of the vector per-step kernels that hold a source or probe cell
    auto flag = [&](int cell) {
        const int cx = cell / P.ny, cy = cell % P.ny;
        H(P.o_tileflag)[(size_t)(cx / wt::STEP4_TX) * P.tiles_y + cy / wt::STEP4_TY] = 1;
    };
    for (int i = 0; i < P.ns; ++i) flag(d->sources_host[i].cell);
    for (int i = 0; i < P.np; ++i) flag(d->probes_host[i].cell);
    // Small tables go to the device inside a kernel's parameters, so the host
    // does not wait: the per-cell maps (plain form only) are filled with -1
    // and every other entry is written explicitly.
    static thread_local wt::IntScatter sc;
    sc.n = 0;
    auto put = [&](size_t off_bytes, size_t count, bool skip_fill, int fill = -1) {
        const int* src = H(off_bytes);
        for (size_t i = 0; i < count; ++i) {
            if (skip_fill && src[i] == fill) continue;
            if (sc.n == wt::INT_SCATTER_CAP) return false;
            sc.idx[sc.n] = (int)(off_bytes / sizeof(int) + i);
            sc.val[sc.n++] = src[i];
        }
        return true;
    };
    const bool plain = P.form == WT_FORM_PLAIN;
    const size_t ntiles = (size_t)P.tiles_x * P.tiles_y;
    bool fits = (!plain || (put(P.o_srcmap, P.plane, true) && put(P.o_prbmap, P.plane, true) &&
                            put(P.o_tileflag, ntiles, true, 0))) &&
                put(P.o_srcnext, P.ns, false) && put(P.o_srcrow, P.ns, false) &&
                put(P.o_srccell, P.ns, false) && put(P.o_prbnext, P.np, false) &&
                put(P.o_prbkind, P.np, false) && put(P.o_fcell, P.np, false) &&
                put(P.o_fkind, P.np, false) && put(P.o_fcol, P.np, false) && put(P.o_err, 1, false);
    int rc;
    if (fits) {
        int* base = at<int>(ws, 0);
        if (plain) {
            if ((rc = wt_launch_fill_int(base + P.o_srcmap / sizeof(int), P.plane, -1, st))) return rc;
            if ((rc = wt_launch_fill_int(base + P.o_prbmap / sizeof(int), P.plane, -1, st))) return rc;
            if ((rc = wt_launch_fill_int(base + P.o_tileflag / sizeof(int), ntiles, 0, st))) return rc;
        }
        return wt_launch_scatter_ints(base, sc, st);
    }
    // too many entries for one parameter block: one staged copy of all tables
    cudaError_t e = cudaMemcpyAsync(ws, h.data(), P.tables_end, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return wt_cuda_status(e);
    // pageable source: make sure the staging copy has consumed `h`
    return wt_cuda_status(cudaStreamSynchronize(st));
}

wt::FusedParams fused_params(const wt_scalars* s, const SeqPlan& P, const float* b, const float* c,
                             const float* x, void* ws) {
    wt::FusedParams F;
    std::memset(&F, 0, sizeof(F));
    F.k = wt_make_scalars(s);
    F.batch = P.B; F.nx = P.nx; F.ny = P.ny; F.steps = P.T;
    F.C = P.L.C; F.R = P.L.R; F.NCP = P.L.NCP; F.LD = P.L.LD; F.seg = P.seg; F.PB = P.L.PB;
    // (R and LD are set per kernel at launch: the two kernels use different strips)
    F.b = b; F.c = c; F.x = x;
    F.coef_stride = P.coef_batched ? P.plane : 0;
    F.n_src = P.ns;
    F.src_cell = at<int>(ws, P.o_srccell);
    F.src_row = at<int>(ws, P.o_srcrow);
    F.n_prb = P.np;
    F.prb_cell = at<int>(ws, P.o_fcell);
    F.prb_kind = at<int>(ws, P.o_fkind);
    F.prb_col = at<int>(ws, P.o_fcol);
    F.prb_kind_col = at<int>(ws, P.o_prbkind);
    F.amp = at<float>(ws, P.o_amp);
    F.ckpt = P.tape ? nullptr : at<float>(ws, P.o_ckpt);
    F.stash = P.tape ? nullptr : at<float>(ws, P.o_stash);
    F.stash_smem = P.L.stash_smem;
    F.lap = P.tape ? at<float>(ws, P.o_lap) : nullptr;
    F.nbuf = P.L.nbuf;
    F.gc_part = at<float>(ws, P.o_gcpart);
    F.err = at<int>(ws, P.o_err);
    F.halo = P.band ? at<unsigned long long>(ws, P.o_halo) : nullptr;
    F.bstate = P.band && !P.tape ? at<float>(ws, P.o_bstate) : nullptr;
    return F;
}

}  // namespace

extern "C" int wt_seq_workspace_bytes(const wt_seq_desc* d, size_t* bytes) {
    if (!bytes) return WT_ERR_INVALID;
    SeqPlan P;
    int st = make_plan(d, &P);
    if (st) return st;
    *bytes = P.total;
    return WT_OK;
}

extern "C" int wt_seq_fwd(const wt_scalars* s, const wt_seq_desc* d, const float* b,
                          const float* c, const float* x, float* out, float* fields,
                          float* probe_sum, void* workspace, size_t workspace_bytes,
                          wt_stream_t stream) {
    if (!scalars_ok(s)) return WT_ERR_INVALID;
    SeqPlan P;
    int st = make_plan(d, &P);
    if (st) return st;
    if (!b || !c || !workspace || workspace_bytes < P.total) return WT_ERR_INVALID;
    if (P.ns > 0 && !x) return WT_ERR_INVALID;
    if (P.np > 0 && !out) return WT_ERR_INVALID;
    if (d->output_fields && !fields) return WT_ERR_INVALID;
    cudaStream_t cs = (cudaStream_t)stream;
    if ((st = upload_tables(d, P, workspace, cs))) return st;
    const StepScalars k = wt_make_scalars(s);
    const size_t plane = P.plane;
    if (P.form == WT_FORM_PLAIN) {
        float* hist = at<float>(workspace, P.o_hist);
        float* zero = at<float>(workspace, P.o_zero);
        if ((st = wt_launch_fill_zero(zero, plane, cs))) return st;
        wt::SeqEpilogue e{};
        e.srcmap = at<int>(workspace, P.o_srcmap);
        e.src_next = at<int>(workspace, P.o_srcnext);
        e.src_row = at<int>(workspace, P.o_srcrow);
        e.x = x;
        e.steps = P.T;
        e.probemap = at<int>(workspace, P.o_prbmap);
        e.probe_next = at<int>(workspace, P.o_prbnext);
        e.probe_kind = at<int>(workspace, P.o_prbkind);
        e.out = out;
        e.amp = at<float>(workspace, P.o_amp);
        e.n_probe = P.np;
        e.tileflag = at<int>(workspace, P.o_tileflag);
        e.tiles_y = P.tiles_y;
        const size_t hbs = (size_t)P.T * plane;   // history is [B][T][nx][ny]
        // the update coefficients once per sequence (each A holds a division)
        float* fco = at<float>(workspace, P.o_fco);
        if ((st = wt_launch_fwd_coef(k, plane, b, c, fco, cs))) return st;
        for (int t = 0; t < P.T; ++t) {
            e.t = t;
            const float* y1 = t >= 1 ? hist + (size_t)(t - 1) * plane : zero;
            const float* y2 = t >= 2 ? hist + (size_t)(t - 2) * plane : zero;
            st = wt_launch_step_fwd(k, P.B, P.nx, P.ny, 0, b, c, y1, t >= 1 ? hbs : 0, y2,
                                    t >= 2 ? hbs : 0, hist + (size_t)t * plane, hbs, &e, cs, fco);
            if (st) return st;
        }
        if (d->output_fields) {
            cudaError_t ce = cudaMemcpyAsync(fields, hist, (size_t)P.B * hbs * sizeof(float),
                                             cudaMemcpyDeviceToDevice, cs);
            if (ce != cudaSuccess) return wt_cuda_status(ce);
        }
    } else {
        wt::FusedParams F = fused_params(s, P, b, c, x, workspace);
        F.out = out;
        F.fields = d->output_fields ? fields : nullptr;
        F.psum = P.np > 0 ? probe_sum : nullptr;   // summed in the probe flushes
        if (P.rctas) {
            if ((st = upload_rounds(P, workspace, cs))) return st;
            return wt_launch_band_rounds(true, F, P.BL, P.rctas, at<int>(workspace, P.o_rfirst),
                                         at<int>(workspace, P.o_ritems), cs);
        }
        return P.band ? wt_launch_band(true, F, P.BL, cs) : wt_launch_fused(true, F, P.L, cs);
    }
    if (probe_sum && P.np > 0)
        return wt_launch_probe_sum(P.B, P.T, P.np, out, probe_sum, cs);
    return WT_OK;
}

extern "C" int wt_seq_bwd(const wt_scalars* s, const wt_seq_desc* d, const float* b,
                          const float* c, const float* x, const float* grad_out, float* grad_c,
                          float* grad_x, void* workspace, size_t workspace_bytes,
                          wt_stream_t stream) {
    if (!scalars_ok(s)) return WT_ERR_INVALID;
    SeqPlan P;
    int st = make_plan(d, &P);
    if (st) return st;
    if (!b || !c || !grad_c || !workspace || workspace_bytes < P.total) return WT_ERR_INVALID;
    if (P.np > 0 && !grad_out) return WT_ERR_INVALID;
    if (grad_x) {
        // dL/dx is served for a single own-row source entry (a point source)
        int own = 0;
        for (int i = 0; i < P.ns; ++i) own += d->sources_host[i].in_row < 0;
        if (own != 1 || P.ns != 1) return WT_ERR_UNSUPPORTED;
    }
    cudaStream_t cs = (cudaStream_t)stream;
    const StepScalars k = wt_make_scalars(s);
    const size_t plane = P.plane;
    const size_t bp = (size_t)P.B * plane;
    if (P.form == WT_FORM_PLAIN) {
        float* hist = at<float>(workspace, P.o_hist);
        float* lam = at<float>(workspace, P.o_lam);
        float* gc = at<float>(workspace, P.o_gc);
        float* kco = at<float>(workspace, P.o_kco);
        if ((st = wt_launch_adj_coef(k, plane, b, c, kco, cs))) return st;
        wt::AdjEpilogue e{};
        e.probemap = at<int>(workspace, P.o_prbmap);
        e.probe_next = at<int>(workspace, P.o_prbnext);
        e.probe_kind = at<int>(workspace, P.o_prbkind);
        e.grad_out = grad_out;
        e.amp = at<float>(workspace, P.o_amp);
        e.n_probe = P.np;
        e.steps = P.T;
        e.srcmap = at<int>(workspace, P.o_srcmap);
        e.src_next = at<int>(workspace, P.o_srcnext);
        e.src_row = at<int>(workspace, P.o_srcrow);
        e.grad_x = grad_x;
        e.tileflag = at<int>(workspace, P.o_tileflag);
        e.tiles_y = P.tiles_y;
        const size_t hbs = (size_t)P.T * plane;
        for (int t = P.T - 1; t >= 0; --t) {
            e.t = t;
            const float* l1 = t + 1 < P.T ? lam + (size_t)((t + 1) % 3) * bp : nullptr;
            const float* l2 = t + 2 < P.T ? lam + (size_t)((t + 2) % 3) * bp : nullptr;
            const float* hp = t >= 1 ? hist + (size_t)(t - 1) * plane : nullptr;
            float* lo = lam + (size_t)(t % 3) * bp;
            if (P.B == 1) {       // one instance: the step accumulates dL/dc itself
                e.G = grad_c;
                e.first = t == P.T - 1;
            }
            // the step's dL/dc terms summed over the batch into grad_c (by the
            // step itself for one instance)
            st = wt_launch_seq_adj_step(k, P.B, P.nx, P.ny, b, c, kco, l1, l2, hp, hbs, lo, gc,
                                        grad_c, t == P.T - 1, e, cs);
            if (st) return st;
        }
        return WT_OK;
    }
    wt::FusedParams F = fused_params(s, P, b, c, x, workspace);
    F.grad_out = grad_out;
    F.grad_x = grad_x;
    if (P.coef_batched) F.gc_part = grad_c;   // per-instance dL/dc is the result
    if (P.rctas && (st = upload_rounds(P, workspace, cs))) return st;
    auto band_launch = [&](bool fwd, const wt::FusedParams& G) {
        return P.rctas ? wt_launch_band_rounds(fwd, G, P.BL, P.rctas, at<int>(workspace, P.o_rfirst),
                                               at<int>(workspace, P.o_ritems), cs)
                       : wt_launch_band(fwd, G, P.BL, cs);
    };
    if (P.band && !P.tape) {
        // from checkpoints, one segment at a time, last first: a launch of the
        // forward rebuilds the segment's Laplacians into the stash, a launch
        // of the adjoint runs the segment's steps from it (its state carried
        // from the previous segment's launch)
        for (int sg = P.nseg - 1; sg >= 0 && !st; --sg) {
            wt::FusedParams G = F;
            G.t_lo = sg * P.seg;
            G.t_hi = std::min(P.T, G.t_lo + P.seg);
            G.lap = G.stash;
            G.recompute = 1;
            st = band_launch(true, G);
            if (st) break;
            G.recompute = 0;
            st = band_launch(false, G);
        }
    } else if (P.band) {
        st = band_launch(false, F);
    } else {
        st = wt_launch_fused(false, F, P.L, cs);
    }
    if (st) return st;
    if (P.coef_batched) return WT_OK;
    return wt_launch_seq_adj_reduce(P.B, plane, F.gc_part, grad_c, 1, cs);
}

extern "C" int wt_seq_device_status(const wt_seq_desc* d, const void* workspace,
                                    size_t workspace_bytes, wt_stream_t stream) {
    SeqPlan P;
    int st = make_plan(d, &P);
    if (st) return st;
    if (!workspace || workspace_bytes < P.total) return WT_ERR_INVALID;
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, static_cast<const char*>(workspace) + P.o_err, sizeof(int),
                                    cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return wt_cuda_status(e);
    if (h == WT_DEVERR_BOUNDS) return WT_ERR_INVALID;
    if (h == WT_DEVERR_TIMEOUT) return WT_ERR_TIMEOUT;
    return WT_OK;
}

extern "C" int wt_test_band_missing_arrival(const wt_scalars* s, const wt_seq_desc* d,
                                            const float* b, const float* c, const float* x,
                                            float* out, void* workspace, size_t workspace_bytes,
                                            int32_t band, wt_stream_t stream) {
    if (!scalars_ok(s)) return WT_ERR_INVALID;
    SeqPlan P;
    int st = make_plan(d, &P);
    if (st) return st;
    if (!P.band) return WT_ERR_UNSUPPORTED;
    if (band < 0 || band >= P.BL.PR) return WT_ERR_INVALID;
    if (!b || !c || !workspace || workspace_bytes < P.total) return WT_ERR_INVALID;
    if ((P.ns > 0 && !x) || (P.np > 0 && !out)) return WT_ERR_INVALID;
    cudaStream_t cs = (cudaStream_t)stream;
    if ((st = upload_tables(d, P, workspace, cs))) return st;
    wt::FusedParams F = fused_params(s, P, b, c, x, workspace);
    F.out = out;
    F.mute_band1 = band + 1;
    return wt_launch_band(true, F, P.BL, cs);
}

extern "C" int wt_test_cluster_missing_arrival(const wt_scalars* s, const wt_seq_desc* d,
                                               const float* b, const float* c, const float* x,
                                               float* out, void* workspace,
                                               size_t workspace_bytes, int32_t cta,
                                               wt_stream_t stream) {
    if (!scalars_ok(s)) return WT_ERR_INVALID;
    SeqPlan P;
    int st = make_plan(d, &P);
    if (st) return st;
    if (P.form != WT_FORM_FUSED || P.band || P.L.C < 2) return WT_ERR_UNSUPPORTED;
    if (cta < 0 || cta >= P.L.C) return WT_ERR_INVALID;
    if (!b || !c || !workspace || workspace_bytes < P.total) return WT_ERR_INVALID;
    if ((P.ns > 0 && !x) || (P.np > 0 && !out)) return WT_ERR_INVALID;
    cudaStream_t cs = (cudaStream_t)stream;
    if ((st = upload_tables(d, P, workspace, cs))) return st;
    wt::FusedParams F = fused_params(s, P, b, c, x, workspace);
    F.out = out;
    F.mute_cta1 = cta + 1;
    return wt_launch_fused(true, F, P.L, cs);
}

extern "C" int wt_test_tape_missing_slice(const wt_scalars* s, const wt_seq_desc* d,
                                          const float* b, const float* c, const float* x,
                                          const float* grad_out, float* grad_c, void* workspace,
                                          size_t workspace_bytes, int32_t step,
                                          wt_stream_t stream) {
    if (!scalars_ok(s)) return WT_ERR_INVALID;
    SeqPlan P;
    int st = make_plan(d, &P);
    if (st) return st;
    if (P.form != WT_FORM_FUSED || P.band || !(P.tape || P.L.ws)) return WT_ERR_UNSUPPORTED;
    if (step < 0 || step >= P.T) return WT_ERR_INVALID;
    if (!b || !c || !grad_c || !workspace || workspace_bytes < P.total) return WT_ERR_INVALID;
    if (P.np > 0 && !grad_out) return WT_ERR_INVALID;
    wt::FusedParams F = fused_params(s, P, b, c, x, workspace);
    F.grad_out = grad_out;
    F.skip_slice1 = step + 1;
    cudaStream_t cs = (cudaStream_t)stream;
    if ((st = wt_launch_fused(false, F, P.L, cs))) return st;
    if (P.coef_batched) return WT_OK;
    return wt_launch_seq_adj_reduce(P.B, P.plane, F.gc_part, grad_c, 1, cs);
}

// ---------------------------------------------------------------------------
// 3. sequences of the nonlinear cell (fused form, tape mode)
static bool nl_ok(const wt_nonlinear* nl) {
    return nl && std::isfinite(nl->satdamp_b0) && std::isfinite(nl->satdamp_uth) &&
           std::isfinite(nl->c_nl) && (nl->satdamp_b0 <= 0.f || nl->satdamp_uth != 0.f);
}

extern "C" int wt_seq_workspace_bytes_nl(const wt_seq_desc* d, size_t* bytes) {
    if (!bytes) return WT_ERR_INVALID;
    SeqPlan P;
    int st = make_plan(d, &P, true);
    if (st) return st;
    if (P.form != WT_FORM_FUSED) return WT_ERR_UNSUPPORTED;
    *bytes = P.total;
    return WT_OK;
}

static void nl_params(wt::FusedParams& F, const SeqPlan& P, const wt_nonlinear* nl, const float* rho,
                      void* ws) {
    F.rho = rho;
    F.b0 = nl->satdamp_b0;
    F.uth = nl->satdamp_uth;
    F.cnl = nl->c_nl;
    F.grho_part = at<float>(ws, P.o_grho);
}

extern "C" int wt_seq_fwd_nl(const wt_scalars* s, const wt_seq_desc* d, const wt_nonlinear* nl,
                             const float* b, const float* c_lin, const float* rho, const float* x,
                             float* out, float* probe_sum, void* workspace, size_t workspace_bytes,
                             wt_stream_t stream) {
    if (!scalars_ok(s) || !nl_ok(nl)) return WT_ERR_INVALID;
    SeqPlan P;
    int st = make_plan(d, &P, true);
    if (st) return st;
    if (P.form != WT_FORM_FUSED) return WT_ERR_UNSUPPORTED;
    if (!b || !c_lin || !rho || !workspace || workspace_bytes < P.total) return WT_ERR_INVALID;
    if (P.ns > 0 && !x) return WT_ERR_INVALID;
    if (P.np > 0 && !out) return WT_ERR_INVALID;
    cudaStream_t cs = (cudaStream_t)stream;
    if ((st = upload_tables(d, P, workspace, cs))) return st;
    wt::FusedParams F = fused_params(s, P, b, c_lin, x, workspace);
    nl_params(F, P, nl, rho, workspace);
    F.out = out;
    F.psum = P.np > 0 ? probe_sum : nullptr;
    return wt_launch_fused_nl(true, F, P.L, cs);
}

extern "C" int wt_seq_bwd_nl(const wt_scalars* s, const wt_seq_desc* d, const wt_nonlinear* nl,
                             const float* b, const float* c_lin, const float* rho, const float* x,
                             const float* grad_out, float* grad_c, float* grad_rho, float* grad_x,
                             void* workspace, size_t workspace_bytes, wt_stream_t stream) {
    if (!scalars_ok(s) || !nl_ok(nl)) return WT_ERR_INVALID;
    SeqPlan P;
    int st = make_plan(d, &P, true);
    if (st) return st;
    if (P.form != WT_FORM_FUSED) return WT_ERR_UNSUPPORTED;
    if (!b || !c_lin || !rho || !grad_c || !grad_rho || !workspace || workspace_bytes < P.total)
        return WT_ERR_INVALID;
    if (P.np > 0 && !grad_out) return WT_ERR_INVALID;
    if (grad_x) {
        int own = 0;
        for (int i = 0; i < P.ns; ++i) own += d->sources_host[i].in_row < 0;
        if (own != 1 || P.ns != 1) return WT_ERR_UNSUPPORTED;
    }
    cudaStream_t cs = (cudaStream_t)stream;
    wt::FusedParams F = fused_params(s, P, b, c_lin, x, workspace);
    nl_params(F, P, nl, rho, workspace);
    F.grad_out = grad_out;
    F.grad_x = grad_x;
    if (P.coef_batched) { F.gc_part = grad_c; F.grho_part = grad_rho; }
    if ((st = wt_launch_fused_nl(false, F, P.L, cs))) return st;
    if (P.coef_batched) return WT_OK;
    if ((st = wt_launch_seq_adj_reduce(P.B, P.plane, F.gc_part, grad_c, 1, cs))) return st;
    return wt_launch_seq_adj_reduce(P.B, P.plane, F.grho_part, grad_rho, 1, cs);
}

// ---------------------------------------------------------------------------
// 4. the training loss fused with the sequence
extern "C" int wt_loss_ce_normalize_power(int32_t batch, int32_t n_probes, const float* probe_sum,
                                          const int64_t* labels, float* loss, float* grad_sum,
                                          wt_stream_t stream) {
    if (batch <= 0 || n_probes <= 0 || !probe_sum || !labels || !loss || !grad_sum)
        return WT_ERR_INVALID;
    return wt_launch_loss_ce_np(batch, n_probes, probe_sum, labels, loss, grad_sum,
                                (cudaStream_t)stream);
}

extern "C" int wt_seq_bwd_sum(const wt_scalars* s, const wt_seq_desc* d, const float* b,
                              const float* c, const float* x, const float* grad_sum,
                              float* grad_c, void* workspace, size_t workspace_bytes,
                              wt_stream_t stream) {
    if (!scalars_ok(s)) return WT_ERR_INVALID;
    SeqPlan P;
    int st = make_plan(d, &P);
    if (st) return st;
    if (P.form != WT_FORM_FUSED) return WT_ERR_UNSUPPORTED;
    if (!b || !c || !grad_c || !grad_sum || !workspace || workspace_bytes < P.total)
        return WT_ERR_INVALID;
    cudaStream_t cs = (cudaStream_t)stream;
    wt::FusedParams F = fused_params(s, P, b, c, x, workspace);
    F.grad_w = grad_sum;
    if (P.coef_batched) F.gc_part = grad_c;
    if ((st = wt_launch_fused(false, F, P.L, cs))) return st;
    if (P.coef_batched) return WT_OK;
    return wt_launch_seq_adj_reduce(P.B, P.plane, F.gc_part, grad_c, 1, cs);
}
