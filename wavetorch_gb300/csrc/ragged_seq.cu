// A ragged batch of models in one forward and one adjoint launch
// (include/wavetorch_gb300.h, section 5): the host-side plan.  Each model is
// cut into bands of R = S * M rows (the band layout of seq_band.cu, on blocks
// of 1024 threads); a band of a model is one work item, run for all of the
// model's steps.  The schedule gives each CTA (one per SM) a list of items:
// models are placed largest first on the least-loaded CTAs, all bands of a
// model starting together, and every CTA takes its items in order of start
// time, one global order (see band_list_kernel).
//
// The reference trains one model at a time (wavetorch/rnn.py:21-72 per
// model); each model here keeps that model's own arithmetic: its Laplacian
// order is that of a batch of one, its sources are its own input.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "internal.cuh"

namespace {

constexpr size_t ALIGN = 256;
constexpr int NT = 1024;               // threads per CTA of the packed launch
constexpr int ONEDNN_MIN_CELLS = 20480;
size_t up(size_t v) { return (v + ALIGN - 1) / ALIGN * ALIGN; }

struct ModelPlan {
    int PR, S, R, NCP, LD, PB, order;
    size_t smem_fwd, smem_bwd;
    size_t o_src_cell, o_src_row, o_prb_cell, o_prb_kind, o_prb_col, o_prb_kcol;
    size_t o_amp, o_lap, o_halo;
    double cost;                       // estimated band-steps of one item
};

struct Plan {
    int M, ctas;
    std::vector<ModelPlan> mp;
    std::vector<int> first;            // [ctas + 1]
    std::vector<int> items;            // (model, band) pairs
    size_t o_params, o_first, o_items, o_err, o_halo, halo_bytes, total;
    size_t smem_fwd, smem_bwd;
    double steps_per_cta;
};

int device_sms(int want) {
    if (want > 0) return want;
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

bool scalars_valid(const wt_scalars* s) {
    return s && std::isfinite(s->dt) && s->dt > 0.f && std::isfinite(s->h) && s->h > 0.f;
}

// Band geometry of one model for strip height M: S strips of NCP threads
// (at most NT threads, no more strips than the rows need), PR bands; the
// shared memory its forward and adjoint take (the band kernels' layout with
// coefficient words for all NT threads).
bool model_geometry(const wt_ragged_model& m, int M, ModelPlan& p) {
    p.NCP = ((m.ny + 31) / 32) * 32;
    if (p.NCP > NT) return false;
    const int rows_for = (m.nx + M - 1) / M;
    p.S = std::max(1, std::min(NT / p.NCP, rows_for));
    p.R = p.S * M;
    p.PR = (m.nx + p.R - 1) / p.R;
    p.LD = (p.R + 2) | 1;
    const int np = m.n_probes;
    p.PB = np > 0 ? std::max(1, std::min(32, 2048 / np)) : 32;
    auto r16 = [](size_t v) { return (v + 15) / 16 * 16; };
    const size_t tiles = 2 * (size_t)(m.ny + 2) * p.LD * sizeof(float);
    p.smem_fwd = tiles + (size_t)((3 * M) | 1) * NT * sizeof(float) +
                 r16((size_t)(2 * np * p.PB + 3 * np) * 4);
    p.smem_bwd = tiles + (size_t)(((4 * M) | 1) + M) * NT * sizeof(float) +
                 r16((size_t)(2 * np * p.PB) * 4);
    return true;
}

int make_plan(const wt_scalars* s, const wt_ragged_model* models, int n, int sm_count, int strip,
              Plan& P) {
    if (!scalars_valid(s) || !models || n <= 0) return WT_ERR_INVALID;
    if (strip != 0 && strip != 4 && strip != 8) return WT_ERR_INVALID;
    P.ctas = device_sms(sm_count);
    if (P.ctas <= 0) return WT_ERR_UNSUPPORTED;
    const size_t SMEM_MAX = 227 * 1024 - 64 - 512;     // the staged parameter block
    for (int i = 0; i < n; ++i) {
        const wt_ragged_model& m = models[i];
        if (m.nx <= 0 || m.ny <= 0 || m.steps <= 0 || m.n_sources < 0 || m.n_probes < 0 ||
            (m.n_sources > 0 && !m.sources_host) || (m.n_probes > 0 && !m.probes_host))
            return WT_ERR_INVALID;
        if ((long long)m.nx * m.ny > (1LL << 30) || m.n_probes >= 1024) return WT_ERR_UNSUPPORTED;
        for (int e = 0; e < m.n_sources; ++e) {
            const wt_source_entry& q = m.sources_host[e];
            if (q.cell < 0 || q.cell >= m.nx * m.ny) return WT_ERR_INVALID;
            if (q.in_row != -1) return WT_ERR_UNSUPPORTED;   // each model drives its own input
        }
        for (int e = 0; e < m.n_probes; ++e) {
            const wt_probe_entry& q = m.probes_host[e];
            if (q.cell < 0 || q.cell >= m.nx * m.ny || (q.kind != 0 && q.kind != 1))
                return WT_ERR_INVALID;
        }
    }
    // the requested strip height, else the tallest every model's shared
    // memory allows (fewer bands)
    P.M = 0;
    for (int M : {8, 4}) {
        if (strip && M != strip) continue;
        bool fits = true;
        for (int i = 0; i < n && fits; ++i) {
            ModelPlan p;
            fits = model_geometry(models[i], M, p) && p.smem_fwd <= SMEM_MAX &&
                   p.smem_bwd <= SMEM_MAX && p.PR <= P.ctas;
        }
        if (fits) { P.M = M; break; }
    }
    if (!P.M) return WT_ERR_UNSUPPORTED;
    P.mp.assign(n, ModelPlan{});
    P.smem_fwd = P.smem_bwd = 0;
    const bool unit_h = 1.0f / (s->h * s->h) == 1.0f;
    for (int i = 0; i < n; ++i) {
        const wt_ragged_model& m = models[i];
        ModelPlan& p = P.mp[i];
        model_geometry(m, P.M, p);
        p.order = (unit_h && m.nx * m.ny <= ONEDNN_MIN_CELLS) ? WT_LAP_PAIRED : WT_LAP_SEQ;
        P.smem_fwd = std::max(P.smem_fwd, p.smem_fwd);
        P.smem_bwd = std::max(P.smem_bwd, p.smem_bwd);
        // two taps of each kind per thread at most (the band kernels' words)
        std::vector<int> cnt((size_t)p.PR * p.S * p.NCP, 0);
        auto key = [&](int cell) {
            const int gx = cell / m.ny, gy = cell % m.ny;
            return ((size_t)(gx / p.R) * p.S + (gx % p.R) / P.M) * p.NCP + gy;
        };
        for (int e = 0; e < m.n_sources; ++e)
            if (++cnt[key(m.sources_host[e].cell)] > 2) return WT_ERR_UNSUPPORTED;
        std::fill(cnt.begin(), cnt.end(), 0);
        for (int e = 0; e < m.n_probes; ++e)
            if (++cnt[key(m.probes_host[e].cell)] > 2) return WT_ERR_UNSUPPORTED;
        // one item's cost in cell-steps of its band, plus a fixed per-step part
        // (barriers, and the exchange between bands when there are several)
        p.cost = (double)m.steps * ((double)p.R * p.NCP + (p.PR > 1 ? 4096.0 : 1024.0));
    }
    // schedule: models by total cost, largest first, each on the PR least
    // loaded CTAs, its bands starting together when the last of them is free
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return P.mp[a].cost * P.mp[a].PR > P.mp[b].cost * P.mp[b].PR;
    });
    std::vector<double> load(P.ctas, 0.0);
    std::vector<std::vector<std::pair<double, std::pair<int, int>>>> lists(P.ctas);
    std::vector<int> ctas(P.ctas);
    for (int i : order) {
        const ModelPlan& p = P.mp[i];
        std::iota(ctas.begin(), ctas.end(), 0);
        std::partial_sort(ctas.begin(), ctas.begin() + p.PR, ctas.end(), [&](int a, int b) {
            return load[a] < load[b] || (load[a] == load[b] && a < b);
        });
        double start = 0.0;
        for (int k = 0; k < p.PR; ++k) start = std::max(start, load[ctas[k]]);
        for (int k = 0; k < p.PR; ++k) {
            load[ctas[k]] = start + p.cost;
            lists[ctas[k]].push_back({start, {i, k}});
        }
    }
    P.first.assign(P.ctas + 1, 0);
    P.items.clear();
    for (int c = 0; c < P.ctas; ++c) {
        auto& L = lists[c];
        // one global order: start time, then model (a model's bands share both)
        std::sort(L.begin(), L.end(), [](const auto& a, const auto& b) {
            return a.first < b.first || (a.first == b.first && a.second.first < b.second.first);
        });
        for (auto& it : L) { P.items.push_back(it.second.first); P.items.push_back(it.second.second); }
        P.first[c + 1] = (int)(P.items.size() / 2);
    }
    P.steps_per_cta = *std::max_element(load.begin(), load.end());
    // workspace: parameter blocks, the lists, the status word, the exchange
    // words of every model (then the abort word), then per model its tables,
    // raw probe amplitudes and Laplacian tape
    size_t o = 0;
    P.o_params = o; o = up(o + (size_t)n * sizeof(wt::FusedParams));
    P.o_first = o; o = up(o + (P.first.size()) * sizeof(int));
    P.o_items = o; o = up(o + P.items.size() * sizeof(int));
    P.o_err = o; o = up(o + sizeof(int));
    P.o_halo = o;
    for (int i = 0; i < n; ++i) {
        P.mp[i].o_halo = o;
        o += (size_t)P.mp[i].PR * 4 * P.mp[i].NCP * sizeof(unsigned long long);
    }
    o = up(o);
    o += 256;                                            // the abort word's line
    P.halo_bytes = o - P.o_halo;
    o = up(o);
    for (int i = 0; i < n; ++i) {
        const wt_ragged_model& m = models[i];
        ModelPlan& p = P.mp[i];
        const size_t ns = m.n_sources + 1, np = m.n_probes + 1;
        p.o_src_cell = o; o = up(o + ns * sizeof(int));
        p.o_src_row = o; o = up(o + ns * sizeof(int));
        p.o_prb_cell = o; o = up(o + np * sizeof(int));
        p.o_prb_kind = o; o = up(o + np * sizeof(int));
        p.o_prb_col = o; o = up(o + np * sizeof(int));
        p.o_prb_kcol = o; o = up(o + np * sizeof(int));
        p.o_amp = o; o = up(o + (size_t)m.steps * np * sizeof(float));
        p.o_lap = o; o = up(o + (size_t)m.steps * p.PR * NT * P.M * sizeof(float));
    }
    P.total = o;
    return WT_OK;
}

template <class T>
T* at(void* ws, size_t off) { return reinterpret_cast<T*>(static_cast<char*>(ws) + off); }

}  // namespace

extern "C" int wt_ragged_workspace_bytes(const wt_scalars* s, const wt_ragged_model* models,
                                         int32_t n_models, int32_t sm_count, int32_t strip,
                                         size_t* bytes) {
    if (!bytes) return WT_ERR_INVALID;
    Plan P;
    int st = make_plan(s, models, n_models, sm_count, strip, P);
    if (st) return st;
    *bytes = P.total;
    return WT_OK;
}

extern "C" int wt_ragged_prepare(const wt_scalars* s, const wt_ragged_model* models,
                                 int32_t n_models, int32_t sm_count, int32_t strip,
                                 void* workspace, size_t workspace_bytes, wt_ragged_plan_t* plan) {
    if (!plan || !workspace) return WT_ERR_INVALID;
    Plan P;
    int st = make_plan(s, models, n_models, sm_count, strip, P);
    if (st) return st;
    if (workspace_bytes < P.total) return WT_ERR_INVALID;
    for (int i = 0; i < n_models; ++i) {
        const wt_ragged_model& m = models[i];
        if (!m.b || !m.c || (m.n_sources > 0 && !m.x) || (m.n_probes > 0 && !m.out) ||
            !m.grad_c || (m.n_probes > 0 && !m.grad_out))
            return WT_ERR_INVALID;
    }
    // host images: the parameter blocks, lists and status word (the head of
    // the workspace, before the exchange words), and each model's tables
    std::vector<char> head(P.o_halo, 0);
    std::vector<std::vector<char>> tables(n_models);
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < n_models; ++i) {
        const wt_ragged_model& m = models[i];
        const ModelPlan& p = P.mp[i];
        std::vector<char>& img = tables[i];
        img.assign(p.o_amp - p.o_src_cell, 0);
        auto T = [&](size_t off) { return reinterpret_cast<int*>(img.data() + (off - p.o_src_cell)); };
        // probes in descending reference order (stable), as the kernels seed them
        std::vector<int> idx(m.n_probes);
        std::iota(idx.begin(), idx.end(), 0);
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
            return m.probes_host[a].order > m.probes_host[b].order;
        });
        int* sc = T(p.o_src_cell);
        int* sr = T(p.o_src_row);
        for (int k = 0; k < m.n_sources; ++k) { sc[k] = m.sources_host[k].cell; sr[k] = -1; }
        int* pc = T(p.o_prb_cell);
        int* pk = T(p.o_prb_kind);
        int* pcol = T(p.o_prb_col);
        int* pkc = T(p.o_prb_kcol);
        for (int j = 0; j < m.n_probes; ++j) {
            const wt_probe_entry& q = m.probes_host[idx[j]];
            pc[j] = q.cell; pk[j] = q.kind; pcol[j] = idx[j];
            pkc[idx[j]] = q.kind;
        }
        wt::FusedParams F;
        std::memset(&F, 0, sizeof(F));
        wt_scalars sm = *s;
        sm.lap_order = p.order;
        F.k = wt_make_scalars(&sm);
        F.batch = 1; F.nx = m.nx; F.ny = m.ny; F.steps = m.steps;
        F.C = p.PR; F.R = p.R; F.NCP = p.NCP; F.LD = p.LD; F.seg = m.steps; F.PB = p.PB;
        F.b = m.b; F.c = m.c; F.coef_stride = 0; F.x = m.x;
        F.n_src = m.n_sources;
        F.src_cell = at<int>(workspace, p.o_src_cell);
        F.src_row = at<int>(workspace, p.o_src_row);
        F.n_prb = m.n_probes;
        F.prb_cell = at<int>(workspace, p.o_prb_cell);
        F.prb_kind = at<int>(workspace, p.o_prb_kind);
        F.prb_col = at<int>(workspace, p.o_prb_col);
        F.prb_kind_col = at<int>(workspace, p.o_prb_kcol);
        F.out = m.out;
        F.amp = at<float>(workspace, p.o_amp);
        F.lap = at<float>(workspace, p.o_lap);
        F.grad_out = m.grad_out;
        F.gc_part = m.grad_c;          // one instance: its dL/dc is the result
        F.err = at<int>(workspace, P.o_err);
        F.halo = at<unsigned long long>(workspace, p.o_halo);
        F.abort_g = at<int>(workspace, P.o_halo + P.halo_bytes - 256);
        std::memcpy(head.data() + P.o_params + (size_t)i * sizeof(F), &F, sizeof(F));
    }
    std::memcpy(head.data() + P.o_first, P.first.data(), P.first.size() * sizeof(int));
    std::memcpy(head.data() + P.o_items, P.items.data(), P.items.size() * sizeof(int));
    e = cudaMemcpy(workspace, head.data(), head.size(), cudaMemcpyHostToDevice);
    for (int i = 0; i < n_models && e == cudaSuccess; ++i)
        e = cudaMemcpy(at<char>(workspace, P.mp[i].o_src_cell), tables[i].data(), tables[i].size(),
                       cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return wt_cuda_status(e);
    std::memset(plan, 0, sizeof(*plan));
    plan->n_models = n_models;
    plan->ctas = P.ctas;
    plan->strip = P.M;
    plan->n_items = (int)(P.items.size() / 2);
    plan->smem_fwd = P.smem_fwd;
    plan->smem_bwd = P.smem_bwd;
    plan->workspace_bytes = P.total;
    plan->off_params = P.o_params;
    plan->off_first = P.o_first;
    plan->off_items = P.o_items;
    plan->off_halo = P.o_halo;
    plan->halo_bytes = P.halo_bytes;
    plan->off_err = P.o_err;
    plan->est_steps_per_cta = P.steps_per_cta;
    return WT_OK;
}

static int ragged_launch(bool fwd, const wt_ragged_plan_t* plan, void* ws, wt_stream_t stream) {
    if (!plan || !ws || plan->ctas <= 0) return WT_ERR_INVALID;
    cudaStream_t st = (cudaStream_t)stream;
    // fresh exchange words (tag 0) and abort word; the forward also clears
    // the status word
    cudaError_t e = cudaMemsetAsync(at<char>(ws, plan->off_halo), 0, plan->halo_bytes, st);
    if (e == cudaSuccess && fwd) e = cudaMemsetAsync(at<char>(ws, plan->off_err), 0, sizeof(int), st);
    if (e != cudaSuccess) return wt_cuda_status(e);
    WtBandList L;
    L.params = at<const wt::FusedParams>(ws, plan->off_params);
    L.first = at<const int>(ws, plan->off_first);
    L.items = at<const int2>(ws, plan->off_items);
    L.abort_g = at<int>(ws, plan->off_halo + plan->halo_bytes - 256);
    return wt_launch_band_list(fwd, L, plan->ctas, plan->strip,
                               fwd ? plan->smem_fwd : plan->smem_bwd, st);
}

extern "C" int wt_ragged_fwd(const wt_ragged_plan_t* plan, void* workspace, wt_stream_t stream) {
    return ragged_launch(true, plan, workspace, stream);
}

extern "C" int wt_ragged_bwd(const wt_ragged_plan_t* plan, void* workspace, wt_stream_t stream) {
    return ragged_launch(false, plan, workspace, stream);
}

extern "C" int wt_ragged_status(const wt_ragged_plan_t* plan, const void* workspace,
                                wt_stream_t stream) {
    if (!plan || !workspace) return WT_ERR_INVALID;
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, static_cast<const char*>(workspace) + plan->off_err,
                                    sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return wt_cuda_status(e);
    if (h == WT_DEVERR_BOUNDS) return WT_ERR_INVALID;
    if (h == WT_DEVERR_TIMEOUT) return WT_ERR_TIMEOUT;
    return WT_OK;
}
