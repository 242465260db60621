// Layout choice for ragged batches (host code): one option per group of a
// batch of models, from measured times, by SM-time with a bound on the
// longest group.  See wt_ragged_plan in include/wavetorch_gb300.h.
#include <vector>

#include "internal.cuh"

namespace {

struct Key {          // lexicographic comparison key
    double a, b;
    bool operator<(const Key& o) const { return a < o.a || (a == o.a && b < o.b); }
};

}  // namespace

extern "C" int wt_ragged_plan(const wt_ragged_group* groups, int32_t n_groups, int32_t n_sm,
                              int32_t* choice) {
    if (n_groups < 0 || (n_groups > 0 && (!groups || !choice)) || n_sm <= 0) return WT_ERR_INVALID;
    for (int g = 0; g < n_groups; ++g) {
        const wt_ragged_group& G = groups[g];
        if (G.instances <= 0 || G.n_options <= 0 || !G.options || !(G.scale > 0.0))
            return WT_ERR_INVALID;
        for (int k = 0; k < G.n_options; ++k)
            if (G.options[k].ctas <= 0 || !(G.options[k].seconds >= 0.0)) return WT_ERR_INVALID;
    }
    auto t = [&](int g, int k) { return groups[g].options[k].seconds * groups[g].scale; };
    auto sms = [&](int g, int k) { return (double)groups[g].options[k].ctas; };
    // least SM-time per group (ties: fewer CTAs, then the earlier option)
    std::vector<int> pick(n_groups, 0);
    for (int g = 0; g < n_groups; ++g) {
        Key best{sms(g, 0) * t(g, 0), sms(g, 0)};
        for (int k = 1; k < groups[g].n_options; ++k) {
            const Key key{sms(g, k) * t(g, k), sms(g, k)};
            if (key < best) { best = key; pick[g] = k; }
        }
    }
    // move the longest group to a faster option while it outlasts the
    // SM-time bound of the whole batch
    for (int it = 0; it < 4 * n_groups + 1 && n_groups > 0; ++it) {
        double bound = 0.0;
        for (int g = 0; g < n_groups; ++g)
            bound += groups[g].instances * sms(g, pick[g]) * t(g, pick[g]);
        bound /= n_sm;
        int kg = 0;
        for (int g = 1; g < n_groups; ++g)
            if (t(g, pick[g]) > t(kg, pick[kg])) kg = g;
        const double tk = t(kg, pick[kg]);
        if (tk <= bound) break;
        int best = -1;
        Key bkey{0.0, 0.0};
        for (int k = 0; k < groups[kg].n_options; ++k) {
            if (!(t(kg, k) < tk)) continue;
            const Key key{sms(kg, k) * t(kg, k), -t(kg, k)};
            if (best < 0 || key < bkey) { best = k; bkey = key; }
        }
        if (best < 0) break;
        pick[kg] = best;
    }
    for (int g = 0; g < n_groups; ++g) choice[g] = pick[g];
    return WT_OK;
}
