// gdp_tune.cu -- the autotuner: picks the row bins (thread_row_max,
// split_tile) and the round-loop schedule (driver, resident CTAs per SM) of a
// problem by timing its propagation under each candidate.
#include <algorithm>
#include <cfloat>
#include <memory>
#include <string>
#include <vector>

#include "gdp_context.h"

namespace gdp {

GDP_RETCODE autotune(int m, int n, int nnz, const int *col, const int *row_ptr, const double *val,
                     const double *lhs, const double *rhs, const double *lbs, const double *ubs,
                     const int *vartype, const gdp_options *base, int repeats, gdp_options *best,
                     double *best_ms, gdp_tune_trial *trials, int max_trials, int *n_trials) {
    if (m <= 0 || n <= 0 || nnz <= 0 || !lbs || !ubs || !best) {
        set_error("autotune needs a non-empty problem, bounds and an output");
        return GDP_ERROR;
    }
    gdp_options b;
    gdp_default_options(&b);
    if (base) b = *base;
    repeats = std::max(1, repeats);
    const int trms[] = {16, 32, 64};
    const int tiles[] = {512, 1024, 2048};
    struct Sched {
        int sync, ctas;
    };
    const Sched scheds[] = {{MEGAKERNEL, 2}, {MEGAKERNEL, 3}, {MEGAKERNEL, 0}, {GPU_LOOP, 0}};
    std::vector<double> lb(n), ub(n);
    double best_t = DBL_MAX;
    int cnt = 0;
    for (int trm : trms) {
        for (int tile : tiles) {
            for (const Sched &sc : scheds) {
                gdp_options o = b;
                o.thread_row_max = trm;
                o.split_tile = tile;
                o.sync_type = sc.sync;
                o.ctas_per_sm = sc.ctas;
                std::unique_ptr<Context> ctx(new Context());
                if (ctx->init(m, n, nnz, col, row_ptr, val, lhs, rhs, vartype, &o) != GDP_OKAY) return GDP_ERROR;
                double t = DBL_MAX;
                int rounds = 0;
                for (int r = 0; r < repeats + 1; r++) {  // the first run warms up
                    std::copy(lbs, lbs + n, lb.begin());
                    std::copy(ubs, ubs + n, ub.begin());
                    gdp_stats st{};
                    if (ctx->propagate_host(lb.data(), ub.data(), &st) != GDP_OKAY) return GDP_ERROR;
                    rounds = st.rounds;
                    if (r > 0) t = std::min(t, st.device_ms);
                }
                if (trials && cnt < max_trials) trials[cnt] = gdp_tune_trial{trm, tile, sc.sync, sc.ctas, rounds, 0, t};
                cnt++;
                if (t < best_t) {
                    best_t = t;
                    *best = o;
                }
            }
        }
    }
    if (best_ms) *best_ms = best_t;
    if (n_trials) *n_trials = std::min(cnt, max_trials);
    return GDP_OKAY;
}

}  // namespace gdp
