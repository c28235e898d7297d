// gdp_tune.cu -- the autotuner: picks the row bins (thread_row_max,
// split_tile) and the round-loop schedule (driver, resident CTAs per SM,
// megakernel CTA size) of a problem by timing its propagation under each
// candidate, and keeps the result per problem shape.
//
// Two stages: the row bins under the base schedule (each needs its own device
// layout), then the schedules on the fastest bins (one layout, regridded per
// candidate). The winner depends on the shape of the problem (how many rows of
// which length, how many non-zeros), not on its coefficients or bounds, so
// later calls for a problem of the same shape -- the nodes or restarts of one
// MIP, or a family of instances from one generator -- reuse it.
#include <algorithm>
#include <cfloat>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "gdp_context.h"

namespace gdp {

namespace {

// The shape a tuning result is kept under.
struct ShapeKey {
    int device, m, n, nnz, max_rounds, use_marking, repeats;
    int hist[32];  // rows by floor(log2(length)) (0: empty rows and length 1)
    bool operator<(const ShapeKey &o) const { return std::memcmp(this, &o, sizeof(ShapeKey)) < 0; }
};

struct Tuned {
    gdp_options best;
    double best_ms;
    std::vector<gdp_tune_trial> trials;
};

struct TuneCache {
    std::mutex mu;
    std::map<ShapeKey, Tuned> entries;
};
TuneCache &tune_cache() {
    static TuneCache *c = new TuneCache;  // never destroyed: used until exit
    return *c;
}

ShapeKey shape_of(int m, int n, int nnz, const int *row_ptr, const gdp_options &b, int repeats) {
    ShapeKey k;
    std::memset(&k, 0, sizeof(k));  // padding included: the key compares as bytes
    k.device = b.device;
    k.m = m;
    k.n = n;
    k.nnz = nnz;
    k.max_rounds = b.max_rounds;
    k.use_marking = b.use_marking;
    k.repeats = repeats;
    for (int i = 0; i < m; i++) {
        const unsigned len = (unsigned)(row_ptr[i + 1] - row_ptr[i]);
        const int bucket = len > 1 ? 31 - __builtin_clz(len) : 0;
        k.hist[bucket]++;
    }
    return k;
}

}  // namespace

GDP_RETCODE autotune_clear_cache() {
    TuneCache &c = tune_cache();
    std::lock_guard<std::mutex> g(c.mu);
    c.entries.clear();
    return GDP_OKAY;
}

GDP_RETCODE autotune(int m, int n, int nnz, const int *col, const int *row_ptr, const double *val,
                     const double *lhs, const double *rhs, const double *lbs, const double *ubs,
                     const int *vartype, const gdp_options *base, int repeats, gdp_options *best,
                     double *best_ms, gdp_tune_trial *trials, int max_trials, int *n_trials) {
    if (m <= 0 || n <= 0 || nnz <= 0 || !lbs || !ubs || !best || !row_ptr) {
        set_error("autotune needs a non-empty problem, bounds and an output");
        return GDP_ERROR;
    }
    gdp_options b;
    gdp_default_options(&b);
    if (base) b = *base;
    if (b.sync_type == CPU_LOOP) b.sync_type = MEGAKERNEL;  // the loop drivers worth tuning
    repeats = std::max(1, repeats);
    if (row_ptr[0] != 0 || row_ptr[m] != nnz) {
        set_error("csr_row_ptrs must start at 0 and end at nnz");
        return GDP_ERROR;
    }
    const ShapeKey key = shape_of(m, n, nnz, row_ptr, b, repeats);
    auto report = [&](const Tuned &t) {
        *best = t.best;
        if (best_ms) *best_ms = t.best_ms;
        const int k = std::min((int)t.trials.size(), std::max(0, max_trials));
        if (trials) std::copy(t.trials.begin(), t.trials.begin() + k, trials);
        if (n_trials) *n_trials = trials ? k : 0;
        return GDP_OKAY;
    };
    {
        TuneCache &c = tune_cache();
        std::lock_guard<std::mutex> g(c.mu);
        auto it = c.entries.find(key);
        if (it != c.entries.end()) return report(it->second);
    }

    Tuned out;
    out.best_ms = DBL_MAX;
    std::vector<double> lb(n), ub(n);
    // times the propagation of ctx under its current options
    auto time_it = [&](Context &ctx, double &t, int &rounds) -> GDP_RETCODE {
        t = DBL_MAX;
        for (int r = 0; r < repeats + 1; r++) {  // the first run warms up
            std::copy(lbs, lbs + n, lb.begin());
            std::copy(ubs, ubs + n, ub.begin());
            gdp_stats st{};
            if (ctx.propagate_host(lb.data(), ub.data(), &st) != GDP_OKAY) return GDP_ERROR;
            rounds = st.rounds;
            if (r > 0) t = std::min(t, st.device_ms);
        }
        return GDP_OKAY;
    };
    auto record = [&](const gdp_options &o, int rounds, double t) {
        out.trials.push_back(gdp_tune_trial{o.thread_row_max, o.split_tile, o.sync_type, o.ctas_per_sm, rounds,
                                            o.cta_threads ? o.cta_threads : 256, t});
        if (t < out.best_ms) {
            out.best_ms = t;
            out.best = o;
        }
    };

    // stage 1: row bins under the base schedule
    const int trms[] = {16, 32, 64};
    const int tiles[] = {512, 1024, 2048};
    for (int trm : trms)
        for (int tile : tiles) {
            gdp_options o = b;
            o.thread_row_max = trm;
            o.split_tile = tile;
            std::unique_ptr<Context> ctx(new Context());
            if (ctx->init(m, n, nnz, col, row_ptr, val, lhs, rhs, vartype, &o) != GDP_OKAY) return GDP_ERROR;
            double t;
            int rounds;
            if (time_it(*ctx, t, rounds) != GDP_OKAY) return GDP_ERROR;
            record(ctx->opts, rounds, t);
        }

    // stage 2: schedules on the fastest bins, one layout regridded per candidate
    struct Sched {
        int sync, ctas, cta_threads;
    };
    const Sched scheds[] = {{MEGAKERNEL, 0, 128}, {MEGAKERNEL, 4, 128}, {MEGAKERNEL, 0, 256}, {MEGAKERNEL, 2, 256},
                            {MEGAKERNEL, 0, 512}, {GPU_LOOP, 0, 256}};
    gdp_options lay = out.best;
    std::unique_ptr<Context> ctx(new Context());
    if (ctx->init(m, n, nnz, col, row_ptr, val, lhs, rhs, vartype, &lay) != GDP_OKAY) return GDP_ERROR;
    for (const Sched &sc : scheds) {
        if (sc.sync == lay.sync_type && sc.ctas == lay.ctas_per_sm && sc.cta_threads == lay.cta_threads)
            continue;  // timed in stage 1
        if (ctx->set_schedule(sc.sync, sc.ctas, sc.cta_threads) != GDP_OKAY) return GDP_ERROR;
        double t;
        int rounds;
        if (time_it(*ctx, t, rounds) != GDP_OKAY) return GDP_ERROR;
        record(ctx->opts, rounds, t);
    }
    {
        TuneCache &c = tune_cache();
        std::lock_guard<std::mutex> g(c.mu);
        c.entries[key] = out;
    }
    return report(out);
}

}  // namespace gdp
