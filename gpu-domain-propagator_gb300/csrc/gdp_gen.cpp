// gdp_gen.cpp -- seeded synthetic MIP generators (see gdp_gen.h).
#include "gdp_gen.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kInf = 1e20;
constexpr int kRowsPerStream = 4096;

// splitmix64: seeds the per-block streams.
inline uint64_t splitmix64(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// xoshiro256** (Blackman & Vigna), one independent stream per seed.
struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (auto &w : s) w = splitmix64(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
    double uniform(double a, double b) { return a + (b - a) * uniform(); }
    int64_t randint(int64_t lo, int64_t hi) {  // inclusive
        const uint64_t span = (uint64_t)(hi - lo) + 1;
        return lo + (int64_t)(next() % span);
    }
    bool coin(double p) { return uniform() < p; }
};

inline uint64_t stream_seed(uint64_t seed, uint64_t tag, uint64_t idx) {
    uint64_t x = seed ^ (tag * 0xD1B54A32D192ED03ULL);
    splitmix64(x);
    x ^= idx * 0x9E3779B97F4A7C15ULL;
    return splitmix64(x);
}

// Clipped Zipf row lengths: numpy-style zipf(s) (P(k) ~ k^-s, k >= 1), then
// clipped into [lo, hi] (the mass below lo goes to lo, above hi to hi).
struct ZipfTable {
    int lo, hi;
    std::vector<double> cdf;  // cdf[i] = P(len <= lo + i)
    ZipfTable(double s, int lo_, int hi_) : lo(lo_), hi(hi_) {
        const int K = hi;
        std::vector<double> p(K + 1, 0.0);
        double z = 0.0;
        for (int k = 1; k <= K; k++) { p[k] = std::pow((double)k, -s); z += p[k]; }
        // tail k > K approximated by the integral of x^-s from K+0.5 to inf
        const double tail = std::pow(K + 0.5, 1.0 - s) / (s - 1.0);
        z += tail;
        cdf.assign(hi - lo + 1, 0.0);
        double acc = 0.0;
        for (int k = 1; k < lo; k++) acc += p[k];
        for (int len = lo; len <= hi; len++) {
            acc += p[len];
            cdf[len - lo] = acc / z;
        }
        cdf.back() = 1.0;  // the tail mass lands on hi
    }
    int sample(Rng &r) const {
        const double u = r.uniform();
        const auto it = std::upper_bound(cdf.begin(), cdf.end(), u);
        const int idx = (int)(it - cdf.begin());
        return lo + std::min(idx, hi - lo);
    }
};

// L distinct columns in [0, n), ascending.
void sample_columns(Rng &r, int n, int L, std::vector<int> &out) {
    out.clear();
    if (L >= n) {
        for (int j = 0; j < n; j++) out.push_back(j);
        return;
    }
    if ((int64_t)L * 4 > n) {  // selection sampling (Knuth, algorithm S)
        int need = L;
        for (int j = 0; j < n && need > 0; j++)
            if (r.uniform() * (n - j) < need) { out.push_back(j); need--; }
        return;
    }
    while ((int)out.size() < L) {
        const int missing = L - (int)out.size();
        for (int t = 0; t < missing; t++) out.push_back((int)r.randint(0, n - 1));
        std::sort(out.begin(), out.end());
        out.erase(std::unique(out.begin(), out.end()), out.end());
    }
}

bool alloc_instance(gdp_instance *o, int m, int n, int64_t nnz) {
    std::memset(o, 0, sizeof(*o));
    if (nnz > 2147483647LL) return false;
    o->m = m; o->n = n; o->nnz = (int)nnz;
    o->row_ptr = (int *)std::malloc(sizeof(int) * (size_t)(m + 1));
    o->col = (int *)std::malloc(sizeof(int) * (size_t)std::max<int64_t>(nnz, 1));
    o->val = (double *)std::malloc(sizeof(double) * (size_t)std::max<int64_t>(nnz, 1));
    o->lhs = (double *)std::malloc(sizeof(double) * (size_t)std::max(m, 1));
    o->rhs = (double *)std::malloc(sizeof(double) * (size_t)std::max(m, 1));
    o->lb = (double *)std::malloc(sizeof(double) * (size_t)std::max(n, 1));
    o->ub = (double *)std::malloc(sizeof(double) * (size_t)std::max(n, 1));
    o->vartype = (int *)std::malloc(sizeof(int) * (size_t)std::max(n, 1));
    o->x0 = (double *)std::malloc(sizeof(double) * (size_t)std::max(n, 1));
    if (!o->row_ptr || !o->col || !o->val || !o->lhs || !o->rhs || !o->lb || !o->ub ||
        !o->vartype || !o->x0) {
        gdp_gen_free(o);
        return false;
    }
    return true;
}

double draw_coef(Rng &r, const gdp_gen_params *p) {
    double mag;
    if (p->coef_dist == 1)
        mag = std::exp(r.uniform(std::log(p->coef_min), std::log(p->coef_max)));
    else
        mag = r.uniform(p->coef_min, p->coef_max);
    if (p->frac_int_coef > 0 && r.coin(p->frac_int_coef)) mag = std::max(1.0, std::round(mag));
    return r.coin(0.5) ? mag : -mag;
}

// Variable types, bounds and hidden point for vars [j0, j1).
void gen_vars(const gdp_gen_params *p, uint64_t seed, int j0, int j1, gdp_instance *o) {
    const double fi = p->frac_int_vars;
    const double finf = fi < 1.0 ? p->frac_inf_vars / (1.0 - fi) : 0.0;
    const double B = p->cont_bound_max;
#pragma omp parallel for schedule(static)
    for (int blk = j0 / kRowsPerStream; blk <= (j1 - 1) / kRowsPerStream; blk++) {
        Rng r(stream_seed(seed, 11, (uint64_t)blk));
        const int a = std::max(j0, blk * kRowsPerStream), b = std::min(j1, (blk + 1) * kRowsPerStream);
        for (int j = a; j < b; j++) {
            if (r.coin(fi)) {
                const int u = (int)r.randint(1, std::max(1, p->int_ub_max));
                o->vartype[j] = (u == 1) ? 0 : 1;
                o->lb[j] = 0.0;
                o->ub[j] = (double)u;
                o->x0[j] = (double)r.randint(0, u);
            } else {
                o->vartype[j] = 3;
                if (r.coin(finf)) {
                    if (r.coin(0.5)) {
                        o->lb[j] = -kInf;
                        o->ub[j] = r.uniform(1.0, B);
                        o->x0[j] = o->ub[j] - r.uniform(0.0, B);
                    } else {
                        o->lb[j] = -r.uniform(1.0, B);
                        o->ub[j] = kInf;
                        o->x0[j] = o->lb[j] + r.uniform(0.0, B);
                    }
                } else {
                    o->lb[j] = -r.uniform(1.0, B);
                    o->ub[j] = r.uniform(1.0, B);
                    o->x0[j] = r.uniform(o->lb[j], o->ub[j]);
                }
            }
        }
    }
}

// Random rows [i0, i1) over vars [c0, c0 + nc), lengths already in row_ptr.
// Equality rows draw their columns from the continuous variables only: an
// equality row that contains integer variables pins them at x0 up to the
// rounding error of its activity, and EPSFLOOR/EPSCEIL of a candidate a few
// ulps below an integer then cuts x0 off (a spurious infeasibility that the
// reference's arithmetic produces as well).
void gen_rows(const gdp_gen_params *p, uint64_t seed, int i0, int i1, int c0, int nc,
              gdp_instance *o) {
    std::vector<int> cont;  // continuous vars of [c0, c0 + nc), relative to c0, ascending
    if (p->frac_equality > 0)
        for (int j = 0; j < nc; j++)
            if (o->vartype[c0 + j] == 3) cont.push_back(j);
#pragma omp parallel for schedule(dynamic, 1)
    for (int blk = i0 / kRowsPerStream; blk <= (i1 - 1) / kRowsPerStream; blk++) {
        Rng r(stream_seed(seed, 22, (uint64_t)blk));
        std::vector<int> cols;
        const int a = std::max(i0, blk * kRowsPerStream), b = std::min(i1, (blk + 1) * kRowsPerStream);
        for (int i = a; i < b; i++) {
            const int L = o->row_ptr[i + 1] - o->row_ptr[i];
            const bool equality = p->frac_equality > 0 && (int)cont.size() >= L && r.coin(p->frac_equality);
            sample_columns(r, equality ? (int)cont.size() : nc, L, cols);
            if (equality)
                for (int &c : cols) c = cont[c];
            double act = 0.0;
            for (int t = 0; t < L; t++) {
                const int k = o->row_ptr[i] + t;
                o->col[k] = c0 + cols[t];
                o->val[k] = draw_coef(r, p);
                act += o->val[k] * o->x0[o->col[k]];
            }
            if (equality) {
                o->lhs[i] = act;
                o->rhs[i] = act;
            } else {
                o->lhs[i] = act - r.uniform(0.0, p->slack_max) * L;
                o->rhs[i] = act + r.uniform(0.0, p->slack_max) * L;
                if (r.coin(p->frac_one_sided)) o->lhs[i] = -kInf;
            }
        }
    }
}

// Row lengths for rows [i0, i1) (into lens[i - i0]).
void gen_lengths(const gdp_gen_params *p, uint64_t seed, int i0, int i1, int ncols,
                 std::vector<int> &lens) {
    lens.assign(i1 - i0, 0);
    const ZipfTable *zt = nullptr;
    ZipfTable table(p->len_dist == 1 ? p->zipf_s : 2.0, std::max(1, p->len_min),
                    std::max(p->len_min, p->len_max));
    if (p->len_dist == 1) zt = &table;
#pragma omp parallel for schedule(static)
    for (int blk = i0 / kRowsPerStream; blk <= (i1 - 1) / kRowsPerStream; blk++) {
        Rng r(stream_seed(seed, 33, (uint64_t)blk));
        const int a = std::max(i0, blk * kRowsPerStream), b = std::min(i1, (blk + 1) * kRowsPerStream);
        for (int i = a; i < b; i++) {
            int L = zt ? zt->sample(r) : (int)r.randint(p->len_min, p->len_max);
            lens[i - i0] = std::min(L, ncols);
        }
    }
    if (p->n_dense_rows > 0) {
        Rng r(stream_seed(seed, 44, 0));
        for (int t = 0; t < p->n_dense_rows && i1 > i0; t++)
            lens[r.randint(0, i1 - i0 - 1)] = std::min(p->dense_len, ncols);
    }
}

}  // namespace

extern "C" {

int gdp_gen_default_params(int workload, gdp_gen_params *p) {
    std::memset(p, 0, sizeof(*p));
    p->len_dist = 0;
    p->len_min = 2;
    p->len_max = 16;
    p->zipf_s = 1.8;
    p->coef_dist = 0;
    p->coef_min = 0.5;
    p->coef_max = 10.0;
    p->frac_int_coef = 0.2;
    p->frac_int_vars = 0.5;
    p->int_ub_max = 20;
    p->frac_inf_vars = 0.1;
    p->cont_bound_max = 100.0;
    p->slack_max = 5.0;
    p->frac_one_sided = 0.2;
    p->frac_equality = 0.0;
    if (workload == 0) {
        p->m = 2000;
        p->n = 1500;
        return 0;
    }
    if (workload == 1) {
        p->m = 2000000;
        p->n = 1500000;
        p->len_dist = 1;
        p->len_min = 2;
        p->len_max = 20000;
        p->n_dense_rows = 32;
        p->dense_len = 100000;
        p->coef_dist = 1;
        p->coef_min = 1e-2;
        p->coef_max = 1e3;
        p->frac_int_coef = 0.0;
        p->frac_equality = 0.3;
        return 0;
    }
    return -1;
}

int gdp_gen_random_mip(const gdp_gen_params *p, gdp_instance *out) {
    if (!p || !out || p->m <= 0 || p->n <= 0 || p->len_min < 1 || p->len_max < p->len_min)
        return -1;
    std::vector<int> lens;
    gen_lengths(p, p->seed, 0, p->m, p->n, lens);
    int64_t nnz = 0;
    for (int L : lens) nnz += L;
    if (!alloc_instance(out, p->m, p->n, nnz)) return -2;
    out->row_ptr[0] = 0;
    for (int i = 0; i < p->m; i++) out->row_ptr[i + 1] = out->row_ptr[i] + lens[i];
    gen_vars(p, p->seed, 0, p->n, out);
    gen_rows(p, p->seed, 0, p->m, 0, p->n, out);
    return 0;
}

int gdp_gen_cover_knapsack(int n_cover_rows, int n_knap_rows, int n_bin, int n_cont,
                           int cover_min, int cover_max, int knap_min, int knap_max,
                           uint64_t seed, gdp_instance *out) {
    if (n_cover_rows < 0 || n_knap_rows < 0 || n_bin <= 0 || n_cont < 0 || cover_min < 1 ||
        cover_max < cover_min || knap_min < 1 || knap_max < knap_min)
        return -1;
    const int m = n_cover_rows + n_knap_rows, n = n_bin + n_cont;
    std::vector<int> lens(m);
    {
        Rng r(stream_seed(seed, 55, 0));
        for (int i = 0; i < n_cover_rows; i++) lens[i] = std::min(n_bin, (int)r.randint(cover_min, cover_max));
        for (int i = n_cover_rows; i < m; i++) lens[i] = std::min(n, (int)r.randint(knap_min, knap_max));
    }
    int64_t nnz = 0;
    for (int L : lens) nnz += L;
    if (!alloc_instance(out, m, n, nnz)) return -2;
    out->row_ptr[0] = 0;
    for (int i = 0; i < m; i++) out->row_ptr[i + 1] = out->row_ptr[i] + lens[i];
    Rng rv(stream_seed(seed, 66, 0));
    for (int j = 0; j < n_bin; j++) {
        out->vartype[j] = 0;
        out->lb[j] = 0.0;
        out->ub[j] = 1.0;
        out->x0[j] = rv.coin(0.08) ? 1.0 : 0.0;
    }
    for (int j = n_bin; j < n; j++) {
        out->vartype[j] = 3;
        out->lb[j] = 0.0;
        out->ub[j] = rv.uniform(1.0, 10.0);
        out->x0[j] = rv.uniform(0.0, 0.2) * out->ub[j];
    }
    // cover rows (sequential so that x0 repairs are deterministic)
    Rng rc(stream_seed(seed, 77, 0));
    std::vector<int> cols;
    for (int i = 0; i < n_cover_rows; i++) {
        sample_columns(rc, n_bin, lens[i], cols);
        bool covered = false;
        for (int t = 0; t < lens[i]; t++) {
            const int k = out->row_ptr[i] + t;
            out->col[k] = cols[t];
            out->val[k] = 1.0;
            covered |= out->x0[cols[t]] > 0.5;
        }
        if (!covered) out->x0[cols[rc.randint(0, lens[i] - 1)]] = 1.0;
        out->lhs[i] = 1.0;
        out->rhs[i] = kInf;
    }
    for (int i = n_cover_rows; i < m; i++) {
        sample_columns(rc, n, lens[i], cols);
        double sum = 0.0, use = 0.0;
        for (int t = 0; t < lens[i]; t++) {
            const int k = out->row_ptr[i] + t;
            out->col[k] = cols[t];
            out->val[k] = (double)rc.randint(1, 1000);
            sum += out->val[k];
            use += out->val[k] * out->x0[cols[t]];
        }
        out->lhs[i] = -kInf;
        out->rhs[i] = std::max(std::floor(0.3 * sum), std::ceil(use));
    }
    return 0;
}

int gdp_gen_chains(int m, int n, int chain_max, double frac_int_vars, double frac_inf_vars,
                   double frac_equality, int make_infeasible, uint64_t seed, gdp_instance *out) {
    if (m < 4 || n < 4 || chain_max < 1) return -1;
    const int m_chain = m / 2;
    // chains over vars [0, nv_chain): each chain of length L uses L+1 vars and L rows
    std::vector<int> chain_len;
    {
        Rng r(stream_seed(seed, 88, 0));
        int rows = 0;
        while (rows < m_chain) {
            int L = (int)std::exp(r.uniform(0.0, std::log((double)chain_max + 1.0)));
            L = std::max(1, std::min(L, m_chain - rows));
            chain_len.push_back(L);
            rows += L;
        }
    }
    const int nv_chain = m_chain + (int)chain_len.size();
    if (nv_chain + 2 > n) return -3;
    gdp_gen_params p;
    gdp_gen_default_params(1, &p);
    p.m = m - m_chain;
    p.n = n - nv_chain;
    p.n_dense_rows = 0;
    p.frac_int_vars = frac_int_vars;
    p.frac_inf_vars = frac_inf_vars;
    p.frac_equality = frac_equality;
    p.len_max = std::min(p.len_max, std::max(2, p.n / 4));
    std::vector<int> lens;
    gen_lengths(&p, seed, m_chain, m, p.n, lens);
    int64_t nnz = 2LL * m_chain;
    for (int L : lens) nnz += L;
    if (!alloc_instance(out, m, n, nnz)) return -2;
    out->row_ptr[0] = 0;
    for (int i = 0; i < m_chain; i++) out->row_ptr[i + 1] = out->row_ptr[i] + 2;
    for (int i = m_chain; i < m; i++) out->row_ptr[i + 1] = out->row_ptr[i] + lens[i - m_chain];
    // non-chain vars and rows (the power-law part)
    gen_vars(&p, seed, nv_chain, n, out);
    gen_rows(&p, seed, m_chain, m, nv_chain, p.n, out);
    // chains: x0 first (feasible), then bounds that make propagation walk the chain
    Rng r(stream_seed(seed, 99, 0));
    int v = 0, row = 0;
    const int bad_chain = make_infeasible ? (int)r.randint(0, (int64_t)chain_len.size() - 1) : -1;
    for (size_t c = 0; c < chain_len.size(); c++) {
        const int L = chain_len[c];
        double x = r.uniform(0.0, 10.0);
        double csum = 0.0;
        for (int t = 0; t <= L; t++) {
            const int j = v + t;
            const bool is_int = r.coin(frac_int_vars);
            out->vartype[j] = is_int ? 1 : 3;
            if (t > 0) {
                const double ci = r.uniform(0.0, 3.0);
                csum += ci;
                const int k = out->row_ptr[row];
                out->col[k] = j - 1;  // x_{i+1} - x_i <= c_i, columns ascending
                out->val[k] = -1.0;
                out->col[k + 1] = j;
                out->val[k + 1] = 1.0;
                out->lhs[row] = -kInf;
                out->rhs[row] = ci;
                row++;
                const double step = r.uniform(0.0, ci);
                x += is_int ? std::floor(step) : step;
            }
            if (is_int) x = std::floor(x);
            out->x0[j] = x;
            const bool inf_b = r.coin(frac_inf_vars);
            out->lb[j] = inf_b ? -kInf : x - 1e6;
            out->ub[j] = inf_b ? kInf : x + 1e6;
        }
        const int j0 = v, jL = v + L;
        out->ub[j0] = out->x0[j0] + r.uniform(0.0, 5.0);
        if (out->vartype[j0] != 3) out->ub[j0] = std::floor(out->ub[j0]);
        if ((int)c == bad_chain)
            out->lb[jL] = std::ceil(out->ub[j0] + csum + 1.0 + r.uniform(0.0, 5.0));
        else
            out->lb[jL] = std::ceil(out->x0[jL] - r.uniform(0.0, 5.0) - 1.0);
        if (out->vartype[jL] == 3 && out->lb[jL] > out->x0[jL] && (int)c != bad_chain)
            out->lb[jL] = out->x0[jL];
        v += L + 1;
    }
    // spare vars between the chains and the power-law block stay unused
    for (int j = v; j < nv_chain; j++) {
        out->vartype[j] = 3; out->lb[j] = 0.0; out->ub[j] = 1.0; out->x0[j] = 0.0;
    }
    return 0;
}

void gdp_gen_free(gdp_instance *o) {
    if (!o) return;
    std::free(o->row_ptr); std::free(o->col); std::free(o->val); std::free(o->lhs);
    std::free(o->rhs); std::free(o->lb); std::free(o->ub); std::free(o->vartype); std::free(o->x0);
    std::memset(o, 0, sizeof(*o));
}

}  // extern "C"
