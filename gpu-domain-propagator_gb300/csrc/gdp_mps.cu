// gdp_mps.cu -- a minimal free-format MPS reader (host code) producing the
// reference's CSR argument convention: rows in ROWS order without objective
// rows, entries of a row in column order, lhs/rhs with infinite sides as
// +-inf, variable bounds, and SCIP variable types (0 binary, 1 integer,
// 3 continuous). The reference reads MPS through python-mip
// (fileReader/readerInterface.py:52-145); this reader follows the same
// conventions: integer variables come from MARKER INTORG/INTEND blocks with
// default bounds [0, +inf); an integer variable with bounds [0, 1] is binary;
// UP with a negative value on a variable whose lower bound is still 0 makes
// the lower bound -inf; RANGES follow the MPS standard (E rows: R > 0 gives
// [rhs, rhs + R], R < 0 gives [rhs + R, rhs]; L rows [rhs - |R|, rhs]; G rows
// [rhs, rhs + |R|]).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <unordered_map>
#include <vector>

#include "gdp_context.h"

namespace {

struct Tokenizer {
    const char *p, *end;
    // next line's tokens (whitespace separated); false at end of text
    bool line(std::vector<std::string> &tok, bool &indented) {
        tok.clear();
        while (p < end) {
            const char *q = p;
            while (q < end && *q != '\n') q++;
            const char *s = p;
            p = q < end ? q + 1 : q;
            if (s == q) continue;
            if (*s == '*') continue;  // comment line
            indented = (*s == ' ' || *s == '\t');
            const char *c = s;
            while (c < q) {
                while (c < q && (*c == ' ' || *c == '\t' || *c == '\r')) c++;
                const char *b = c;
                while (c < q && *c != ' ' && *c != '\t' && *c != '\r') c++;
                if (c > b) tok.emplace_back(b, c - b);
            }
            if (!tok.empty()) return true;
        }
        return false;
    }
};

bool to_num(const std::string &s, double &v) {
    char *e = nullptr;
    v = std::strtod(s.c_str(), &e);
    return e && *e == '\0' && !s.empty();
}

}  // namespace

#pragma GCC visibility push(default)
extern "C" {

GDP_RETCODE gdp_mps_parse(const char *text, long long len, gdp_mps_problem *out) {
    if (!text || len < 0 || !out) {
        gdp::set_error("null MPS text or output");
        return GDP_ERROR;
    }
    std::memset(out, 0, sizeof(*out));
    const double INF = std::numeric_limits<double>::infinity();
    Tokenizer tk{text, text + len};
    std::vector<std::string> tok;
    bool ind = false;
    enum Sec { NONE, ROWS, COLUMNS, RHS, RANGES, BOUNDS, OTHER } sec = NONE;
    std::unordered_map<std::string, int> row_id;   // constraint rows: index; objective / free rows: -1
    std::unordered_map<std::string, int> col_id;
    std::vector<char> row_type;
    std::vector<double> rhs_v, range_v;
    std::vector<char> has_range;
    std::vector<std::vector<std::pair<int, double>>> rows;  // per row: (col, val) in column order
    std::vector<double> lb, ub;
    std::vector<char> is_int, lb_set;
    bool in_int = false;
    long long lineno = 0;
    auto fail = [&](const std::string &msg) {
        gdp::set_error("MPS line " + std::to_string(lineno) + ": " + msg);
        return GDP_ERROR;
    };
    while (tk.line(tok, ind)) {
        lineno++;
        if (!ind) {
            const std::string &h = tok[0];
            if (h == "NAME" || h == "OBJSENSE" || h == "OBJSENSE MAX") sec = OTHER;
            else if (h == "ROWS") sec = ROWS;
            else if (h == "COLUMNS") sec = COLUMNS;
            else if (h == "RHS") sec = RHS;
            else if (h == "RANGES") sec = RANGES;
            else if (h == "BOUNDS") sec = BOUNDS;
            else if (h == "ENDATA") break;
            else if (sec == OTHER) continue;  // e.g. the OBJSENSE value line
            else if (h == "MIN" || h == "MAX" || h == "MINIMIZE" || h == "MAXIMIZE") continue;
            else return fail("unknown section " + h);
            continue;
        }
        switch (sec) {
        case ROWS: {
            if (tok.size() < 2) return fail("ROWS entry needs type and name");
            const char t = tok[0][0];
            if (t == 'N') {
                row_id[tok[1]] = -1;
            } else if (t == 'L' || t == 'G' || t == 'E') {
                row_id[tok[1]] = (int)row_type.size();
                row_type.push_back(t);
                rhs_v.push_back(0.0);
                range_v.push_back(0.0);
                has_range.push_back(0);
                rows.emplace_back();
            } else {
                return fail("unknown row type " + tok[0]);
            }
            break;
        }
        case COLUMNS: {
            if (tok.size() >= 3 && tok[1] == "'MARKER'") {
                if (tok[2] == "'INTORG'") in_int = true;
                else if (tok[2] == "'INTEND'") in_int = false;
                break;
            }
            if (tok.size() < 3 || tok.size() % 2 == 0) return fail("COLUMNS entry needs name (row value)+");
            auto it = col_id.find(tok[0]);
            int j;
            if (it == col_id.end()) {
                j = (int)lb.size();
                col_id[tok[0]] = j;
                lb.push_back(0.0);
                ub.push_back(INF);
                is_int.push_back(in_int ? 1 : 0);
                lb_set.push_back(0);
            } else {
                j = it->second;
            }
            for (size_t k = 1; k + 1 < tok.size(); k += 2) {
                auto r = row_id.find(tok[k]);
                if (r == row_id.end()) return fail("unknown row " + tok[k]);
                double v;
                if (!to_num(tok[k + 1], v)) return fail("bad number " + tok[k + 1]);
                if (r->second >= 0 && v != 0.0) rows[r->second].emplace_back(j, v);
            }
            break;
        }
        case RHS:
        case RANGES: {
            // optional set name: an odd token count means the name is present
            size_t k = tok.size() % 2 == 1 ? 1 : 0;
            for (; k + 1 < tok.size(); k += 2) {
                auto r = row_id.find(tok[k]);
                if (r == row_id.end()) return fail("unknown row " + tok[k]);
                double v;
                if (!to_num(tok[k + 1], v)) return fail("bad number " + tok[k + 1]);
                if (r->second < 0) continue;  // objective constant / free row
                if (sec == RHS) {
                    rhs_v[r->second] = v;
                } else {
                    range_v[r->second] = v;
                    has_range[r->second] = 1;
                }
            }
            break;
        }
        case BOUNDS: {
            if (tok.size() < 3) return fail("BOUNDS entry too short");
            const std::string &t = tok[0];
            const bool novalue = t == "FR" || t == "MI" || t == "PL" || t == "BV";
            // with a bound set name: type name col [value]; without: type col [value]
            const size_t need = novalue ? 3 : 4;
            const size_t ci = tok.size() >= need ? 2 : 1;
            auto c = col_id.find(tok[ci]);
            if (c == col_id.end()) return fail("unknown column " + tok[ci]);
            const int j = c->second;
            double v = 0.0;
            if (!novalue && !to_num(tok[ci + 1 < tok.size() ? ci + 1 : ci], v)) return fail("bad bound value");
            if (t == "UP" || t == "UI") {
                ub[j] = v;
                if (v < 0.0 && !lb_set[j] && lb[j] == 0.0) lb[j] = -INF;
                if (t == "UI") is_int[j] = 1;
            } else if (t == "LO" || t == "LI") {
                lb[j] = v;
                lb_set[j] = 1;
                if (t == "LI") is_int[j] = 1;
            } else if (t == "FX") {
                lb[j] = v;
                ub[j] = v;
                lb_set[j] = 1;
            } else if (t == "FR") {
                lb[j] = -INF;
                ub[j] = INF;
                lb_set[j] = 1;
            } else if (t == "MI") {
                lb[j] = -INF;
                lb_set[j] = 1;
            } else if (t == "PL") {
                ub[j] = INF;
            } else if (t == "BV") {
                lb[j] = 0.0;
                ub[j] = 1.0;
                is_int[j] = 1;
                lb_set[j] = 1;
            } else {
                return fail("unsupported bound type " + t);
            }
            break;
        }
        default:
            break;
        }
    }
    const int m = (int)row_type.size(), n = (int)lb.size();
    long long nnz = 0;
    for (auto &r : rows) nnz += (long long)r.size();
    if (nnz > 2147483647LL) return fail("too many non-zeros");
    out->n_cons = m;
    out->n_vars = n;
    out->nnz = (int)nnz;
    out->row_ptr = (int *)std::malloc(sizeof(int) * (size_t)(m + 1));
    out->col = (int *)std::malloc(sizeof(int) * (size_t)std::max<long long>(nnz, 1));
    out->val = (double *)std::malloc(sizeof(double) * (size_t)std::max<long long>(nnz, 1));
    out->lhs = (double *)std::malloc(sizeof(double) * (size_t)std::max(m, 1));
    out->rhs = (double *)std::malloc(sizeof(double) * (size_t)std::max(m, 1));
    out->lb = (double *)std::malloc(sizeof(double) * (size_t)std::max(n, 1));
    out->ub = (double *)std::malloc(sizeof(double) * (size_t)std::max(n, 1));
    out->vartype = (int *)std::malloc(sizeof(int) * (size_t)std::max(n, 1));
    if (!out->row_ptr || !out->col || !out->val || !out->lhs || !out->rhs || !out->lb || !out->ub ||
        !out->vartype) {
        gdp_mps_free(out);
        gdp::set_error("host allocation failed (MPS)");
        return GDP_ERROR;
    }
    long long k = 0;
    out->row_ptr[0] = 0;
    for (int i = 0; i < m; i++) {
        for (auto &e : rows[i]) {  // columns were read in increasing index order
            out->col[k] = e.first;
            out->val[k] = e.second;
            k++;
        }
        out->row_ptr[i + 1] = (int)k;
        const double b = rhs_v[i], R = range_v[i];
        double lo, hi;
        if (row_type[i] == 'L') { lo = -INF; hi = b; }
        else if (row_type[i] == 'G') { lo = b; hi = INF; }
        else { lo = b; hi = b; }
        if (has_range[i]) {
            if (row_type[i] == 'L') lo = b - std::fabs(R);
            else if (row_type[i] == 'G') hi = b + std::fabs(R);
            else if (R > 0) hi = b + R;
            else lo = b + R;
        }
        out->lhs[i] = lo;
        out->rhs[i] = hi;
    }
    for (int j = 0; j < n; j++) {
        out->lb[j] = lb[j];
        out->ub[j] = ub[j];
        out->vartype[j] = !is_int[j] ? GDP_CONTINUOUS : (lb[j] == 0.0 && ub[j] == 1.0 ? GDP_BINARY : GDP_INTEGER);
    }
    return GDP_OKAY;
}

void gdp_mps_free(gdp_mps_problem *p) {
    if (!p) return;
    std::free(p->row_ptr);
    std::free(p->col);
    std::free(p->val);
    std::free(p->lhs);
    std::free(p->rhs);
    std::free(p->lb);
    std::free(p->ub);
    std::free(p->vartype);
    std::memset(p, 0, sizeof(*p));
}

}  // extern "C"
#pragma GCC visibility pop
