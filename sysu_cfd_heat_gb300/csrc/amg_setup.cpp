// Host part of the aggregation multigrid (see amg.hpp): aggregation, coarse
// patterns and the Galerkin gather lists, built once per matrix pattern.
#include <algorithm>
#include <cmath>
#include <string>
#include <unordered_map>

#include "amg.hpp"
#include "case.hpp"

namespace sysu {

namespace {

// Greedy aggregation of one level (the three passes of amg.hpp).  Returns the
// number of aggregates; agg[i] is row i's aggregate.
int aggregate(const SellPattern &p, const std::vector<double> &val, double theta, std::vector<int> &agg) {
    const int n = p.n;
    // strong neighbours of each row, in row order, with their coupling strength
    std::vector<int> sptr(n + 1, 0), scol;
    std::vector<double> sval;
    scol.reserve(p.nnz_true);
    sval.reserve(p.nnz_true);
    for (int i = 0; i < n; ++i) {
        const double d = val[p.pos(i, 0)];
        const double sg = d < 0.0 ? -1.0 : 1.0;
        double cmax = 0.0;
        for (int k = 1; k < p.row_len[i]; ++k) {
            const int j = p.col[p.pos(i, k)];
            if (j == i) continue;
            cmax = std::max(cmax, -val[p.pos(i, k)] * sg);
        }
        if (cmax > 0.0) {
            for (int k = 1; k < p.row_len[i]; ++k) {
                const int j = p.col[p.pos(i, k)];
                if (j == i) continue;
                const double c = -val[p.pos(i, k)] * sg;
                if (c >= theta * cmax) {
                    scol.push_back(j);
                    sval.push_back(c);
                }
            }
        }
        sptr[i + 1] = (int)scol.size();
    }
    agg.assign(n, -1);
    int na = 0;
    // pass 1: seeds whose strong neighbours are all free
    for (int i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        bool free = true;
        for (int q = sptr[i]; q < sptr[i + 1] && free; ++q) free = agg[scol[q]] < 0;
        if (!free) continue;
        agg[i] = na;
        for (int q = sptr[i]; q < sptr[i + 1]; ++q) agg[scol[q]] = na;
        ++na;
    }
    // pass 2: the strongest aggregated strong neighbour (first on ties)
    for (int i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        int best = -1;
        double bc = -1.0;
        for (int q = sptr[i]; q < sptr[i + 1]; ++q) {
            const int j = scol[q];
            if (agg[j] >= 0 && sval[q] > bc) {
                bc = sval[q];
                best = agg[j];
            }
        }
        if (best >= 0) agg[i] = best;
    }
    // pass 3: singletons
    for (int i = 0; i < n; ++i)
        if (agg[i] < 0) agg[i] = na++;
    return na;
}

}  // namespace

std::vector<MgHostLevel> mg_build_hierarchy(const SellPattern &fine, const std::vector<double> &val, double theta,
                                            int dense_max) {
    std::vector<MgHostLevel> L;
    L.emplace_back();
    L[0].n = fine.n;
    L[0].pat = fine;
    L[0].val = val;
    while ((int)L.size() < MG_MAX_LEVELS && L.back().n > dense_max) {
        MgHostLevel &f = L.back();
        const SellPattern &p = f.pat;
        const int n = p.n;
        const int na = aggregate(p, f.val, theta, f.agg);
        if (na >= n) {  // no coarsening possible (no couplings): stop here
            f.agg.clear();
            break;
        }
        // members of each aggregate, ascending
        f.mem_ptr.assign(na + 1, 0);
        for (int i = 0; i < n; ++i) ++f.mem_ptr[f.agg[i] + 1];
        for (int I = 0; I < na; ++I) f.mem_ptr[I + 1] += f.mem_ptr[I];
        f.mem_idx.assign(n, 0);
        {
            std::vector<int> fill(f.mem_ptr.begin(), f.mem_ptr.end() - 1);
            for (int i = 0; i < n; ++i) f.mem_idx[fill[f.agg[i]]++] = i;
        }
        // coarse rows: diagonal first, then columns in order of first appearance;
        // every fine true entry goes to one coarse entry
        std::vector<int> crp(na + 1, 0), ccol;
        std::vector<std::vector<long>> csrc;  // per coarse CSR entry: fine SELL positions
        ccol.reserve(p.nnz_true);
        std::unordered_map<int, int> slot;
        for (int I = 0; I < na; ++I) {
            slot.clear();
            const int base = (int)ccol.size();
            ccol.push_back(I);
            csrc.emplace_back();
            slot[I] = base;
            for (int m = f.mem_ptr[I]; m < f.mem_ptr[I + 1]; ++m) {
                const int i = f.mem_idx[m];
                for (int k = 0; k < p.row_len[i]; ++k) {
                    const long pos = p.pos(i, k);
                    const int J = f.agg[p.col[pos]];
                    auto it = slot.find(J);
                    int e;
                    if (it == slot.end()) {
                        e = (int)ccol.size();
                        slot[J] = e;
                        ccol.push_back(J);
                        csrc.emplace_back();
                    } else {
                        e = it->second;
                    }
                    csrc[e].push_back(pos);
                }
            }
            crp[I + 1] = (int)ccol.size();
        }
        MgHostLevel c;
        c.n = na;
        c.pat = make_sell(na, crp, ccol);
        c.val.assign(c.pat.nnz, 0.0);
        // gather lists in coarse SELL position order (padding: empty lists)
        f.gal_ptr.assign(c.pat.nnz + 1, 0);
        std::vector<int> pos_entry(c.pat.nnz, -1);
        for (int I = 0; I < na; ++I)
            for (int k = 0; k < c.pat.row_len[I]; ++k) pos_entry[c.pat.pos(I, k)] = crp[I] + k;
        for (long q = 0; q < c.pat.nnz; ++q) {
            const int e = pos_entry[q];
            f.gal_ptr[q + 1] = f.gal_ptr[q] + (e >= 0 ? (int)csrc[e].size() : 0);
        }
        f.gal_src.assign(f.gal_ptr[c.pat.nnz], 0);
        for (long q = 0; q < c.pat.nnz; ++q) {
            const int e = pos_entry[q];
            if (e < 0) continue;
            int o = f.gal_ptr[q];
            double s = 0.0;
            for (long src : csrc[e]) {
                f.gal_src[o++] = (int)src;
                s += f.val[src];
            }
            c.val[q] = s;
        }
        L.push_back(std::move(c));
    }
    return L;
}

}  // namespace sysu

// ---- host-only export of the hierarchy (no device work; CPU tests) ---------
#include "../../include/sysu_cfd.h"
#include "csr_device.hpp"

namespace {
thread_local std::string g_mg_err;

std::vector<sysu::MgHostLevel> host_hierarchy(int n, const int *rowptr, const int *col, const double *val,
                                              double theta, int dense_max) {
    std::vector<int> rp, cl;
    std::vector<double> vl;
    sysu::csr_rows_diag_first(n, rowptr, col, val, rp, cl, vl);
    sysu::SellPattern p = sysu::make_sell(n, rp, cl);
    std::vector<double> sv(p.nnz, 0.0);
    for (int i = 0; i < n; ++i)
        for (int k = rp[i]; k < rp[i + 1]; ++k) sv[p.pos(i, k - rp[i])] = vl[k];
    return sysu::mg_build_hierarchy(p, sv, theta, dense_max);
}
}  // namespace

extern "C" {

int sysu_mg_hierarchy(int n, const int *rowptr, const int *col, const double *val, double theta, int dense_max,
                      int max_levels, int *nlevels, int *rows, long *nnz) {
    if (n < 1 || !rowptr || !col || !val || !nlevels || !(theta > 0.0 && theta < 1.0) || dense_max < 1) {
        g_mg_err = "sysu_mg_hierarchy: bad arguments";
        return SYSU_ERR_INPUT;
    }
    try {
        auto H = host_hierarchy(n, rowptr, col, val, theta, dense_max);
        *nlevels = (int)H.size();
        for (int l = 0; l < (int)H.size() && l < max_levels; ++l) {
            if (rows) rows[l] = H[l].n;
            if (nnz) nnz[l] = H[l].pat.nnz_true;
        }
        return SYSU_OK;
    } catch (const sysu::CaseError &e) {
        g_mg_err = e.msg;
        return SYSU_ERR_INPUT;
    }
}

int sysu_mg_level(int n, const int *rowptr, const int *col, const double *val, double theta, int dense_max,
                  int level, int *agg, int *rowptr_out, int *col_out, double *val_out) {
    if (n < 1 || !rowptr || !col || !val || level < 0) {
        g_mg_err = "sysu_mg_level: bad arguments";
        return SYSU_ERR_INPUT;
    }
    try {
        auto H = host_hierarchy(n, rowptr, col, val, theta, dense_max);
        if (level >= (int)H.size()) throw sysu::CaseError{"sysu_mg_level: no such level"};
        const sysu::MgHostLevel &h = H[level];
        if (agg && !h.agg.empty()) std::copy(h.agg.begin(), h.agg.end(), agg);
        if (rowptr_out) {
            long k = 0;
            rowptr_out[0] = 0;
            for (int i = 0; i < h.n; ++i) {
                for (int j = 0; j < h.pat.row_len[i]; ++j, ++k) {
                    if (col_out) col_out[k] = h.pat.col[h.pat.pos(i, j)];
                    if (val_out) val_out[k] = h.val[h.pat.pos(i, j)];
                }
                rowptr_out[i + 1] = (int)k;
            }
        }
        return SYSU_OK;
    } catch (const sysu::CaseError &e) {
        g_mg_err = e.msg;
        return SYSU_ERR_INPUT;
    }
}

const char *sysu_mg_last_error(void) { return g_mg_err.c_str(); }

}  // extern "C"
