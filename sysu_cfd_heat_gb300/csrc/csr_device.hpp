// A host CSR matrix uploaded as a SELL-32 matrix on the device (the standalone
// entry points of the C ABI: csr_api.cpp, gnn_api.cpp).
#pragma once

#include <vector>

#include "krylov.hpp"

namespace sysu {

// CSR (any column order, 0-based) -> row lists with the diagonal first.
inline void csr_rows_diag_first(int n, const int *rowptr, const int *col, const double *val, std::vector<int> &rp,
                                std::vector<int> &cl, std::vector<double> &vl) {
    rp.assign(n + 1, 0);
    cl.clear();
    vl.clear();
    cl.reserve((size_t)rowptr[n] + n);
    vl.reserve((size_t)rowptr[n] + n);
    for (int i = 0; i < n; ++i) {
        double d = 0.0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
            if (col[k] == i) d += val[k];
        cl.push_back(i);
        vl.push_back(d);
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            if (col[k] < 0 || col[k] >= n) throw CaseError{"column index out of range"};
            if (col[k] == i) continue;
            cl.push_back(col[k]);
            vl.push_back(val[k]);
        }
        rp[i + 1] = (int)cl.size();
    }
}

struct CsrDevice {
    SellPattern pat;
    SellDev A;
    DevBuf<double> val;
    std::vector<int> rp, cl;  // diagonal-first row lists of the pattern
    void load(int n, const int *rowptr, const int *col, const double *v, cudaStream_t st) {
        std::vector<double> vl;
        csr_rows_diag_first(n, rowptr, col, v, rp, cl, vl);
        pat = make_sell(n, rp, cl);
        A.upload(pat, st);
        upload_values(vl, st);
    }
    // new values for the same pattern (same rowptr and col as load)
    void reload_values(int n, const int *rowptr, const int *col, const double *v, cudaStream_t st) {
        std::vector<int> rp2, cl2;
        std::vector<double> vl;
        csr_rows_diag_first(n, rowptr, col, v, rp2, cl2, vl);
        if (n != pat.n || rp2 != rp || cl2 != cl) throw CaseError{"matrix pattern differs from the loaded one"};
        upload_values(vl, st);
    }
    void upload_values(const std::vector<double> &vl, cudaStream_t st) {
        std::vector<double> sv(pat.nnz, 0.0);
        for (int i = 0; i < pat.n; ++i)
            for (int k = rp[i]; k < rp[i + 1]; ++k) sv[pat.pos(i, k - rp[i])] = vl[k];
        val.upload(sv, st);
        SYSU_CUDA(cudaStreamSynchronize(st));
    }
};

}  // namespace sysu
