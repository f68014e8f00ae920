// Jacobi-preconditioned CG on a caller-owned device CSR matrix that allocates
// nothing: its scratch (residual, direction, product, inverse diagonal, the
// per-block partial sums, the grid barrier and the status words) lives in one
// file-scope device array, g_noalloc_scratch, of fixed size.
//
// Who needs it: callers that cannot call cudaMalloc -- host applications that
// own all device memory through their own pool and do not let libraries
// allocate behind their back, and time-critical loops that must not pay
// cudaMalloc/cudaFree, which synchronise the whole device.  Such a caller
// passes its own device buffers for the matrix, b and x, and this entry point
// uses only the static array besides them.
//
// Limits and rules (also in include/sysu_cfd.h):
// * at most SYSU_NOALLOC_MAX_ROWS rows (262,144); larger systems are rejected;
// * the array costs 8.4 MB on every GPU that loads the library, until exit;
// * all calls share the array and it keeps the last call's contents: each call
//   clears what must start at zero (barrier counter, status words) itself;
//   calls that overlap on the GPU (two streams, two threads) race on it;
// * every call looks up the array's device address (cudaGetSymbolAddress,
//   which allocates nothing) with the calling thread's device current, so a
//   cudaDeviceReset between calls is harmless; the first call on a device
//   also queries the cooperative-launch occupancy once and caches it;
// * every call waits for its stream (it reads the iteration count, residual
//   and status back), so it cannot be captured into a CUDA graph: a call on a
//   capturing stream is refused with SYSU_ERR_INPUT before anything is queued;
// * the CSR arrays are the caller's: a row pointer that decreases, a column
//   outside 0..n-1 or a row without a nonzero diagonal is reported as
//   SYSU_ERR_INPUT (first offending row in the message) and such entries are
//   never used to index x.  The caller must still make rowptr[n] no larger
//   than the length of d_col and d_val.
#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <mutex>
#include <string>

#include "../../include/sysu_cfd.h"
#include "device.hpp"

namespace {

constexpr int NA_MAX_ROWS = 262144;
constexpr int NA_KB = 256;
constexpr int NA_MAX_BLOCKS = 1024;
constexpr int NA_NV = 3;

// what a malformed CSR row was found to hold (low two bits of NaHeader::bad)
enum NaBad : int { NA_BAD_NONE = 0, NA_BAD_ROWPTR = 1, NA_BAD_COL = 2, NA_BAD_DIAG = 3 };

struct NaHeader {  // at the start of the array, cleared by every call
    sysu::GridBarrier barrier;
    int err;
    int status;
    int iters;
    int pad;
    double res;
    // lowest malformed row and what it holds, as (row << 2) | NaBad, kept by
    // atomicMin; all ones (set by the host before each call) when none is
    unsigned long long bad;
};

// layout in doubles: header (64 B) | r | p | q | dinv | partials (2*NA_NV*NA_MAX_BLOCKS)
constexpr size_t NA_HDR = 8;
static_assert(sizeof(NaHeader) <= NA_HDR * sizeof(double), "NaHeader must fit its 64-byte slot");
constexpr size_t NA_DOUBLES = NA_HDR + 4 * (size_t)NA_MAX_ROWS + 2 * (size_t)NA_NV * NA_MAX_BLOCKS;

static __device__ __align__(256) double g_noalloc_scratch[NA_DOUBLES];

struct NaArgs {
    int n;
    const int *rowptr, *col;
    const double *val, *b;
    double *x;
    double omega;
    int maxit;
    double eps;
    double *base;  // device address of g_noalloc_scratch
};

__shared__ double na_red_smem[NA_NV * (NA_KB / 32)];
__shared__ double na_red_res[NA_NV];

template <int NV>
__device__ bool na_reduce(double (&v)[NV], double *partials, int &parity, sysu::GridBarrier *gb, int *err) {
    sysu::block_sum<NV>(v, na_red_smem);
    double *buf = partials + (size_t)parity * NA_NV * gridDim.x;
    parity ^= 1;
    if (threadIdx.x == 0)
        for (int k = 0; k < NV; ++k) buf[(size_t)k * gridDim.x + blockIdx.x] = v[k];
    if (!sysu::grid_sync(gb, err)) return false;
    if (threadIdx.x < 32)
        for (int k = 0; k < NV; ++k) {
            double s = sysu::warp_sum_partials(buf + (size_t)k * gridDim.x, gridDim.x);
            if (threadIdx.x == 0) na_red_res[k] = s;
        }
    __syncthreads();
    for (int k = 0; k < NV; ++k) v[k] = na_red_res[k];
    __syncthreads();
    return true;
}

// Row i of A times x.  Entries whose column lies outside 0..n-1 are skipped
// (k_na_dinv has already reported them, and the solve does not run).
__device__ __forceinline__ double csr_row(const NaArgs &a, int i, const double *x) {
    double s = 0.0;
    for (int k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k) {
        int c = a.col[k];
        if ((unsigned)c < (unsigned)a.n) s += a.val[k] * x[c];
    }
    return s;
}

constexpr unsigned long long NA_GOOD = ~0ull;

__device__ __forceinline__ void na_report(NaHeader *h, int row, int kind) {
    atomicMin(&h->bad, ((unsigned long long)row << 2) | (unsigned long long)kind);
}

// D^-1 scaled by omega, and the checks of the caller's CSR: rows whose pointer
// decreases, columns outside 0..n-1 and rows without a nonzero diagonal are
// recorded in the header (lowest row) instead of being used.
__global__ void k_na_dinv(NaArgs a) {
    NaHeader *h = reinterpret_cast<NaHeader *>(a.base);
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    int k0 = a.rowptr[i], k1 = a.rowptr[i + 1];
    double d = 0.0;
    int kind = NA_BAD_NONE;
    if (k0 < 0 || k1 < k0) {
        kind = NA_BAD_ROWPTR;
    } else {
        for (int k = k0; k < k1; ++k) {
            int c = a.col[k];
            if ((unsigned)c >= (unsigned)a.n) { kind = NA_BAD_COL; break; }
            if (c == i) d += a.val[k];
        }
        if (kind == NA_BAD_NONE && !(d != 0.0 && isfinite(d))) kind = NA_BAD_DIAG;
    }
    if (kind != NA_BAD_NONE) {
        na_report(h, i, kind);
        d = 1.0;
    }
    a.base[NA_HDR + 3 * (size_t)NA_MAX_ROWS + i] = a.omega / d;
}

// Same recurrences as the SELL persistent CG (Templates Fig. 2.5, Jacobi).
__global__ void __launch_bounds__(NA_KB) k_na_cg(NaArgs a) {
    NaHeader *h = reinterpret_cast<NaHeader *>(a.base);
    double *r = a.base + NA_HDR, *p = r + NA_MAX_ROWS, *q = p + NA_MAX_ROWS, *dinv = q + NA_MAX_ROWS;
    double *partials = dinv + NA_MAX_ROWS;
    const int n = a.n, T = gridDim.x * NA_KB, t0 = blockIdx.x * NA_KB + threadIdx.x;
    // k_na_dinv ran before this launch on the same stream: every block reads the
    // same check result, so on a malformed matrix all leave together, before any
    // row loop or barrier
    if (__ldcg(&h->bad) != NA_GOOD) return;
    int parity = 0;
    double v3[3] = {0.0, 0.0, 0.0};
    for (int i = t0; i < n; i += T) {
        double bi = a.b[i];
        double ri = bi - csr_row(a, i, a.x);
        r[i] = ri;
        v3[0] += bi * bi;
        v3[1] += ri * ri;
        v3[2] += ri * (dinv[i] * ri);
    }
    if (!na_reduce<3>(v3, partials, parity, &h->barrier, &h->err)) return;
    double bnorm = sqrt(v3[0]);
    if (bnorm == 0.0) bnorm = 1.0;
    double res = sqrt(v3[1]) / bnorm, rho = v3[2], rho_prev = 1.0;
    int it = 0, status = sysu::DEV_OK;
    while (!(res < a.eps) && it < a.maxit) {
        if (!isfinite(res)) { status = sysu::DEV_NONFINITE; break; }
        ++it;
        double beta = (it == 1) ? 0.0 : rho / rho_prev;
        for (int i = t0; i < n; i += T) {
            double z = dinv[i] * r[i];
            p[i] = (it == 1) ? z : z + beta * p[i];
        }
        if (!sysu::grid_sync(&h->barrier, &h->err)) return;
        double v1[1] = {0.0};
        for (int i = t0; i < n; i += T) {
            double qi = csr_row(a, i, p);
            q[i] = qi;
            v1[0] += p[i] * qi;
        }
        if (!na_reduce<1>(v1, partials, parity, &h->barrier, &h->err)) return;
        if (v1[0] == 0.0) { status = sysu::DEV_BREAKDOWN; break; }
        double alpha = rho / v1[0];
        double v2[2] = {0.0, 0.0};
        for (int i = t0; i < n; i += T) {
            a.x[i] += alpha * p[i];
            double ri = r[i] - alpha * q[i];
            r[i] = ri;
            v2[0] += ri * ri;
            v2[1] += ri * (dinv[i] * ri);
        }
        if (!na_reduce<2>(v2, partials, parity, &h->barrier, &h->err)) return;
        res = sqrt(v2[0]) / bnorm;
        rho_prev = rho;
        rho = v2[1];
    }
    if (status == sysu::DEV_OK && !(res < a.eps)) status = isfinite(res) ? sysu::DEV_MAXITER : sysu::DEV_NONFINITE;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        h->status = status;
        h->iters = it;
        h->res = res;
    }
}

thread_local std::string g_na_err;
std::mutex g_na_mu;
int g_na_blocks[64] = {0};

int na_fail(int code, const std::string &m) {
    g_na_err = m;
    return code;
}

}  // namespace

extern "C" {

int sysu_csr_cg_noalloc(int n, const int *d_rowptr, const int *d_col, const double *d_val, const double *d_b,
                        double *d_x, int maxit, double eps, double omega, void *stream, int *iters, double *res,
                        int *status) {
    if (n < 1 || n > NA_MAX_ROWS)
        return na_fail(SYSU_ERR_INPUT, "sysu_csr_cg_noalloc: n = " + std::to_string(n) + " is outside 1.." +
                                           std::to_string(NA_MAX_ROWS) + " (the size of the static scratch)");
    if (!d_rowptr || !d_col || !d_val || !d_b || !d_x) return na_fail(SYSU_ERR_INPUT, "null device pointer");
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_fail(SYSU_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return na_fail(SYSU_ERR_CUDA, "device ordinal out of range");
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &cap);
    if (e != cudaSuccess) return na_fail(SYSU_ERR_CUDA, std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(e));
    if (cap != cudaStreamCaptureStatusNone)
        return na_fail(SYSU_ERR_INPUT, "sysu_csr_cg_noalloc waits for its stream to read the result back and "
                                       "cannot run on a stream that is being captured");
    // the array's device address in the current context: looked up on every call
    // (it allocates nothing), so a context torn down and re-created between calls
    // never leaves a stale address behind
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return na_fail(SYSU_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    double *base = static_cast<double *>(ptr);
    int blocks;
    {
        std::lock_guard<std::mutex> lock(g_na_mu);
        if (!g_na_blocks[dev]) {  // once per device: cooperative-launch occupancy
            int per_sm = 0, sms = 0, coop = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_na_cg, NA_KB, 0);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
            if (e != cudaSuccess) return na_fail(SYSU_ERR_CUDA, std::string("device query: ") + cudaGetErrorString(e));
            if (!coop || per_sm < 1) return na_fail(SYSU_ERR_CUDA, "cooperative launch unavailable");
            g_na_blocks[dev] = per_sm * sms < NA_MAX_BLOCKS ? per_sm * sms : NA_MAX_BLOCKS;
        }
        blocks = g_na_blocks[dev];
    }
    int G = (n + NA_KB - 1) / NA_KB;
    if (G > blocks) G = blocks;
    NaArgs a{n, d_rowptr, d_col, d_val, d_b, d_x, omega, maxit, eps, base};
    // what must start at zero: the barrier counter and the status words; the
    // malformed-row key starts at all ones (no row found)
    e = cudaMemsetAsync(base, 0, offsetof(NaHeader, bad), st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(reinterpret_cast<char *>(base) + offsetof(NaHeader, bad), 0xff, sizeof(unsigned long long),
                            st);
    if (e != cudaSuccess) return na_fail(SYSU_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    k_na_dinv<<<(n + NA_KB - 1) / NA_KB, NA_KB, 0, st>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return na_fail(SYSU_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    void *args[] = {&a};
    e = cudaLaunchCooperativeKernel((const void *)k_na_cg, dim3(G), dim3(NA_KB), args, 0, st);
    if (e != cudaSuccess) return na_fail(SYSU_ERR_CUDA, std::string("cooperative launch: ") + cudaGetErrorString(e));
    NaHeader h;
    e = cudaMemcpyAsync(&h, base, sizeof(NaHeader), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return na_fail(SYSU_ERR_CUDA, std::string("read-back: ") + cudaGetErrorString(e));
    if (h.bad != NA_GOOD) {
        static const char *what[] = {"", "a row pointer that decreases", "a column index outside 0..n-1",
                                     "no nonzero finite diagonal entry"};
        return na_fail(SYSU_ERR_INPUT, "sysu_csr_cg_noalloc: malformed CSR matrix: row " +
                                           std::to_string(h.bad >> 2) + " has " + what[h.bad & 3]);
    }
    if (iters) *iters = h.iters;
    if (res) *res = h.res;
    if (status) *status = h.err ? sysu::DEV_BARRIER_TIMEOUT : h.status;
    return SYSU_OK;
}

const char *sysu_noalloc_last_error(void) { return g_na_err.c_str(); }

}  // extern "C"
