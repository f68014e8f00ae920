// Device part of the aggregation multigrid (see amg.hpp): Galerkin values,
// smoother weights, the coarsest-level inverse and the V-cycle kernels.
//
// Every cycle kernel is a flat grid-stride loop over rows (SELL-32: thread i
// reads row i's entries at sl_ptr[i/32] + 32 k + i%32, so a warp's loads are
// coalesced; on coarse levels a group of lanes per row) and returns at once when
// the flexible CG it serves has finished (*done != 0), so the rest of a loop body
// of iterations costs little past convergence.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <memory>
#include <type_traits>

#include "amg.hpp"
#include "krylov_dev.cuh"

namespace sysu {
namespace {

constexpr int MB = 256;  // threads per block of the flat kernels
constexpr int DENSE_THREADS = 1024;

struct MgView {
    int n;
    const int *sl_ptr, *sl_w, *col;
    const float *val;
};

int flat_blocks(long n) { return (int)std::max(1L, std::min((n + MB - 1) / MB, (long)num_sms() * 8)); }

// f(std::integral_constant<int, G>) for the group width g (1, 2, 4, ..., 32)
template <class F>
void with_group(int g, F f) {
    switch (g) {
        case 1: f(std::integral_constant<int, 1>{}); break;
        case 2: f(std::integral_constant<int, 2>{}); break;
        case 4: f(std::integral_constant<int, 4>{}); break;
        case 8: f(std::integral_constant<int, 8>{}); break;
        case 16: f(std::integral_constant<int, 16>{}); break;
        default: f(std::integral_constant<int, 32>{}); break;
    }
}

// coarse value at stored position q = sum of its fine entries (fixed order)
__global__ void k_mg_galerkin(long npos, const int *gal_ptr, const int *gal_src, const double *fval, double *cval,
                              float *cval32) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < npos; q += (long)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int k = gal_ptr[q]; k < gal_ptr[q + 1]; ++k) s += fval[gal_src[k]];
        cval[q] = s;
        cval32[q] = (float)s;
    }
}

// w_i = omega / a_ii (entry 0 of row i is its diagonal)
__global__ void k_mg_weights(int n, const int *sl_ptr, const double *val, double omega, float *w) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double d = val[sl_ptr[i >> 5] + (i & 31)];
        w[i] = (float)(d != 0.0 ? omega / d : 0.0);
    }
}

__device__ __forceinline__ float row_times(const MgView &A, int i, const float *x) {
    const int base = A.sl_ptr[i >> 5], wd = A.sl_w[i >> 5], lane = i & 31;
    float s = 0.f;
    for (int k = 0; k < wd; ++k) {
        const int pos = base + k * 32 + lane;
        s += A.val[pos] * x[A.col[pos]];
    }
    return s;
}

// Coarse levels have wide rows (aggregation merges neighbourhoods) and few of
// them: one thread per row walks a long chain of dependent loads (column, then
// the gathered value) while most of the GPU idles; a 500-row level took 10 us.
// The cycle kernels therefore give each row (or aggregate) a group of G lanes
// of one warp: lane s of the group takes entries s, s + G, ..., and the partial
// sums meet in a fixed xor butterfly, so every lane of the group holds the sum
// and every run adds in the same order.  The loops advance whole warps (the
// butterfly needs every lane), with the lanes past the end contributing 0.
constexpr int MG_GROUP_ENTRIES = 6;  // entries per lane aimed at when choosing G

// Lanes per row for `rows` rows of `width` entries: enough that a lane takes
// about MG_GROUP_ENTRIES entries, but no more than the GPU's resident threads
// need -- a level that fills the SMs at one row per thread (level 1 of the 2M-row
// p' system, 250k rows) ran slower with 4 lanes a row (13 -> 20 us), its loads no
// longer coalesced.
int mg_group(int width, long rows) {
    const long cap = (long)num_sms() * 2048;
    int g = 1;
    while (g < 32 && (width + g - 1) / g > MG_GROUP_ENTRIES && rows * 2 * g <= cap) g *= 2;
    return g;
}

template <int G>
__device__ __forceinline__ float group_sum(float v) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
    return v;
}

// lane s's share of row i of A times x (entries s, s + G, ...)
template <int G>
__device__ __forceinline__ float row_part(const MgView &A, int i, const float *x, int s) {
    const int base = A.sl_ptr[i >> 5], wd = A.sl_w[i >> 5], lane = i & 31;
    float acc = 0.f;
#pragma unroll 4
    for (int k = s; k < wd; k += G) {
        const int pos = base + k * 32 + lane;
        acc += A.val[pos] * x[A.col[pos]];
    }
    return acc;
}

// the grid-stride walk over n groups of G lanes: f(valid, i, s) with i the
// group (row or aggregate), s the lane in the group, valid = i < n; whole warps
// advance together
template <int G, class F>
__device__ __forceinline__ void group_loop(int n, F f) {
    const long total = (long)n * G, stride = (long)gridDim.x * blockDim.x;
    for (long base = (long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < total; base += stride) {
        const long vt = base + (threadIdx.x & 31);
        const bool valid = vt < total;
        f(valid, valid ? (int)(vt / G) : 0, (int)(vt % G));
    }
}

// t = r - A (w r)   (pre-smoothing from zero and its residual)
template <int G>
__global__ void k_mg_down(MgView A, const float *w, const float *r, float *t, const int *done) {
    if (done && *done) return;
    group_loop<G>(A.n, [&](bool valid, int i, int s) {
        float acc = 0.f;
        if (valid) {
            const int base = A.sl_ptr[i >> 5], wd = A.sl_w[i >> 5], lane = i & 31;
            int k = s;
            if (G == 1) {  // one lane a row (the finest level): four entries' loads before their gathers
                for (; k + 4 <= wd; k += 4) {
                    const int p0 = base + k * 32 + lane;
                    const int j0 = A.col[p0], j1 = A.col[p0 + 32], j2 = A.col[p0 + 64], j3 = A.col[p0 + 96];
                    const float v0 = A.val[p0], v1 = A.val[p0 + 32], v2 = A.val[p0 + 64], v3 = A.val[p0 + 96];
                    const float y0 = w[j0] * r[j0], y1 = w[j1] * r[j1], y2 = w[j2] * r[j2], y3 = w[j3] * r[j3];
                    acc += v0 * y0;
                    acc += v1 * y1;
                    acc += v2 * y2;
                    acc += v3 * y3;
                }
            }
            for (; k < wd; k += G) {
                const int pos = base + k * 32 + lane;
                const int j = A.col[pos];
                acc += A.val[pos] * (w[j] * r[j]);
            }
        }
        acc = group_sum<G>(acc);
        if (valid && s == 0) t[i] = r[i] - acc;
    });
}

// rc[I] = sum of t over the rows of aggregate I (members in ascending order,
// lane s taking members s, s + G, ...)
template <int G>
__global__ void k_mg_restrict(int nc, const int *mem_ptr, const int *mem_idx, const float *t, float *rc,
                              const int *done) {
    if (done && *done) return;
    group_loop<G>(nc, [&](bool valid, int i, int s) {
        float acc = 0.f;
        if (valid) {
            const int k1 = mem_ptr[i + 1];
#pragma unroll 4
            for (int k = mem_ptr[i] + s; k < k1; k += G) acc += t[mem_idx[k]];
        }
        acc = group_sum<G>(acc);
        if (valid && s == 0) rc[i] = acc;
    });
}

// z_i = w_i r_i + gamma zc[agg(i)]; four rows a thread with 16-byte loads (the
// level's arrays are whole allocations; r may be the caller's fine residual,
// which is read four rows at a time only when 16-byte aligned)
__global__ void k_mg_prolong(int n, const float *w, const float *r, const int *agg, const float *zc, float gamma,
                             float *z, const int *done) {
    if (done && *done) return;
    const int T = gridDim.x * blockDim.x, t0 = blockIdx.x * blockDim.x + threadIdx.x;
    int n4 = 0;
    if ((reinterpret_cast<uintptr_t>(r) & 15) == 0 && (reinterpret_cast<uintptr_t>(z) & 15) == 0) {
        n4 = n >> 2;
        for (int j = t0; j < n4; j += T) {
            const float4 wj = reinterpret_cast<const float4 *>(w)[j], rj = reinterpret_cast<const float4 *>(r)[j];
            const int4 aj = reinterpret_cast<const int4 *>(agg)[j];
            float4 zj;
            zj.x = wj.x * rj.x + gamma * zc[aj.x];
            zj.y = wj.y * rj.y + gamma * zc[aj.y];
            zj.z = wj.z * rj.z + gamma * zc[aj.z];
            zj.w = wj.w * rj.w + gamma * zc[aj.w];
            reinterpret_cast<float4 *>(z)[j] = zj;
        }
    }
    for (int i = 4 * n4 + t0; i < n; i += T) z[i] = w[i] * r[i] + gamma * zc[agg[i]];
}

// zout = z + w (r - A z)
template <int G>
__global__ void k_mg_post(MgView A, const float *w, const float *r, const float *z, float *zout, const int *done) {
    if (done && *done) return;
    group_loop<G>(A.n, [&](bool valid, int i, int s) {
        float acc = valid ? row_part<G>(A, i, z, s) : 0.f;
        acc = group_sum<G>(acc);
        if (valid && s == 0) zout[i] = z[i] + w[i] * (r[i] - acc);
    });
}

// t = r - A z
__global__ void k_mg_resid(MgView A, const float *r, const float *z, float *t, const int *done) {
    if (done && *done) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x)
        t[i] = r[i] - row_times(A, i, z);
}

// e -= z (training pair of the post-smoother)
__global__ void k_mg_sub(int n, float *e, const float *z) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) e[i] -= z[i];
}

__global__ void k_mg_to_f64(int n, const float *a, double *b) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = a[i];
}

// z = w r (a coarsest level too large for the dense inverse: Jacobi sweeps)
__global__ void k_mg_scale(int n, const float *w, const float *r, float *z, const int *done) {
    if (done && *done) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) z[i] = w[i] * r[i];
}

// z = Minv r on the dense coarsest level (one CTA; a warp per row)
__global__ void __launch_bounds__(DENSE_THREADS) k_mg_dense_apply(int nd, const float *minv, const float *r,
                                                                   float *z, const int *done) {
    if (done && *done) return;
    __shared__ float rs[MG_DENSE_MAX];
    for (int j = threadIdx.x; j < nd; j += blockDim.x) rs[j] = r[j];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int i = warp; i < nd; i += nw) {
        float s = 0.f;
        for (int j = lane; j < nd; j += 32) s += minv[(size_t)i * nd + j] * rs[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL_MASK, s, o);
        if (lane == 0) z[i] = s;
    }
}

// Dense inverse of the coarsest level (FP32 Gauss-Jordan, no pivoting: the p'
// operators are weakly diagonally dominant), one CTA, matrix in shared memory.
// A level whose rows sum to zero (relative 1e-9) gets alpha 1 1^T first,
// alpha = mean(a_ii) / nd.  *err = 1 if a pivot vanishes.
__global__ void __launch_bounds__(DENSE_THREADS) k_mg_dense_inverse(int nd, const int *sl_ptr, const int *sl_w,
                                                                     const int *col, const double *val, float *minv,
                                                                     int *err) {
    extern __shared__ float M[];  // nd x nd
    __shared__ float fcol[MG_DENSE_MAX];
    __shared__ double s_rowsum, s_diag, s_dsum;
    __shared__ int s_bad;
    const int tid = threadIdx.x;
    for (int q = tid; q < nd * nd; q += blockDim.x) M[q] = 0.f;
    if (tid == 0) {
        s_rowsum = 0.0;
        s_diag = 0.0;
        s_dsum = 0.0;
        s_bad = 0;
    }
    __syncthreads();
    if (tid < 32) {
        // row sums and diagonal in FP64, one lane per row (lane-ordered max/sum)
        double rmax = 0.0, dmax = 0.0, dsum = 0.0;
        for (int i = tid; i < nd; i += 32) {
            const int base = sl_ptr[i >> 5], wd = sl_w[i >> 5], lane = i & 31;
            double rs = 0.0;
            for (int k = 0; k < wd; ++k) rs += val[base + k * 32 + lane];
            const double d = val[base + lane];
            rmax = fmax(rmax, fabs(rs));
            dmax = fmax(dmax, fabs(d));
            dsum += d;
        }
        for (int o = 16; o > 0; o >>= 1) {
            rmax = fmax(rmax, __shfl_xor_sync(FULL_MASK, rmax, o));
            dmax = fmax(dmax, __shfl_xor_sync(FULL_MASK, dmax, o));
            dsum += __shfl_xor_sync(FULL_MASK, dsum, o);
        }
        if (tid == 0) {
            s_rowsum = rmax;
            s_diag = dmax;
            s_dsum = dsum;
        }
    }
    __syncthreads();
    const bool singular = s_rowsum <= 1e-9 * s_diag;
    const float alpha = singular ? (float)(s_dsum / nd / nd) : 0.f;
    // scatter the rows (padding entries add 0 to their own diagonal)
    for (int i = tid; i < nd; i += blockDim.x) {
        const int base = sl_ptr[i >> 5], wd = sl_w[i >> 5], lane = i & 31;
        for (int k = 0; k < wd; ++k) {
            const int pos = base + k * 32 + lane;
            M[i * nd + col[pos]] += (float)val[pos];
        }
    }
    __syncthreads();
    if (singular)
        for (int q = tid; q < nd * nd; q += blockDim.x) M[q] += alpha;
    __syncthreads();
    for (int k = 0; k < nd; ++k) {
        const float p = M[k * nd + k];
        if (!(fabsf(p) > 0.f) || !isfinite(p)) {
            if (tid == 0) s_bad = 1;
            break;  // uniform: every thread read the same pivot
        }
        for (int i = tid; i < nd; i += blockDim.x) fcol[i] = i == k ? 0.f : M[i * nd + k];
        __syncthreads();
        const float inv = 1.0f / p;
        for (int j = tid; j < nd; j += blockDim.x) M[k * nd + j] = (j == k ? 1.0f : M[k * nd + j]) * inv;
        __syncthreads();
        for (int q = tid; q < nd * nd; q += blockDim.x) {
            const int i = q / nd, j = q - i * nd;
            if (i == k) continue;
            if (j == k) M[q] = -fcol[i] * M[k * nd + k];
            else M[q] -= fcol[i] * M[k * nd + j];
        }
        __syncthreads();
    }
    __syncthreads();
    if (s_bad) {
        if (tid == 0) atomicExch(err, 1);
        return;
    }
    for (int q = tid; q < nd * nd; q += blockDim.x) minv[q] = M[q];
}

MgView view_of(const SellDev &A, const float *val) { return MgView{A.n, A.sl_ptr.get(), A.sl_w.get(), A.col.get(), val}; }

// ---- the coarse levels in one persistent cooperative launch ------------------
// (option; measured slower than one launch per phase on the 2M-cell p' system:
// 135 us per cycle against about 110 us, because every phase is a chain of
// dependent L2 loads that a grid barrier does not shorten, and the finest
// level's phases run at one 1024-thread block per SM)
// Phases (each closed by a grid barrier): restriction of the finest level's t into
// level 1; for l = 1 .. L-2: t_l = r_l - A_l (w_l r_l), restriction into l+1; the
// coarsest solve; for l = L-2 .. 1: prolongation w_l r_l + gamma z_{l+1}[agg] into
// t_l, post-smoothing into z_l; finally the finest prolongation
// z0 = w0 r0 + gamma z_1[agg0].  Every row is computed by the same arithmetic in
// the same order as the one-kernel-per-phase path, so both give the same bits.
// Vectors written inside the launch are read with ld.global.cg (L2, not L1): t is
// gathered again after other blocks rewrote it.
constexpr int MGP_THREADS = 1024;

struct MgLvl {
    int n;
    const int *sl_ptr, *sl_w, *col;
    const float *val, *w;
    float *r, *z, *t;
    const int *agg, *mem_ptr, *mem_idx;  // to the next level
};

struct MgPersistArgs {
    int nlev;
    MgLvl lv[MG_MAX_LEVELS];
    const float *r0, *t0;
    float *z0;
    int nd;              // rows of the coarsest level if it is dense, else 0
    const float *minv;
    float gamma;
    GridBarrier *gb;
    int *err;
    const int *done;
};

__device__ __forceinline__ float lvl_row(const MgLvl &L, int i, const float *x) {
    const int base = L.sl_ptr[i >> 5], wd = L.sl_w[i >> 5], lane = i & 31;
    float s = 0.f;
    for (int k = 0; k < wd; ++k) {
        const int pos = base + k * 32 + lane;
        s += L.val[pos] * __ldcg(x + L.col[pos]);
    }
    return s;
}

__device__ __forceinline__ float lvl_row_wr(const MgLvl &L, int i) {
    const int base = L.sl_ptr[i >> 5], wd = L.sl_w[i >> 5], lane = i & 31;
    float s = 0.f;
    for (int k = 0; k < wd; ++k) {
        const int pos = base + k * 32 + lane;
        const int j = L.col[pos];
        s += L.val[pos] * (L.w[j] * __ldcg(L.r + j));
    }
    return s;
}

__global__ void __launch_bounds__(MGP_THREADS, 1) k_mg_coarse(MgPersistArgs a) {
    if (a.done && *a.done) return;  // written by earlier launches: every block sees the same value
    const int T = gridDim.x * blockDim.x, t0 = blockIdx.x * blockDim.x + threadIdx.x;
    const int L = a.nlev;
    // restriction of the finest level's t into level 1
    {
        const MgLvl &f = a.lv[0];
        const MgLvl &c = a.lv[1];
        for (int I = t0; I < c.n; I += T) {
            float s = 0.f;
            for (int k = f.mem_ptr[I]; k < f.mem_ptr[I + 1]; ++k) s += __ldcg(a.t0 + f.mem_idx[k]);
            c.r[I] = s;
        }
    }
    if (!grid_sync(a.gb, a.err)) return;
    for (int l = 1; l < L - 1; ++l) {
        const MgLvl &f = a.lv[l];
        for (int i = t0; i < f.n; i += T) f.t[i] = __ldcg(f.r + i) - lvl_row_wr(f, i);
        if (!grid_sync(a.gb, a.err)) return;
        const MgLvl &c = a.lv[l + 1];
        for (int I = t0; I < c.n; I += T) {
            float s = 0.f;
            for (int k = f.mem_ptr[I]; k < f.mem_ptr[I + 1]; ++k) s += __ldcg(f.t + f.mem_idx[k]);
            c.r[I] = s;
        }
        if (!grid_sync(a.gb, a.err)) return;
    }
    const MgLvl &c = a.lv[L - 1];
    if (a.nd > 0) {
        const int warp = t0 >> 5, lane = threadIdx.x & 31, nw = T >> 5;
        for (int i = warp; i < a.nd; i += nw) {
            float s = 0.f;
            for (int j = lane; j < a.nd; j += 32) s += a.minv[(size_t)i * a.nd + j] * __ldcg(c.r + j);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL_MASK, s, o);
            if (lane == 0) c.z[i] = s;
        }
        if (!grid_sync(a.gb, a.err)) return;
    } else {  // three Jacobi steps from zero
        for (int i = t0; i < c.n; i += T) c.z[i] = c.w[i] * __ldcg(c.r + i);
        if (!grid_sync(a.gb, a.err)) return;
        for (int i = t0; i < c.n; i += T) c.t[i] = __ldcg(c.z + i) + c.w[i] * (__ldcg(c.r + i) - lvl_row(c, i, c.z));
        if (!grid_sync(a.gb, a.err)) return;
        for (int i = t0; i < c.n; i += T) c.z[i] = __ldcg(c.t + i) + c.w[i] * (__ldcg(c.r + i) - lvl_row(c, i, c.t));
        if (!grid_sync(a.gb, a.err)) return;
    }
    for (int l = L - 2; l >= 1; --l) {
        const MgLvl &f = a.lv[l];
        const MgLvl &cc = a.lv[l + 1];
        for (int i = t0; i < f.n; i += T) f.t[i] = f.w[i] * __ldcg(f.r + i) + a.gamma * __ldcg(cc.z + f.agg[i]);
        if (!grid_sync(a.gb, a.err)) return;
        for (int i = t0; i < f.n; i += T) f.z[i] = __ldcg(f.t + i) + f.w[i] * (__ldcg(f.r + i) - lvl_row(f, i, f.t));
        if (!grid_sync(a.gb, a.err)) return;
    }
    {
        const MgLvl &f = a.lv[0];
        const MgLvl &c1 = a.lv[1];
        for (int i = t0; i < f.n; i += T) a.z0[i] = f.w[i] * a.r0[i] + a.gamma * __ldcg(c1.z + f.agg[i]);
    }
}

}  // namespace

void mg_to_f64(const float *a, double *b, int n, cudaStream_t st) {
    k_mg_to_f64<<<flat_blocks(n), MB, 0, st>>>(n, a, b);
    ++g_launches;
    SYSU_CUDA(cudaGetLastError());
}

void AggMultigrid::setup(const SellDev &A, const SellPattern &pat, const double *val64_dev, double theta,
                         cudaStream_t st) {
    A0_ = &A;
    std::vector<double> hv(pat.nnz);
    SYSU_CUDA(cudaMemcpyAsync(hv.data(), val64_dev, sizeof(double) * pat.nnz, cudaMemcpyDeviceToHost, st));
    SYSU_CUDA(cudaStreamSynchronize(st));
    sgn_ = hv.empty() || hv[0] >= 0.0 ? 1.0f : -1.0f;
    std::vector<MgHostLevel> H = mg_build_hierarchy(pat, hv, theta, MG_DENSE_MAX);
    lv_.clear();
    hpat_.assign(H.size(), SellPattern{});
    for (size_t l = 1; l < H.size(); ++l) hpat_[l] = H[l].pat;
    for (size_t l = 0; l < H.size(); ++l) {
        auto d = std::make_unique<MgLevelDev>();
        const MgHostLevel &h = H[l];
        d->n = h.n;
        if (l > 0) {
            d->A.upload(h.pat, st);
            d->val64.alloc(h.pat.nnz);
            d->val32.alloc(h.pat.nnz);
        }
        d->grow = mg_group(l > 0 ? d->A.wmax : A.wmax, h.n);
        d->w.alloc(h.n);
        d->r.alloc(h.n);
        d->z.alloc(h.n);
        d->t.alloc(h.n);
        if (!h.agg.empty()) {
            d->agg.upload(h.agg, st);
            d->mem_ptr.upload(h.mem_ptr, st);
            d->mem_idx.upload(h.mem_idx, st);
            int widest = 1;
            for (size_t I = 0; I + 1 < h.mem_ptr.size(); ++I) widest = std::max(widest, h.mem_ptr[I + 1] - h.mem_ptr[I]);
            d->gagg = mg_group(widest, (long)h.mem_ptr.size() - 1);
            d->gal_ptr.upload(h.gal_ptr, st);
            d->gal_src.upload(h.gal_src, st);
        }
        lv_.push_back(std::move(d));
    }
    nd_ = lv_.back()->n;
    if (lv_.size() > 1 && nd_ <= MG_DENSE_MAX) dinv_.alloc((size_t)nd_ * nd_);
    tmpz_.alloc(A.n);
    tmpt_.alloc(A.n);
    err_.alloc(1);
    err_.zero(st);
    gb_.alloc(1);
    gb_.zero(st);  // the barrier's counter returns to 0 or 2^31 after every completed launch
    if (pblocks_ == 0) {
        int per_sm = 0;
        SYSU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mg_coarse, MGP_THREADS, 0));
        pblocks_ = std::max(1, std::min(per_sm, 1)) * num_sms();
    }
    static bool attr = false;
    if (!attr) {
        SYSU_CUDA(cudaFuncSetAttribute(k_mg_dense_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       MG_DENSE_MAX * MG_DENSE_MAX * (int)sizeof(float)));
        attr = true;
    }
    SYSU_CUDA(cudaStreamSynchronize(st));  // the host hierarchy goes out of scope
}

void AggMultigrid::refresh(const double *val64_dev, const float *val32_dev, cudaStream_t st) {
    if (!ready()) throw CaseError{"multigrid: no hierarchy"};
    gb_.zero(st);  // a barrier that timed out in an earlier solve starts clean
    val0_32_ = val32_dev;
    const double *fval = val64_dev;
    for (size_t l = 0; l < lv_.size(); ++l) {
        MgLevelDev &d = *lv_[l];
        const SellDev &A = l == 0 ? *A0_ : d.A;
        const double *v = l == 0 ? val64_dev : d.val64.get();
        if (l > 0) {
            const MgLevelDev &f = *lv_[l - 1];
            k_mg_galerkin<<<flat_blocks(A.nnz), MB, 0, st>>>(A.nnz, f.gal_ptr.get(), f.gal_src.get(), fval,
                                                              d.val64.get(), d.val32.get());
            ++g_launches;
        }
        k_mg_weights<<<flat_blocks(A.n), MB, 0, st>>>(A.n, A.sl_ptr.get(), v, omega, d.w.get());
        ++g_launches;
        fval = v;
    }
    if (lv_.size() > 1 && nd_ <= MG_DENSE_MAX) {
        const MgLevelDev &c = *lv_.back();
        k_mg_dense_inverse<<<1, DENSE_THREADS, (size_t)nd_ * nd_ * sizeof(float), st>>>(
            nd_, c.A.sl_ptr.get(), c.A.sl_w.get(), c.A.col.get(), c.val64.get(), dinv_.get(), err_.get());
        ++g_launches;
    }
    SYSU_CUDA(cudaGetLastError());
}

// level l (l < coarsest): t = r - A (w r) on level l, restricted into level l+1's r
void AggMultigrid::enqueue_down(int l, const float *r, const int *done, cudaStream_t st) {
    MgLevelDev &d = *lv_[l];
    MgLevelDev &c = *lv_[l + 1];
    const SellDev &A = l == 0 ? *A0_ : d.A;
    const float *v32 = l == 0 ? val0_32_ : d.val32.get();
    with_group(d.grow, [&](auto G) {
        k_mg_down<G.value><<<flat_blocks((long)A.n * G.value), MB, 0, st>>>(view_of(A, v32), d.w.get(), r, d.t.get(),
                                                                             done);
    });
    with_group(d.gagg, [&](auto G) {
        k_mg_restrict<G.value><<<flat_blocks((long)c.n * G.value), MB, 0, st>>>(c.n, d.mem_ptr.get(), d.mem_idx.get(),
                                                                                 d.t.get(), c.r.get(), done);
    });
    g_launches += 2;
}

// level l >= 1 (not the coarsest): prolong the coarse correction and post-smooth
// into zout (level l's z holds the prolonged value)
void AggMultigrid::enqueue_up(int l, float *zout, const int *done, cudaStream_t st) {
    MgLevelDev &d = *lv_[l];
    MgLevelDev &c = *lv_[l + 1];
    const SellDev &A = d.A;
    k_mg_prolong<<<flat_blocks(d.n), MB, 0, st>>>(d.n, d.w.get(), d.r.get(), d.agg.get(), c.z.get(), (float)gamma,
                                                   d.t.get(), done);
    ++g_launches;
    if (post_hook && l == post_level) {
        post_hook(l, d.r.get(), d.t.get(), zout, done, st);
        return;
    }
    with_group(d.grow, [&](auto G) {
        k_mg_post<G.value><<<flat_blocks((long)d.n * G.value), MB, 0, st>>>(view_of(A, d.val32.get()), d.w.get(),
                                                                             d.r.get(), d.t.get(), zout, done);
    });
    ++g_launches;
}

void AggMultigrid::level_rhs(int l, const float *r0, float *out, cudaStream_t st) {
    if (l < 1 || l >= levels()) throw CaseError{"multigrid: no such coarse level"};
    enqueue_down(0, r0, nullptr, st);
    for (int k = 1; k < l; ++k) enqueue_down(k, lv_[k]->r.get(), nullptr, st);
    SYSU_CUDA(cudaMemcpyAsync(out, lv_[l]->r.get(), sizeof(float) * lv_[l]->n, cudaMemcpyDeviceToDevice, st));
}

// Levels 1.. of the cycle for the residual r at level 0; leaves the prolonged
// fine correction (w r + gamma P z_1) in z.
void AggMultigrid::enqueue_cycle_to_fine(const float *r, float *z, const int *done, cudaStream_t st) {
    const int L = (int)lv_.size();
    MgLevelDev &f = *lv_[0];
    if (L == 1) {  // no coarse level: Jacobi
        k_mg_scale<<<flat_blocks(f.n), MB, 0, st>>>(f.n, f.w.get(), r, z, done);
        ++g_launches;
        return;
    }
    if (persistent && !(post_hook && post_level >= 1)) {
        MgLevelDev &d0 = *lv_[0];
        with_group(d0.grow, [&](auto G) {
            k_mg_down<G.value><<<flat_blocks((long)f.n * G.value), MB, 0, st>>>(view_of(*A0_, val0_32_), d0.w.get(),
                                                                                 r, d0.t.get(), done);
        });
        ++g_launches;
        MgPersistArgs pa{};
        pa.nlev = L;
        for (int l = 0; l < L; ++l) {
            MgLevelDev &d = *lv_[l];
            const SellDev &A = l == 0 ? *A0_ : d.A;
            pa.lv[l] = MgLvl{d.n, A.sl_ptr.get(), A.sl_w.get(), A.col.get(), l == 0 ? val0_32_ : d.val32.get(),
                             d.w.get(), d.r.get(), d.z.get(), d.t.get(), d.agg.get(), d.mem_ptr.get(),
                             d.mem_idx.get()};
        }
        pa.r0 = r;
        pa.t0 = d0.t.get();
        pa.z0 = z;
        pa.nd = nd_ <= MG_DENSE_MAX ? nd_ : 0;
        pa.minv = dinv_.get();
        pa.gamma = (float)gamma;
        pa.gb = gb_.get();
        pa.err = err_.get();
        pa.done = done;
        void *args[] = {&pa};
        SYSU_CUDA(cudaLaunchCooperativeKernel((const void *)k_mg_coarse, dim3(pblocks_), dim3(MGP_THREADS), args, 0,
                                              st));
        ++g_launches;
        return;
    }
    enqueue_down(0, r, done, st);
    for (int l = 1; l < L - 1; ++l) enqueue_down(l, lv_[l]->r.get(), done, st);
    MgLevelDev &c = *lv_[L - 1];
    if (nd_ <= MG_DENSE_MAX) {
        k_mg_dense_apply<<<1, DENSE_THREADS, 0, st>>>(nd_, dinv_.get(), c.r.get(), c.z.get(), done);
        ++g_launches;
    } else {  // coarsest too large for the dense inverse: three Jacobi steps from zero
        k_mg_scale<<<flat_blocks(c.n), MB, 0, st>>>(c.n, c.w.get(), c.r.get(), c.z.get(), done);
        with_group(c.grow, [&](auto G) {
            const int gb = flat_blocks((long)c.n * G.value);
            k_mg_post<G.value><<<gb, MB, 0, st>>>(view_of(c.A, c.val32.get()), c.w.get(), c.r.get(), c.z.get(),
                                                  c.t.get(), done);
            k_mg_post<G.value><<<gb, MB, 0, st>>>(view_of(c.A, c.val32.get()), c.w.get(), c.r.get(), c.t.get(),
                                                  c.z.get(), done);
        });
        g_launches += 3;
    }
    for (int l = L - 2; l >= 1; --l) enqueue_up(l, lv_[l]->z.get(), done, st);
    MgLevelDev &c1 = *lv_[1];
    k_mg_prolong<<<flat_blocks(f.n), MB, 0, st>>>(f.n, f.w.get(), r, f.agg.get(), c1.z.get(), (float)gamma, z, done);
    ++g_launches;
}

void AggMultigrid::apply_to_fine(const float *r, float *z2, const int *fs_done, cudaStream_t st) {
    enqueue_cycle_to_fine(r, z2, fs_done, st);
    SYSU_CUDA(cudaGetLastError());
}

void AggMultigrid::apply_fixed(const float *r, float *z2, float *t, const int *fs_done, cudaStream_t st) {
    enqueue_cycle_to_fine(r, z2, fs_done, st);
    k_mg_resid<<<flat_blocks(A0_->n), MB, 0, st>>>(view_of(*A0_, val0_32_), r, z2, t, fs_done);
    ++g_launches;
    SYSU_CUDA(cudaGetLastError());
}

void AggMultigrid::apply(const float *r, float *z, const int *fs_done, cudaStream_t st) {
    enqueue_cycle_to_fine(r, tmpz_.get(), fs_done, st);
    with_group(lv_[0]->grow, [&](auto G) {
        k_mg_post<G.value><<<flat_blocks((long)A0_->n * G.value), MB, 0, st>>>(
            view_of(*A0_, val0_32_), lv_[0]->w.get(), r, tmpz_.get(), z, fs_done);
    });
    ++g_launches;
    SYSU_CUDA(cudaGetLastError());
}

void AggMultigrid::smoother_pair(float *r, float *e, cudaStream_t st) {
    apply_fixed(r, tmpz_.get(), tmpt_.get(), nullptr, st);
    const int n = A0_->n;
    SYSU_CUDA(cudaMemcpyAsync(r, tmpt_.get(), sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
    k_mg_sub<<<flat_blocks(n), MB, 0, st>>>(n, e, tmpz_.get());
    ++g_launches;
    SYSU_CUDA(cudaGetLastError());
}

int AggMultigrid::err_flag(cudaStream_t st) {
    int e = 0;
    if (err_.size()) {
        err_.download(&e, 1, st);
        SYSU_CUDA(cudaStreamSynchronize(st));
    }
    return e;
}

}  // namespace sysu
