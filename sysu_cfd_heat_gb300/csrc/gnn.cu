// Learned preconditioner (see gnn.hpp): network forward / backward on the
// tensor cores, Adam, and flexible CG with fallback to Jacobi.
//
// Network kernels work on tiles of 128 rows, one thread per row, four warps
// per CTA; warp w of a tile owns SELL slice 4t + w, so matrix loads are the
// coalesced SELL-32 pattern, and thread t's row is TMEM lane t of the MMA
// accumulator.  A thread gathers its row's neighbours (FP32 accumulation of
// BF16 activations), writes its operand row to shared memory, one elected
// thread issues the MMAs, the commit arrives on an mbarrier (bounded wait),
// and every thread reads its own accumulator row back for the epilogue.
//
// Reductions (scale, loss, the flexible-CG scalars) are per-block partial
// sums that the last block to finish adds up in block order, so results are
// run-to-run deterministic; so are the parameter gradients (per-CTA records,
// summed in CTA order by the Adam kernel).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <random>

#include "gnn.hpp"
#include "graph_loop.hpp"
#include "krylov_dev.cuh"
#include "umma.cuh"

namespace sysu {
namespace {

constexpr int GT = 128;  // rows per tile = threads per CTA of the network kernels
constexpr int FB = 256;  // threads per block of the flat kernels
constexpr uint32_t IDESC_F = umma::idesc_bf16_f32(128, 32);   // forward: 128 x 32, K = 64
constexpr uint32_t IDESC_B1 = umma::idesc_bf16_f32(128, 64);  // backward, input gradient: 128 x 64, K = 32
constexpr uint32_t IDESC_B2 = umma::idesc_bf16_f32(128, 32);  // backward, weight gradient: 128 x 32, K = 128

constexpr int FWD_SMEM = 16384 + 4096 + 1024;
constexpr int BWD_SMEM = 8192 + 4096 + 32768 + 8192 + 2048 + 1024;
// The backward kernel holds 128 TMEM columns; requesting this much shared
// memory caps it at three resident CTAs per SM (384 of 512 columns).
constexpr int BWD_SMEM_REQ = 64 * 1024;
static_assert(BWD_SMEM <= BWD_SMEM_REQ, "backward shared-memory layout");

struct GView {
    int n;
    const int *sl_ptr, *sl_w, *col;
    const float *val;
    const float *dinv;
};

__device__ __forceinline__ float bf_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf_hi(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }
__device__ __forceinline__ uint32_t bf_pack(float a, float b) {
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(a)) |
           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(b)) << 16);
}
__device__ __forceinline__ float bf_round(float a) { return __bfloat162float(__float2bfloat16_rn(a)); }

// The flexible-CG kernels accumulate each thread's rows (a handful) in FP32 and
// hand those partials to grid_sums_f (FP32 warp sums, FP64 block and grid
// sums): per-row FP64 arithmetic and conversions run on GB300's FP64 pipe (1/64
// of the FP32 rate) and took half of these kernels' time.  Convergence is
// decided on the FP64 residual b - A x.

// ---------------------------------------------------------------- forward --

struct NetArgs {
    GView g;
    const float *r;
    const float *inv_s_p, *s_p;
    const uint16_t *wbf;  // this layer's BF16 weights (Wt[32][64] at +0)
    const float *prm;
    int layer;
    const uint16_t *hin;
    uint16_t *hout, *mout;
    uint32_t *mask;
    float *aw;
    float *z;
    const float *zbase;  // multigrid form: z = zbase + network output
    float skip;          // weight of the Jacobi term u in the decoder (1 as a whole preconditioner)
    const float *qprev;
    FcgState *fs;
    double *part;
    int *err;
};

template <bool L1, bool TRAIN, bool DEC>
__global__ void __launch_bounds__(GT) k_gnn_fwd(NetArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA = smem;          // X tile: 128 rows x 64 (K-adjacent, K = 64)
    uint8_t *sB = smem + 16384;  // Wt: 32 outputs x 64 inputs
    float *sprm = reinterpret_cast<float *>(smem + 20480);  // bias, e, c, w_d, b_d
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 20480 + 136 * 4);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (a.fs && (a.fs->done || !a.fs->use_gnn)) return;

    for (int q = tid; q < 32 * 8; q += GT) {
        int o = q >> 3, c = q & 7;
        uint4 w = *reinterpret_cast<const uint4 *>(a.wbf + o * 64 + c * 8);
        *reinterpret_cast<uint4 *>(sB + ((o >> 3) * 8 + c) * 128 + (o & 7) * 16) = w;
    }
    const float *lp = a.prm + GNN_OFF_LAYER + a.layer * GNN_LAYER_STRIDE;
    if (tid < 32) {
        sprm[tid] = lp[2048 + tid];
        sprm[32 + tid] = a.prm[GNN_OFF_ENC + tid];
        sprm[64 + tid] = a.prm[GNN_OFF_ENC + 32 + tid];
        sprm[96 + tid] = a.prm[GNN_OFF_DEC + tid];
        if (tid == 0) sprm[128] = a.prm[GNN_OFF_DEC + 32];
    }
    if (warp == 0) umma::tmem_alloc(tslot, 32);
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_init_fence();
    }
    umma::fence_smem_to_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tslot;
    const float inv_s = *a.inv_s_p, s = *a.s_p;
    const int n = a.g.n, ntiles = (n + GT - 1) / GT;
    const uint32_t a0 = umma::smem_addr(sA), b0 = umma::smem_addr(sB);
    float zq = 0.f;
    int it = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
        const int row = t * GT + tid;
        const bool valid = row < n;
        float mv[32];
        uint32_t hs[16];
#pragma unroll
        for (int c = 0; c < 32; ++c) mv[c] = 0.f;
#pragma unroll
        for (int c = 0; c < 16; ++c) hs[c] = 0u;
        float ui = 0.f, di = 0.f;
        if (valid) {
            const int sl = row >> 5;
            const int base = a.g.sl_ptr[sl], w = a.g.sl_w[sl];
            di = a.g.dinv[row];
            if (L1) {
                float su = 0.f, sw = 0.f;
                for (int k = 1; k < w; ++k) {
                    int pos = base + k * 32 + lane;
                    int j = a.g.col[pos];
                    float v = a.g.val[pos];
                    su += v * (a.g.dinv[j] * a.r[j]);
                    sw += v;
                }
                float ai = di * su * inv_s, wi = di * sw;
                ui = di * a.r[row] * inv_s;
#pragma unroll
                for (int c = 0; c < 32; c += 2) {
                    float e0 = sprm[32 + c], e1 = sprm[33 + c], c0 = sprm[64 + c], c1 = sprm[65 + c];
                    hs[c >> 1] = bf_pack(ui * e0 + c0, ui * e1 + c1);
                    mv[c] = ai * e0 + wi * c0;
                    mv[c + 1] = ai * e1 + wi * c1;
                }
                if (TRAIN) {
                    a.aw[2 * (size_t)row] = ai;
                    a.aw[2 * (size_t)row + 1] = wi;
                }
            } else {
                {
                    const uint4 *hp = reinterpret_cast<const uint4 *>(a.hin + (size_t)row * 32);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        uint4 h4 = __ldg(hp + q);
                        hs[4 * q] = h4.x;
                        hs[4 * q + 1] = h4.y;
                        hs[4 * q + 2] = h4.z;
                        hs[4 * q + 3] = h4.w;
                    }
                }
                // two neighbours per step: eight 16-byte loads in flight per thread
                for (int k = 1; k < w; k += 2) {
                    const int pos = base + k * 32 + lane;
                    const bool two = k + 1 < w;
                    const int j0 = a.g.col[pos];
                    const float v0 = a.g.val[pos];
                    const int j1 = two ? a.g.col[pos + 32] : j0;
                    const float v1 = two ? a.g.val[pos + 32] : 0.f;
                    const uint4 *p0 = reinterpret_cast<const uint4 *>(a.hin + (size_t)j0 * 32);
                    const uint4 *p1 = reinterpret_cast<const uint4 *>(a.hin + (size_t)j1 * 32);
                    uint4 x[4], y[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        x[q] = __ldg(p0 + q);
                        y[q] = __ldg(p1 + q);
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        uint32_t xw[4] = {x[q].x, x[q].y, x[q].z, x[q].w};
                        uint32_t yw[4] = {y[q].x, y[q].y, y[q].z, y[q].w};
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            mv[8 * q + 2 * e] += v0 * bf_lo(xw[e]) + v1 * bf_lo(yw[e]);
                            mv[8 * q + 2 * e + 1] += v0 * bf_hi(xw[e]) + v1 * bf_hi(yw[e]);
                        }
                    }
                }
#pragma unroll
                for (int c = 0; c < 32; ++c) mv[c] *= di;
            }
        }
        uint32_t mp[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) mp[c] = bf_pack(mv[2 * c], mv[2 * c + 1]);
        uint8_t *rowp = sA + (tid >> 3) * 8 * 128 + (tid & 7) * 16;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            *reinterpret_cast<uint4 *>(rowp + q * 128) = make_uint4(hs[4 * q], hs[4 * q + 1], hs[4 * q + 2], hs[4 * q + 3]);
            *reinterpret_cast<uint4 *>(rowp + (4 + q) * 128) =
                make_uint4(mp[4 * q], mp[4 * q + 1], mp[4 * q + 2], mp[4 * q + 3]);
        }
        if (TRAIN && !L1 && valid) {
            uint4 *mo = reinterpret_cast<uint4 *>(a.mout + (size_t)row * 32);
#pragma unroll
            for (int q = 0; q < 4; ++q) mo[q] = make_uint4(mp[4 * q], mp[4 * q + 1], mp[4 * q + 2], mp[4 * q + 3]);
        }
        umma::fence_smem_to_async();
        umma::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            umma::fence_after_sync();
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
                umma::mma_bf16(tmem, umma::smem_desc(a0 + kk * 256, 128, 1024), umma::smem_desc(b0 + kk * 256, 128, 1024),
                               IDESC_F, kk > 0);
            umma::commit(bar);
        }
        __syncwarp();
        bool fail = !mbar_wait(bar, it & 1);
        if (__syncthreads_or(fail)) {
            if (tid == 0) atomicExch(a.err, (int)DEV_BARRIER_TIMEOUT);
            break;
        }
        umma::fence_after_sync();
        float pre[32];
        umma::ld32(tmem + ((uint32_t)(warp * 32) << 16), pre);
        if (valid) {
            uint32_t ho[16];
            uint32_t mbits = 0;
#pragma unroll
            for (int c = 0; c < 32; c += 2) {
                float p0 = pre[c] + sprm[c], p1 = pre[c + 1] + sprm[c + 1];
                float h0 = bf_lo(hs[c >> 1]) + fmaxf(p0, 0.f);
                float h1 = bf_hi(hs[c >> 1]) + fmaxf(p1, 0.f);
                mbits |= (p0 > 0.f ? 1u : 0u) << c;
                mbits |= (p1 > 0.f ? 1u : 0u) << (c + 1);
                ho[c >> 1] = bf_pack(h0, h1);
            }
            if (!DEC || TRAIN) {
                uint4 *hp = reinterpret_cast<uint4 *>(a.hout + (size_t)row * 32);
#pragma unroll
                for (int q = 0; q < 4; ++q) hp[q] = make_uint4(ho[4 * q], ho[4 * q + 1], ho[4 * q + 2], ho[4 * q + 3]);
            }
            if (TRAIN) a.mask[row] = mbits;
            if (DEC) {
                float acc = sprm[128];
#pragma unroll
                for (int c = 0; c < 32; c += 2) acc += sprm[96 + c] * bf_lo(ho[c >> 1]) + sprm[97 + c] * bf_hi(ho[c >> 1]);
                float u = di * a.r[row] * inv_s;
                float zi = s * (a.skip * u + acc);
                if (a.zbase) zi += a.zbase[row];
                a.z[row] = zi;
                if (a.qprev) zq = fmaf(zi, a.qprev[row], zq);
            }
        }
    }
    if (DEC && a.fs) {
        const float fv[1] = {zq};
        double v[1];
        if (grid_sums_f<1>(fv, v, a.part, &a.fs->cnt[0])) a.fs->zq = v[0];
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_free(tmem, 32);
}

// --------------------------------------------------------------- backward --

struct BwdArgs {
    GView g;
    float sgn;
    int kind;
    const float *r;
    const float *inv_s_p, *s_p;
    const uint16_t *wbf;
    const float *prm;
    int layer;
    const uint16_t *hprev, *mcur;
    const uint32_t *mask;
    const float *aw;
    const uint16_t *h4;
    const float *y;
    const GnnScalars *sc;
    const float *dIn, *gIn;
    float *dOut, *gOut;
    float *rec;
    int *err;
};

template <bool TOP, bool L1>
__global__ void __launch_bounds__(GT) k_gnn_bwd(BwdArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA1 = smem;                  // dpre: 128 rows x 32 (K = 32)
    uint8_t *sB1 = smem + 8192;           // W: 64 inputs x 32 outputs (K = 32)
    uint8_t *sA2 = smem + 12288;          // [X^T; 1; 0]: 128 x 128 rows (K = 128)
    uint8_t *sB2 = smem + 45056;          // dpre^T: 32 outputs x 128 rows (K = 128)
    float *sprm = reinterpret_cast<float *>(smem + 53248);  // e, c, w_d
    float *sred = sprm + 96;                                 // [4 warps][64]
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 53248 + 2048);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    for (int q = tid; q < 64 * 4; q += GT) {
        int i = q >> 2, c = q & 3;
        uint4 w = *reinterpret_cast<const uint4 *>(a.wbf + 2048 + i * 32 + c * 8);
        *reinterpret_cast<uint4 *>(sB1 + ((i >> 3) * 4 + c) * 128 + (i & 7) * 16) = w;
    }
    for (int q = tid; q < 32768 / 16; q += GT) reinterpret_cast<uint4 *>(sA2)[q] = make_uint4(0, 0, 0, 0);
    if (tid < 32) {
        sprm[tid] = a.prm[GNN_OFF_ENC + tid];
        sprm[32 + tid] = a.prm[GNN_OFF_ENC + 32 + tid];
        sprm[64 + tid] = a.prm[GNN_OFF_DEC + tid];
    }
    if (warp == 0) umma::tmem_alloc(tslot, 128);
    if (tid == 0) {
        mbar_init(bar, 1);
        mbar_init_fence();
    }
    umma::fence_smem_to_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tslot;
    const float inv_s = *a.inv_s_p, s = *a.s_p;
    const int n = a.g.n, ntiles = (n + GT - 1) / GT;
    const uint32_t a1 = umma::smem_addr(sA1), b1 = umma::smem_addr(sB1);
    const uint32_t a2 = umma::smem_addr(sA2), b2 = umma::smem_addr(sB2);
    const double den = TOP ? a.sc->loss_den : 1.0;
    const float gscale = TOP ? (float)(2.0 / (den > 0.0 ? den : 1.0)) : 0.f;
    // per-CTA sums kept by lane c % 32 of each warp: [0] value c, [1] value c + 32
    float acc0 = 0.f, acc1 = 0.f, acc2 = 0.f;
    int it = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
        const int row = t * GT + tid;
        const bool valid = row < n;
        float delta[32];
        float xh[32], xm[32];
        float ui = 0.f, ai = 0.f, wi = 0.f, di = 0.f, gs = 0.f;
#pragma unroll
        for (int c = 0; c < 32; ++c) {
            delta[c] = 0.f;
            xh[c] = 0.f;
            xm[c] = 0.f;
        }
        uint32_t mbits = 0;
        if (valid) {
            const int sl = row >> 5;
            const int base = a.g.sl_ptr[sl], w = a.g.sl_w[sl];
            di = a.g.dinv[row];
            mbits = a.mask[row];
            if (TOP) {
                float gz;
                if (a.kind == 0) {
                    gz = gscale * a.y[row];
                } else {
                    float sy = 0.f;
                    for (int k = 0; k < w; ++k) {
                        int pos = base + k * 32 + lane;
                        sy += a.g.val[pos] * a.y[a.g.col[pos]];
                    }
                    gz = gscale * a.sgn * sy;
                }
                gs = gz * s;
#pragma unroll
                for (int c = 0; c < 32; ++c) delta[c] = gs * sprm[64 + c];
            } else {
                const float4 *dp = reinterpret_cast<const float4 *>(a.dIn + (size_t)row * 32);
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    float4 d4 = dp[q];
                    delta[4 * q] = d4.x;
                    delta[4 * q + 1] = d4.y;
                    delta[4 * q + 2] = d4.z;
                    delta[4 * q + 3] = d4.w;
                }
                for (int k = 1; k < w; ++k) {
                    int pos = base + k * 32 + lane;
                    int j = a.g.col[pos];
                    float v = a.g.val[pos];
                    const float4 *gp = reinterpret_cast<const float4 *>(a.gIn + (size_t)j * 32);
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        float4 g4 = gp[q];
                        delta[4 * q] += v * g4.x;
                        delta[4 * q + 1] += v * g4.y;
                        delta[4 * q + 2] += v * g4.z;
                        delta[4 * q + 3] += v * g4.w;
                    }
                }
            }
            if (L1) {
                ai = a.aw[2 * (size_t)row];
                wi = a.aw[2 * (size_t)row + 1];
                ui = di * a.r[row] * inv_s;
#pragma unroll
                for (int c = 0; c < 32; ++c) {
                    xh[c] = bf_round(ui * sprm[c] + sprm[32 + c]);
                    xm[c] = bf_round(ai * sprm[c] + wi * sprm[32 + c]);
                }
            } else {
                const uint4 *hp = reinterpret_cast<const uint4 *>(a.hprev + (size_t)row * 32);
                const uint4 *mp = reinterpret_cast<const uint4 *>(a.mcur + (size_t)row * 32);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    uint4 h4 = hp[q], m4 = mp[q];
                    uint32_t hw[4] = {h4.x, h4.y, h4.z, h4.w}, mw[4] = {m4.x, m4.y, m4.z, m4.w};
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        xh[8 * q + 2 * e] = bf_lo(hw[e]);
                        xh[8 * q + 2 * e + 1] = bf_hi(hw[e]);
                        xm[8 * q + 2 * e] = bf_lo(mw[e]);
                        xm[8 * q + 2 * e + 1] = bf_hi(mw[e]);
                    }
                }
            }
        }
        // decoder gradient (w_d, b_d) from the stored h4
        if (TOP) {
            float h4v[32];
#pragma unroll
            for (int c = 0; c < 32; ++c) h4v[c] = 0.f;
            if (valid) {
                const uint4 *hp = reinterpret_cast<const uint4 *>(a.h4 + (size_t)row * 32);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    uint4 h4 = hp[q];
                    uint32_t hw[4] = {h4.x, h4.y, h4.z, h4.w};
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        h4v[8 * q + 2 * e] = bf_lo(hw[e]);
                        h4v[8 * q + 2 * e + 1] = bf_hi(hw[e]);
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                float v = gs * h4v[c];
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
                if (lane == c) acc0 += v;
            }
            float v = gs;
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
            if (lane == 0) acc2 += v;
        }
        // operand tiles
        uint32_t dp16[16];
#pragma unroll
        for (int c = 0; c < 32; c += 2) {
            float d0 = (mbits >> c) & 1u ? delta[c] : 0.f;
            float d1 = (mbits >> (c + 1)) & 1u ? delta[c + 1] : 0.f;
            dp16[c >> 1] = bf_pack(d0, d1);
        }
        {
            uint8_t *rowp = sA1 + (tid >> 3) * 4 * 128 + (tid & 7) * 16;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                *reinterpret_cast<uint4 *>(rowp + q * 128) =
                    make_uint4(dp16[4 * q], dp16[4 * q + 1], dp16[4 * q + 2], dp16[4 * q + 3]);
        }
        {
            // transposed tiles: element (feature, row = tid)
            const uint32_t colo = ((tid >> 3) << 7) + ((tid & 7) << 1);
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                uint16_t v = (uint16_t)((c & 1) ? (dp16[c >> 1] >> 16) : (dp16[c >> 1] & 0xFFFFu));
                *reinterpret_cast<uint16_t *>(sB2 + ((c >> 3) * 16) * 128 + ((c & 7) << 4) + colo) = v;
            }
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                *reinterpret_cast<uint16_t *>(sA2 + ((c >> 3) * 16) * 128 + ((c & 7) << 4) + colo) =
                    __bfloat16_as_ushort(__float2bfloat16_rn(xh[c]));
                *reinterpret_cast<uint16_t *>(sA2 + (((c + 32) >> 3) * 16) * 128 + ((c & 7) << 4) + colo) =
                    __bfloat16_as_ushort(__float2bfloat16_rn(xm[c]));
            }
            *reinterpret_cast<uint16_t *>(sA2 + (8 * 16) * 128 + colo) = valid ? (uint16_t)0x3F80u : (uint16_t)0u;
        }
        umma::fence_smem_to_async();
        umma::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            umma::fence_after_sync();
#pragma unroll
            for (int kk = 0; kk < 2; ++kk)
                umma::mma_bf16(tmem, umma::smem_desc(a1 + kk * 256, 128, 512), umma::smem_desc(b1 + kk * 256, 128, 512),
                               IDESC_B1, kk > 0);
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
                umma::mma_bf16(tmem + 64, umma::smem_desc(a2 + kk * 256, 128, 2048),
                               umma::smem_desc(b2 + kk * 256, 128, 2048), IDESC_B2, it > 0 || kk > 0);
            umma::commit(bar);
        }
        __syncwarp();
        bool fail = !mbar_wait(bar, it & 1);
        if (__syncthreads_or(fail)) {
            if (tid == 0) atomicExch(a.err, (int)DEV_BARRIER_TIMEOUT);
            break;
        }
        umma::fence_after_sync();
        float dxh[32], dxm[32];
        const uint32_t lb = (uint32_t)(warp * 32) << 16;
        umma::ld32(tmem + lb, dxh);
        umma::ld32(tmem + lb + 32, dxm);
        if (!L1) {
            if (valid) {
                float4 *dp = reinterpret_cast<float4 *>(a.dOut + (size_t)row * 32);
                float4 *gp = reinterpret_cast<float4 *>(a.gOut + (size_t)row * 32);
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    dp[q] = make_float4(delta[4 * q] + dxh[4 * q], delta[4 * q + 1] + dxh[4 * q + 1],
                                        delta[4 * q + 2] + dxh[4 * q + 2], delta[4 * q + 3] + dxh[4 * q + 3]);
                    gp[q] = make_float4(di * dxm[4 * q], di * dxm[4 * q + 1], di * dxm[4 * q + 2], di * dxm[4 * q + 3]);
                }
            }
        } else {
            // encoder: h0 = u e + c, m1 = a e + w c
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                float dh0 = valid ? delta[c] + dxh[c] : 0.f;
                float dm1 = valid ? dxm[c] : 0.f;
                float ve = ui * dh0 + ai * dm1, vc = dh0 + wi * dm1;
                for (int o = 16; o > 0; o >>= 1) {
                    ve += __shfl_xor_sync(FULL_MASK, ve, o);
                    vc += __shfl_xor_sync(FULL_MASK, vc, o);
                }
                if (lane == c) {
                    acc0 += ve;
                    acc1 += vc;
                }
            }
        }
        umma::fence_before_sync();
    }
    // weight and bias gradients of this CTA from the accumulator (rows 0..64)
    float *rec = a.rec + (size_t)blockIdx.x * GNN_NPARAM_PAD;
    float *lrec = rec + GNN_OFF_LAYER + a.layer * GNN_LAYER_STRIDE;
    __syncthreads();
    umma::fence_after_sync();
    if (warp < 3) {
        float dw[32];
        umma::ld32(tmem + ((uint32_t)(warp * 32) << 16) + 64, dw);
        const int m = warp * 32 + lane;
        if (m < 64) {
#pragma unroll
            for (int o = 0; o < 32; ++o) lrec[m * 32 + o] = it > 0 ? dw[o] : 0.f;
        } else if (m == 64) {
#pragma unroll
            for (int o = 0; o < 32; ++o) lrec[2048 + o] = it > 0 ? dw[o] : 0.f;
        }
    }
    if (TOP || L1) {
        sred[warp * 64 + lane] = acc0;
        sred[warp * 64 + 32 + lane] = TOP ? (lane == 0 ? acc2 : 0.f) : acc1;
        __syncthreads();
        if (tid < 64) {
            float v = sred[tid] + sred[64 + tid] + sred[128 + tid] + sred[192 + tid];
            if (TOP) {
                if (tid < 32) rec[GNN_OFF_DEC + tid] = v;
                else if (tid == 32) rec[GNN_OFF_DEC + 32] = v;
            } else {
                rec[GNN_OFF_ENC + tid] = v;
            }
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_free(tmem, 128);
}

// ------------------------------------------------------- loss, Adam, misc --

__global__ void k_gnn_loss(GView g, float sgn, int kind, const float *z, const float *e, float *y, double *part,
                           GnnScalars *sc) {
    double v[2] = {0.0, 0.0};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < g.n; row += gridDim.x * blockDim.x) {
        const int sl = row >> 5, lane = row & 31;
        const int base = g.sl_ptr[sl], w = g.sl_w[sl];
        float st = 0.f, se = 0.f;
        for (int k = 0; k < w; ++k) {
            int pos = base + k * 32 + lane;
            int j = g.col[pos];
            float av = g.val[pos];
            st += av * (z[j] - e[j]);
            se += av * e[j];
        }
        st *= sgn;
        se *= sgn;
        y[row] = st;
        if (kind == 0) {
            v[0] += (double)(z[row] - e[row]) * st;
            v[1] += (double)e[row] * se;
        } else {
            v[0] += (double)st * st;
            v[1] += (double)se * se;
        }
    }
    if (grid_sums<2>(v, part, &sc->cnt[1])) {
        sc->loss_num = v[0];
        sc->loss_den = v[1];
    }
}

__global__ void k_gnn_store_loss(const GnnScalars *sc, double *out) {
    double d = sc->loss_den;
    *out = d > 0.0 ? sc->loss_num / d : 0.0;
}

__global__ void k_gnn_scale(GView g, const float *r, double *part, GnnScalars *sc) {
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        double u = (double)g.dinv[i] * r[i];
        v[0] += u * u;
    }
    if (grid_sums<1>(v, part, &sc->cnt[0])) {
        double s = sqrt(v[0] / (double)g.n);
        sc->s = (float)s;
        sc->inv_s = s > 0.0 ? (float)(1.0 / s) : 0.f;
    }
}

// Sum the per-CTA gradient records; update (Adam) or just report.
__global__ void k_gnn_adam(const float *rec, int nrec, float *p, float *m, float *v, uint16_t *wbf, float *grad_out,
                           double lr, int t, int update) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= GNN_NPARAM) return;
    double g = 0.0;
    for (int b = 0; b < nrec; ++b) g += rec[(size_t)b * GNN_NPARAM_PAD + q];
    if (grad_out) grad_out[q] = (float)g;
    if (!update) return;
    const double b1 = 0.9, b2 = 0.999, eps = 1e-8;
    double mq = b1 * m[q] + (1.0 - b1) * g;
    double vq = b2 * v[q] + (1.0 - b2) * g * g;
    m[q] = (float)mq;
    v[q] = (float)vq;
    double mh = mq / (1.0 - pow(b1, (double)t)), vh = vq / (1.0 - pow(b2, (double)t));
    float pn = (float)(p[q] - lr * mh / (sqrt(vh) + eps));
    p[q] = pn;
    int rel = q - GNN_OFF_LAYER;
    if (rel >= 0 && rel < GNN_LAYERS * GNN_LAYER_STRIDE && rel % GNN_LAYER_STRIDE < 2048) {
        int l = rel / GNN_LAYER_STRIDE, k = rel % GNN_LAYER_STRIDE, in = k / 32, o = k % 32;
        uint16_t b = __bfloat16_as_ushort(__float2bfloat16_rn(pn));
        wbf[l * GNN_WBF_LAYER + o * 64 + in] = b;
        wbf[l * GNN_WBF_LAYER + 2048 + in * 32 + o] = b;
    }
}

__global__ void k_gnn_refresh(const float *p, uint16_t *wbf) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= GNN_LAYERS * 2048) return;
    int l = q / 2048, k = q % 2048, in = k / 32, o = k % 32;
    uint16_t b = __bfloat16_as_ushort(__float2bfloat16_rn(p[GNN_OFF_LAYER + l * GNN_LAYER_STRIDE + k]));
    wbf[l * GNN_WBF_LAYER + o * 64 + in] = b;
    wbf[l * GNN_WBF_LAYER + 2048 + in * 32 + o] = b;
}

__global__ void k_gnn_dinv(int n, const int *sl_ptr, const double *val, float *dinv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double d = val[sl_ptr[i >> 5] + (i & 31)];
    dinv[i] = d != 0.0 ? (float)(1.0 / d) : 0.f;
}

// training pair from a partial solve: r = b - A x1, e = xs - x1 (x1 == nullptr: 0)
__global__ void k_pair_from(GView g, const double *val64, const double *b, const double *x1, const double *xs,
                            float *r, float *e) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    double ri = b[i], ei = xs[i];
    if (x1) {
        const int sl = i >> 5, lane = i & 31;
        const int base = g.sl_ptr[sl], w = g.sl_w[sl];
        double ax = 0.0;
        for (int k = 0; k < w; ++k) {
            int pos = base + k * 32 + lane;
            ax += val64[pos] * x1[g.col[pos]];
        }
        ri -= ax;
        ei -= x1[i];
    }
    r[i] = (float)ri;
    e[i] = (float)ei;
}

__global__ void k_to_f32(int n, const double *a, float *b) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}
__global__ void k_post_jacobi(int n, const float *z2, const float *w, const float *t, float *z) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) z[i] = z2[i] + w[i] * t[i];
}

__global__ void k_to_f64(int n, const float *a, double *b) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (double)a[i];
}

// ----------------------------------------------------------- flexible CG --

struct FcgArgs {
    GView g;      // FP32 matrix
    const double *val64;
    float sgn;
    const double *b;
    double *x;
    float *r, *z, *p, *q, *e;
    FcgState *fs;
    double *part;
    double inner_tol2;
    int stall_max;
};

// Row i of the FP32 matrix times x, the column indices and values of four
// entries loaded before their gathers (the sum runs in entry order, as a plain
// loop's); default cache policy, so the matrix stays in L2 between the kernels
// of an iteration that read it
__device__ __forceinline__ float sell_dot32(const GView &g, int i, const float *x) {
    const int lane = i & 31;
    int e = g.sl_ptr[i >> 5] + lane;
    const int w = g.sl_w[i >> 5];
    float acc = 0.f;
    int k = 0;
    for (; k + 4 <= w; k += 4, e += 128) {
        const int c0 = g.col[e], c1 = g.col[e + 32], c2 = g.col[e + 64], c3 = g.col[e + 96];
        const float v0 = g.val[e], v1 = g.val[e + 32], v2 = g.val[e + 64], v3 = g.val[e + 96];
        const float x0 = x[c0], x1 = x[c1], x2 = x[c2], x3 = x[c3];
        acc += v0 * x0;
        acc += v1 * x1;
        acc += v2 * x2;
        acc += v3 * x3;
    }
    for (; k < w; ++k, e += 32) acc += g.val[e] * x[g.col[e]];
    return acc;
}

__device__ __forceinline__ double spmv64_row(const GView &g, const double *val64, const double *x, int row) {
    const int sl = row >> 5, lane = row & 31;
    const int base = g.sl_ptr[sl], w = g.sl_w[sl];
    double s = 0.0;
    for (int k = 0; k < w; ++k) {
        int pos = base + k * 32 + lane;
        s += val64[pos] * x[g.col[pos]];
    }
    return s;
}

__global__ void k_fcg_init(FcgArgs a, int x0_zero, double eps, int maxit, int use_gnn) {
    double v[3] = {0.0, 0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.g.n; i += gridDim.x * blockDim.x) {
        double bi = a.b[i];
        double ri = x0_zero ? bi : bi - spmv64_row(a.g, a.val64, a.x, i);
        a.r[i] = (float)ri;
        a.e[i] = 0.f;
        double u = (double)a.g.dinv[i] * ri;
        v[0] += bi * bi;
        v[1] += ri * ri;
        v[2] += u * u;
    }
    if (grid_sums<3>(v, a.part, &a.fs->cnt[0])) {
        FcgState *f = a.fs;
        f->bnorm2 = v[0];
        f->eps2 = v[0] > 0.0 ? eps * eps * v[0] : eps * eps;
        f->rr = f->rr_upd = f->rr_best = v[1];
        double s = sqrt(v[2] / (double)a.g.n);
        f->s = (float)s;
        f->inv_s = s > 0.0 ? (float)(1.0 / s) : 0.f;
        f->res = v[0] > 0.0 ? sqrt(v[1] / v[0]) : sqrt(v[1]);
        f->iters = 0;
        f->refinements = 0;
        f->status = DEV_OK;
        f->done = v[1] <= f->eps2 ? 1 : 0;
        f->use_gnn = use_gnn;
        f->stall = 0;
        f->restart = 1;
        f->need_update = 0;
        f->fallback_at = -1;
        f->maxit = maxit;
        f->loops = 0;
        f->zq = f->pq = f->pq_prev = f->pr = f->alpha = 0.0;
    }
}

// x = 0 for a zero initial guess (before k_fcg_init reads it).
__global__ void k_fcg_zero(int n, double *x) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = 0.0;
}

__global__ void k_fcg_jacobi(FcgArgs a) {
    if (a.fs->done || a.fs->use_gnn) return;
    float f0 = 0.f;
    const bool rs = a.fs->restart;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.g.n; i += gridDim.x * blockDim.x) {
        float zi = a.g.dinv[i] * a.r[i];
        a.z[i] = zi;
        if (!rs) f0 += zi * a.q[i];
    }
    const float fv[1] = {f0};
    double v[1];
    if (grid_sums_f<1>(fv, v, a.part, &a.fs->cnt[0])) a.fs->zq = v[0];
}

// multigrid form, finest level after the coarse correction z2: t = r - A z2, then
// either (network off) z = z2 + w t and z.q_prev for the flexible beta, or
// (network on) t for the network and its scale s2 = rms(D^-1 t)
__global__ void k_fcg_mgfine(FcgArgs a, const float *z2, float *t, const float *w, int fine_net) {
    if (a.fs->done) return;
    const bool net = fine_net && a.fs->use_gnn, rs = a.fs->restart;
    float f0 = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.g.n; i += gridDim.x * blockDim.x) {
        const float ti = a.r[i] - sell_dot32(a.g, i, z2);
        if (net) {
            t[i] = ti;
            const float u = a.g.dinv[i] * ti;
            f0 += u * u;
        } else {
            const float zi = z2[i] + w[i] * ti;
            a.z[i] = zi;
            if (!rs) f0 += zi * a.q[i];
        }
    }
    const float fv[1] = {f0};
    double v[1];
    if (grid_sums_f<1>(fv, v, a.part, &a.fs->cnt[0])) {
        if (net) {
            double s = sqrt(v[0] / (double)a.g.n);
            a.fs->s2 = (float)s;
            a.fs->inv_s2 = s > 0.0 ? (float)(1.0 / s) : 0.f;
        } else {
            a.fs->zq = v[0];
        }
    }
}

// network as a coarse level's post-smoother: t = r - A zp on that level, and
// (network on) the network's input scale s2 = rms(D^-1 t) into the finest-level
// flexible CG's state
__global__ void k_lvl_resid(GView g, const float *r, const float *zp, float *t, FcgState *fs, double *part) {
    if (fs->done) return;
    const bool net = fs->use_gnn;  // written by other launches only: uniform here
    float f0 = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        const int base = g.sl_ptr[i >> 5], wd = g.sl_w[i >> 5], lane = i & 31;
        float az = 0.f;
        for (int k = 0; k < wd; ++k) {
            int pos = base + k * 32 + lane;
            az += g.val[pos] * zp[g.col[pos]];
        }
        const float ti = r[i] - az;
        t[i] = ti;
        if (net) {
            const float u = g.dinv[i] * ti;
            f0 += u * u;
        }
    }
    if (!net) return;
    const float fv[1] = {f0};
    double v[1];
    if (grid_sums_f<1>(fv, v, part, &fs->cnt[3])) {
        double s = sqrt(v[0] / (double)g.n);
        fs->s2 = (float)s;
        fs->inv_s2 = s > 0.0 ? (float)(1.0 / s) : 0.f;
    }
}

// the Jacobi post-smoothing step of that level while the network is off
__global__ void k_lvl_jacobi(int n, const float *zp, const float *w, const float *t, float *z, const FcgState *fs) {
    if (fs->done || fs->use_gnn) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) z[i] = zp[i] + w[i] * t[i];
}

// r = b - A x1 (FP64) rounded to FP32; x1 == nullptr: r = b
__global__ void k_res32(GView g, const double *val64, const double *b, const double *x1, float *r) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        double ri = b[i];
        if (x1) {
            const int base = g.sl_ptr[i >> 5], wd = g.sl_w[i >> 5], lane = i & 31;
            for (int k = 0; k < wd; ++k) {
                int pos = base + k * 32 + lane;
                ri -= val64[pos] * x1[g.col[pos]];
            }
        }
        r[i] = (float)ri;
    }
}

__global__ void k_fcg_dir(FcgArgs a) {
    if (a.fs->done) return;
    const bool rs = a.fs->restart;
    const double beta = rs ? 0.0 : a.fs->zq / a.fs->pq_prev;
    const float bf = (float)beta;
    float f0 = 0.f, f1 = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.g.n; i += gridDim.x * blockDim.x) {
        const float az = sell_dot32(a.g, i, a.z);
        float qi = rs ? az : az - bf * a.q[i];
        float pi = rs ? a.z[i] : a.z[i] - bf * a.p[i];
        a.q[i] = qi;
        a.p[i] = pi;
        f0 += pi * qi;
        f1 += pi * a.r[i];
    }
    const float fv[2] = {f0, f1};
    double v[2];
    if (grid_sums_f<2>(fv, v, a.part, &a.fs->cnt[1])) {
        FcgState *f = a.fs;
        double pq = v[0], pr = v[1];
        double alpha = pr / pq;
        bool bad = !((double)a.sgn * pq > 0.0) || !isfinite(alpha);
        f->pq = pq;
        f->pr = pr;
        if (bad) {
            f->alpha = 0.0;
            f->restart = 1;
            if (f->use_gnn) {
                f->use_gnn = 0;
                f->fallback_at = f->iters;
            } else {
                f->status = DEV_BREAKDOWN;
                f->need_update = 1;
            }
        } else {
            f->alpha = alpha;
            f->restart = 0;
        }
    }
}

// e += alpha p, r -= alpha q; r.r and |D^-1 r|^2.  Four rows a thread with
// 16-byte loads (the arrays are whole allocations, 16-byte aligned): a pure
// vector pass, where one row a thread left it at half of HBM.
__device__ __forceinline__ void fcg_upd_row(float al, float &r, float &e, float p, float q, float d, float &f0,
                                            float &f1) {
    if (al != 0.f) {
        e += al * p;
        r -= al * q;
    }
    const float u = d * r;
    f0 += r * r;
    f1 += u * u;
}

__global__ void k_fcg_upd(FcgArgs a) {
    if (a.fs->done) return;
    const float al = (float)a.fs->alpha;
    float f0 = 0.f, f1 = 0.f;
    const int n4 = a.g.n >> 2, T = gridDim.x * blockDim.x, t0 = blockIdx.x * blockDim.x + threadIdx.x;
    for (int j = t0; j < n4; j += T) {
        float4 r = ld4(a.r, j), e = ld4(a.e, j);
        const float4 p = ld4(a.p, j), q = ld4(a.q, j), d = ld4(a.g.dinv, j);
        fcg_upd_row(al, r.x, e.x, p.x, q.x, d.x, f0, f1);
        fcg_upd_row(al, r.y, e.y, p.y, q.y, d.y, f0, f1);
        fcg_upd_row(al, r.z, e.z, p.z, q.z, d.z, f0, f1);
        fcg_upd_row(al, r.w, e.w, p.w, q.w, d.w, f0, f1);
        if (al != 0.f) {
            st4(a.e, j, e);
            st4(a.r, j, r);
        }
    }
    for (int i = 4 * n4 + t0; i < a.g.n; i += T) {
        float r = a.r[i], e = a.e[i];
        fcg_upd_row(al, r, e, a.p[i], a.q[i], a.g.dinv[i], f0, f1);
        if (al != 0.f) {
            a.e[i] = e;
            a.r[i] = r;
        }
    }
    const float fv[2] = {f0, f1};
    double v[2];
    if (grid_sums_f<2>(fv, v, a.part, &a.fs->cnt[2])) {
        FcgState *f = a.fs;
        f->iters += 1;
        f->rr = v[0];
        double s = sqrt(v[1] / (double)a.g.n);
        f->s = (float)s;
        f->inv_s = s > 0.0 ? (float)(1.0 / s) : 0.f;
        f->pq_prev = f->pq;
        if (v[0] < f->rr_best) {
            f->rr_best = v[0];
            f->stall = 0;
        } else {
            f->stall += 1;
        }
        if (f->use_gnn && f->stall >= a.stall_max) {
            f->use_gnn = 0;
            f->restart = 1;
            f->fallback_at = f->iters;
        }
        if (v[0] <= a.inner_tol2 * f->rr_upd || v[0] <= f->eps2 || f->iters >= f->maxit || !isfinite(v[0]))
            f->need_update = 1;
    }
}

__global__ void k_fcg_rel1(FcgArgs a) {
    if (a.fs->done || !a.fs->need_update) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.g.n; i += gridDim.x * blockDim.x) {
        a.x[i] += (double)a.e[i];
        a.e[i] = 0.f;
    }
}

__global__ void k_fcg_rel2(FcgArgs a) {
    if (a.fs->done || !a.fs->need_update) return;
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.g.n; i += gridDim.x * blockDim.x) {
        double ri = a.b[i] - spmv64_row(a.g, a.val64, a.x, i);
        a.r[i] = (float)ri;
        double u = (double)a.g.dinv[i] * ri;
        v[0] += ri * ri;
        v[1] += u * u;
    }
    if (grid_sums<2>(v, a.part, &a.fs->cnt[3])) {
        FcgState *f = a.fs;
        f->refinements += 1;
        f->rr = f->rr_upd = f->rr_best = v[0];
        f->stall = 0;
        f->res = f->bnorm2 > 0.0 ? sqrt(v[0] / f->bnorm2) : sqrt(v[0]);
        double s = sqrt(v[1] / (double)a.g.n);
        f->s = (float)s;
        f->inv_s = s > 0.0 ? (float)(1.0 / s) : 0.f;
        f->need_update = 0;
        if (!isfinite(v[0])) {
            f->done = 1;
            f->status = DEV_NONFINITE;
        } else if (v[0] <= f->eps2) {
            f->done = 1;
            f->status = DEV_OK;
        } else if (f->status == DEV_BREAKDOWN || f->iters >= f->maxit) {
            f->done = 1;
            if (f->status != DEV_BREAKDOWN) f->status = DEV_MAXITER;
        }
    }
}

__global__ void k_fcg_info(const FcgState *f, SolveInfo *info) {
    info->status[0] = f->status;
    info->iters[0] = f->iters;
    info->res[0] = f->res;
    info->refinements = f->refinements;
    info->err = 0;
}

int blocks_flat(int n) { return std::max(1, std::min((n + FB - 1) / FB, num_sms() * 8)); }

}  // namespace

void GnnPrecond::drop_graphs() {
    for (SolveGraph &g : graphs_) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = SolveGraph{};
    }
}

void GnnPrecond::attach_multigrid(AggMultigrid *mg) {
    if (mg && (!mg->ready() || !bound() || mg->level_rows(0) != n_))
        throw CaseError{"multigrid: hierarchy not built for the bound matrix"};
    drop_graphs();
    mg_ = mg;
    if (mg_ && z2_.size() < (size_t)n_) {
        z2_.alloc(n_);
        t_.alloc(n_);
    }
}

void GnnPrecond::transform_pair(int k, cudaStream_t st) {
    if (!mg_) return;
    mg_->smoother_pair(pr_.get() + (size_t)k * n_, pe_.get() + (size_t)k * n_, st);
}

void GnnPrecond::bind(const SellDev &A, const double *val64, const float *val32, cudaStream_t st) {
    drop_graphs();
    mg_ = nullptr;
    A_ = &A;
    val64_ = val64;
    val32_ = val32;
    n_ = A.n;
    ntiles_ = (n_ + GT - 1) / GT;
    static bool attr = false;
    if (!attr) {
        SYSU_CUDA(cudaFuncSetAttribute(k_gnn_bwd<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, BWD_SMEM_REQ));
        SYSU_CUDA(cudaFuncSetAttribute(k_gnn_bwd<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, BWD_SMEM_REQ));
        SYSU_CUDA(cudaFuncSetAttribute(k_gnn_bwd<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, BWD_SMEM_REQ));
        attr = true;
    }
    // forward: as many co-resident CTAs as registers and shared memory allow
    // (the gather is latency-bound).  Computed from the kernel's attributes:
    // the runtime's occupancy query reports one CTA per SM for kernels that
    // allocate tensor memory.
    cudaFuncAttributes fa{};
    SYSU_CUDA(cudaFuncGetAttributes(&fa, k_gnn_fwd<false, true, true>));
    int by_regs = 65536 / std::max(1, fa.numRegs * GT);
    int by_smem = (227 * 1024) / (FWD_SMEM + (int)fa.sharedSizeBytes + 1024);
    int occ = std::max(1, std::min(std::min(by_regs, by_smem), 8));
    if (fwd_per_sm > 0) occ = fwd_per_sm;
    gfwd_ = std::max(1, std::min(ntiles_, num_sms() * occ));
    gtiles_ = std::max(1, std::min(ntiles_, num_sms() * 3));
    gflat_ = blocks_flat(n_);
    const size_t n = (size_t)n_;
    dinv_.alloc(n);
    refresh(st);
    double d0 = 0.0;  // the matrix's sign (entry 0 is row 0's diagonal)
    SYSU_CUDA(cudaMemcpyAsync(&d0, val64_, sizeof(double), cudaMemcpyDeviceToHost, st));
    SYSU_CUDA(cudaStreamSynchronize(st));
    sgn_ = d0 < 0.0 ? -1.0f : 1.0f;
    if (p_.size() == 0) {
        p_.alloc(GNN_NPARAM_PAD);
        m_.alloc(GNN_NPARAM_PAD);
        v_.alloc(GNN_NPARAM_PAD);
        wbf_.alloc(GNN_LAYERS * GNN_WBF_LAYER);
        p_.zero(st);
        m_.zero(st);
        v_.zero(st);
        wbf_.zero(st);
        sc_.alloc(1);
        fs_.alloc(1);
        sc_.zero(st);
        fs_.zero(st);
        losses_.alloc(1 << 16);
        err_.alloc(1);
        err_.zero(st);
    }
    rec_.alloc((size_t)gtiles_ * GNN_NPARAM_PAD);
    part_.alloc((size_t)std::max(std::max(gtiles_, gfwd_), gflat_) * 4);
    H_.alloc(5 * n * 32);
    M_.alloc(4 * n * 32);
    mask_.alloc(4 * n);
    aw_.alloc(2 * n);
    dA_.alloc(n * 32);
    gA_.alloc(n * 32);
    dB_.alloc(n * 32);
    gB_.alloc(n * 32);
    for (DevBuf<float> *b : {&z32_, &y32_, &r32_, &e32_, &p32_, &q32_, &x32_}) b->alloc(n);
    pr_.alloc((size_t)capacity_ * n);
    pe_.alloc((size_t)capacity_ * n);
    r64_.alloc(n);
    count_ = next_ = 0;
}

// New values of the bound matrix (same pattern and the same sign convention,
// which bind read): the Jacobi weights.  No host round trip, so a refresh can be
// part of a captured outer iteration.
void GnnPrecond::refresh(cudaStream_t st) {
    k_gnn_dinv<<<(n_ + FB - 1) / FB, FB, 0, st>>>(n_, A_->sl_ptr.get(), val64_, dinv_.get());
    ++g_launches;
    SYSU_CUDA(cudaGetLastError());
}

void GnnPrecond::refresh_bf16(cudaStream_t st) {
    k_gnn_refresh<<<(GNN_LAYERS * 2048 + FB - 1) / FB, FB, 0, st>>>(p_.get(), wbf_.get());
    ++g_launches;
    SYSU_CUDA(cudaGetLastError());
}

void GnnPrecond::init_params(unsigned long long seed, cudaStream_t st) {
    std::vector<float> h(GNN_NPARAM_PAD, 0.f);
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<float> U(-1.f, 1.f);
    for (int c = 0; c < 64; ++c) h[GNN_OFF_ENC + c] = U(rng);
    const float a = std::sqrt(6.0f / 96.0f) * 0.5f;
    for (int l = 0; l < GNN_LAYERS; ++l)
        for (int k = 0; k < 2048; ++k) h[GNN_OFF_LAYER + l * GNN_LAYER_STRIDE + k] = a * U(rng);
    set_params(h.data(), st);
}

void GnnPrecond::set_params(const float *host, cudaStream_t st) {
    if (!p_.size()) throw CaseError{"learned preconditioner: bind a matrix first"};
    p_.upload(host, GNN_NPARAM, st);
    SYSU_CUDA(cudaStreamSynchronize(st));
    refresh_bf16(st);
    reset_adam(st);
}

void GnnPrecond::get_params(float *host, cudaStream_t st) {
    p_.download(host, GNN_NPARAM, st);
    SYSU_CUDA(cudaStreamSynchronize(st));
}

void GnnPrecond::reset_adam(cudaStream_t st) {
    m_.zero(st);
    v_.zero(st);
    adam_t_ = 0;
}

static GView gview(const SellDev &A, const float *val32, const float *dinv) {
    return GView{A.n, A.sl_ptr.get(), A.sl_w.get(), A.col.get(), val32, dinv};
}

void GnnPrecond::scale_of(const float *r32, cudaStream_t st) {
    k_gnn_scale<<<gflat_, FB, 0, st>>>(gview(*A_, val32_, dinv_.get()), r32, part_.get(), sc_.get());
    ++g_launches;
    SYSU_CUDA(cudaGetLastError());
}

void GnnPrecond::forward(const float *r32, float *z32, bool train, FcgState *fs, const float *qprev, cudaStream_t st,
                         const float *zbase) {
    NetArgs a{};
    a.g = gview(*A_, val32_, dinv_.get());
    a.r = r32;
    a.inv_s_p = fs ? (zbase ? &fs->inv_s2 : &fs->inv_s) : &sc_.get()->inv_s;
    a.s_p = fs ? (zbase ? &fs->s2 : &fs->s) : &sc_.get()->s;
    a.zbase = zbase;
    a.skip = skip;
    a.prm = p_.get();
    a.aw = aw_.get();
    a.z = z32;
    a.qprev = qprev;
    a.fs = fs;
    a.part = part_.get();
    a.err = err_.get();
    const size_t nn = (size_t)n_ * 32;
    for (int l = 0; l < GNN_LAYERS; ++l) {
        a.layer = l;
        a.wbf = wbf_.get() + l * GNN_WBF_LAYER;
        if (train) {
            a.hin = l ? H_.get() + (size_t)l * nn : nullptr;
            a.hout = H_.get() + (size_t)(l + 1) * nn;
            a.mout = M_.get() + (size_t)l * nn;
            a.mask = mask_.get() + (size_t)l * n_;
        } else {
            a.hin = l ? H_.get() + (size_t)(l & 1 ? 1 : 2) * nn : nullptr;
            a.hout = H_.get() + (size_t)(l & 1 ? 2 : 1) * nn;
            a.mout = nullptr;
            a.mask = nullptr;
        }
        dim3 grid(gfwd_), blk(GT);
        if (l == 0) {
            if (train) k_gnn_fwd<true, true, false><<<grid, blk, FWD_SMEM, st>>>(a);
            else k_gnn_fwd<true, false, false><<<grid, blk, FWD_SMEM, st>>>(a);
        } else if (l == GNN_LAYERS - 1) {
            if (train) k_gnn_fwd<false, true, true><<<grid, blk, FWD_SMEM, st>>>(a);
            else k_gnn_fwd<false, false, true><<<grid, blk, FWD_SMEM, st>>>(a);
        } else {
            if (train) k_gnn_fwd<false, true, false><<<grid, blk, FWD_SMEM, st>>>(a);
            else k_gnn_fwd<false, false, false><<<grid, blk, FWD_SMEM, st>>>(a);
        }
        ++g_launches;
        SYSU_CUDA(cudaGetLastError());
    }
}

void GnnPrecond::backward(const float *r32, cudaStream_t st) {
    BwdArgs a{};
    a.g = gview(*A_, val32_, dinv_.get());
    a.sgn = sgn_;
    a.kind = loss_kind;
    a.r = r32;
    a.inv_s_p = &sc_.get()->inv_s;
    a.s_p = &sc_.get()->s;
    a.prm = p_.get();
    a.aw = aw_.get();
    a.h4 = H_.get() + (size_t)4 * n_ * 32;
    a.y = y32_.get();
    a.sc = sc_.get();
    a.rec = rec_.get();
    a.err = err_.get();
    const size_t nn = (size_t)n_ * 32;
    float *dbuf[2] = {dA_.get(), dB_.get()}, *gbuf[2] = {gA_.get(), gB_.get()};
    for (int l = GNN_LAYERS - 1; l >= 0; --l) {
        a.layer = l;
        a.wbf = wbf_.get() + l * GNN_WBF_LAYER;
        a.hprev = l ? H_.get() + (size_t)l * nn : nullptr;
        a.mcur = M_.get() + (size_t)l * nn;
        a.mask = mask_.get() + (size_t)l * n_;
        int in = (l + 1) & 1, out = l & 1;
        a.dIn = dbuf[in];
        a.gIn = gbuf[in];
        a.dOut = dbuf[out];
        a.gOut = gbuf[out];
        dim3 grid(gtiles_), blk(GT);
        if (l == GNN_LAYERS - 1) k_gnn_bwd<true, false><<<grid, blk, BWD_SMEM_REQ, st>>>(a);
        else if (l == 0) k_gnn_bwd<false, true><<<grid, blk, BWD_SMEM_REQ, st>>>(a);
        else k_gnn_bwd<false, false><<<grid, blk, BWD_SMEM_REQ, st>>>(a);
        ++g_launches;
        SYSU_CUDA(cudaGetLastError());
    }
}

void GnnPrecond::apply(const double *r, double *z, cudaStream_t st) {
    if (!bound()) throw CaseError{"learned preconditioner: no matrix bound"};
    int nb = (n_ + FB - 1) / FB;
    k_to_f32<<<nb, FB, 0, st>>>(n_, r, r32_.get());
    ++g_launches;
    scale_of(r32_.get(), st);
    forward(r32_.get(), z32_.get(), false, nullptr, nullptr, st);
    k_to_f64<<<nb, FB, 0, st>>>(n_, z32_.get(), z);
    ++g_launches;
    SYSU_CUDA(cudaGetLastError());
    check_err(st);
}

void GnnPrecond::post_smooth(const float *r, const float *zp, float *z, FcgState *fs, const float *w, cudaStream_t st) {
    if (!bound()) throw CaseError{"coarse-level network: no matrix bound"};
    if (t_.size() < (size_t)n_) t_.alloc(n_);
    k_lvl_resid<<<gflat_, FB, 0, st>>>(gview(*A_, val32_, dinv_.get()), r, zp, t_.get(), fs, part_.get());
    ++g_launches;
    forward(t_.get(), z, false, fs, nullptr, st, zp);
    k_lvl_jacobi<<<gflat_, FB, 0, st>>>(n_, zp, w, t_.get(), z, fs);
    ++g_launches;
    SYSU_CUDA(cudaGetLastError());
}

void GnnPrecond::residual32(const double *b, const double *x1, float *r, cudaStream_t st) {
    if (!bound()) throw CaseError{"learned preconditioner: no matrix bound"};
    k_res32<<<gflat_, FB, 0, st>>>(gview(*A_, val32_, dinv_.get()), val64_, b, x1, r);
    ++g_launches;
    SYSU_CUDA(cudaGetLastError());
}

void GnnPrecond::apply_mg(const double *r, double *z, bool use_gnn, cudaStream_t st) {
    if (!bound() || !mg_) throw CaseError{"multigrid form: no matrix bound or no hierarchy attached"};
    int nb = (n_ + FB - 1) / FB;
    k_to_f32<<<nb, FB, 0, st>>>(n_, r, r32_.get());
    ++g_launches;
    mg_->apply_fixed(r32_.get(), z2_.get(), t_.get(), nullptr, st);
    if (use_gnn) {
        scale_of(t_.get(), st);
        forward(t_.get(), z32_.get(), false, nullptr, nullptr, st, z2_.get());
    } else {
        k_post_jacobi<<<nb, FB, 0, st>>>(n_, z2_.get(), mg_->w0(), t_.get(), z32_.get());
        ++g_launches;
    }
    k_to_f64<<<nb, FB, 0, st>>>(n_, z32_.get(), z);
    ++g_launches;
    SYSU_CUDA(cudaGetLastError());
    check_err(st);
}

double GnnPrecond::time_apply(const double *r, int reps, cudaStream_t st) {
    int nb = (n_ + FB - 1) / FB;
    k_to_f32<<<nb, FB, 0, st>>>(n_, r, r32_.get());
    ++g_launches;
    scale_of(r32_.get(), st);
    forward(r32_.get(), z32_.get(), false, nullptr, nullptr, st);
    cudaEvent_t e0, e1;
    SYSU_CUDA(cudaEventCreate(&e0));
    SYSU_CUDA(cudaEventCreate(&e1));
    SYSU_CUDA(cudaEventRecord(e0, st));
    for (int i = 0; i < reps; ++i) forward(r32_.get(), z32_.get(), false, nullptr, nullptr, st);
    SYSU_CUDA(cudaEventRecord(e1, st));
    SYSU_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    check_err(st);
    return ms / std::max(reps, 1);
}

void GnnPrecond::check_err(cudaStream_t st) {
    int e = 0;
    SYSU_CUDA(cudaMemcpyAsync(&e, err_.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
    SYSU_CUDA(cudaStreamSynchronize(st));
    if (e) {
        err_.zero(st);
        throw CaseError{"learned preconditioner: a tensor-core wait timed out"};
    }
}

void GnnPrecond::add_pair(const double *r, const double *e, cudaStream_t st) {
    if (!bound()) throw CaseError{"learned preconditioner: no matrix bound"};
    int nb = (n_ + FB - 1) / FB;
    size_t off = (size_t)next_ * n_;
    k_to_f32<<<nb, FB, 0, st>>>(n_, r, pr_.get() + off);
    k_to_f32<<<nb, FB, 0, st>>>(n_, e, pe_.get() + off);
    g_launches += 2;
    SYSU_CUDA(cudaGetLastError());
    transform_pair(next_, st);
    next_ = (next_ + 1) % capacity_;
    count_ = std::min(count_ + 1, capacity_);
}

void GnnPrecond::add_pair_from(const double *b, const double *x1, const double *xs, cudaStream_t st) {
    if (!bound()) throw CaseError{"learned preconditioner: no matrix bound"};
    size_t off = (size_t)next_ * n_;
    k_pair_from<<<(n_ + FB - 1) / FB, FB, 0, st>>>(gview(*A_, val32_, dinv_.get()), val64_, b, x1, xs,
                                                  pr_.get() + off, pe_.get() + off);
    ++g_launches;
    SYSU_CUDA(cudaGetLastError());
    transform_pair(next_, st);
    next_ = (next_ + 1) % capacity_;
    count_ = std::min(count_ + 1, capacity_);
}

void GnnPrecond::train_step(int k, double lr, cudaStream_t st) {
    if (count_ == 0) throw CaseError{"learned preconditioner: no training pairs"};
    k %= count_;
    const float *r = pr_.get() + (size_t)k * n_, *e = pe_.get() + (size_t)k * n_;
    scale_of(r, st);
    forward(r, z32_.get(), true, nullptr, nullptr, st);
    k_gnn_loss<<<gflat_, FB, 0, st>>>(gview(*A_, val32_, dinv_.get()), sgn_, loss_kind, z32_.get(), e, y32_.get(),
                                      part_.get(), sc_.get());
    ++g_launches;
    backward(r, st);
    ++adam_t_;
    k_gnn_adam<<<(GNN_NPARAM + FB - 1) / FB, FB, 0, st>>>(rec_.get(), gtiles_, p_.get(), m_.get(), v_.get(),
                                                          wbf_.get(), nullptr, lr, adam_t_, 1);
    k_gnn_store_loss<<<1, 1, 0, st>>>(sc_.get(), losses_.get() + ((adam_t_ - 1) & ((1 << 16) - 1)));
    g_launches += 2;
    SYSU_CUDA(cudaGetLastError());
}

void GnnPrecond::loss_grad(int k, double *loss, float *grad_host, cudaStream_t st) {
    if (count_ == 0) throw CaseError{"learned preconditioner: no training pairs"};
    k %= count_;
    const float *r = pr_.get() + (size_t)k * n_, *e = pe_.get() + (size_t)k * n_;
    scale_of(r, st);
    forward(r, z32_.get(), true, nullptr, nullptr, st);
    k_gnn_loss<<<gflat_, FB, 0, st>>>(gview(*A_, val32_, dinv_.get()), sgn_, loss_kind, z32_.get(), e, y32_.get(),
                                      part_.get(), sc_.get());
    ++g_launches;
    backward(r, st);
    DevBuf<float> g(GNN_NPARAM);
    k_gnn_adam<<<(GNN_NPARAM + FB - 1) / FB, FB, 0, st>>>(rec_.get(), gtiles_, p_.get(), m_.get(), v_.get(),
                                                          wbf_.get(), g.get(), 0.0, 1, 0);
    k_gnn_store_loss<<<1, 1, 0, st>>>(sc_.get(), losses_.get());
    g_launches += 2;
    SYSU_CUDA(cudaGetLastError());
    g.download(grad_host, GNN_NPARAM, st);
    SYSU_CUDA(cudaMemcpyAsync(loss, losses_.get(), sizeof(double), cudaMemcpyDeviceToHost, st));
    SYSU_CUDA(cudaStreamSynchronize(st));
    check_err(st);
}

void GnnPrecond::last_losses(std::vector<double> &out, int count, cudaStream_t st) {
    count = std::min(count, std::min(adam_t_, 1 << 16));
    out.assign(count, 0.0);
    for (int i = 0; i < count; ++i) {
        int idx = (adam_t_ - count + i) & ((1 << 16) - 1);
        SYSU_CUDA(cudaMemcpyAsync(&out[i], losses_.get() + idx, sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    SYSU_CUDA(cudaStreamSynchronize(st));
}

// One flexible-CG iteration (network or Jacobi preconditioner, direction,
// update, conditional reliable update) enqueued on st.
void GnnPrecond::fcg_iteration(const void *args, bool use_gnn, cudaStream_t st) {
    const FcgArgs &a = *static_cast<const FcgArgs *>(args);
    if (mg_) {
        mg_->apply_to_fine(a.r, z2_.get(), &a.fs->done, st);
        k_fcg_mgfine<<<gflat_, FB, 0, st>>>(a, z2_.get(), t_.get(), mg_->w0(), net_level == 0 ? 1 : 0);
        ++g_launches;
        if (use_gnn && net_level == 0) forward(t_.get(), a.z, false, a.fs, a.q, st, z2_.get());
    } else {
        if (use_gnn) forward(a.r, a.z, false, a.fs, a.q, st);
        k_fcg_jacobi<<<gflat_, FB, 0, st>>>(a);
    }
    k_fcg_dir<<<gflat_, FB, 0, st>>>(a);
    k_fcg_upd<<<gflat_, FB, 0, st>>>(a);
    k_fcg_rel1<<<gflat_, FB, 0, st>>>(a);
    k_fcg_rel2<<<gflat_, FB, 0, st>>>(a);
    g_launches += mg_ ? 4 : 5;
    SYSU_CUDA(cudaGetLastError());
}

// Everything a captured flexible-CG solve bakes in: its kernels' arguments, the
// caller's b, x and statistics pointers, the initial kernel's scalars and the
// attached cycle's parameters.
struct FcgKey {
    FcgArgs a;
    const double *b_in;
    double *x_out;
    SolveInfo *info;
    int x0_zero, maxit, use_gnn, chunk, gflat, net_level, post_level, hook, mg_persistent;
    double eps, mg_gamma;
    float skip;
    const void *mg;
};

void GnnPrecond::fcg(const double *b, double *x, bool x0_zero, const KrylovOpts &o, bool use_gnn, SolveInfo *info_dev,
                     cudaStream_t st) {
    if (!bound()) throw CaseError{"learned preconditioner: no matrix bound"};
    // the iterations run over fixed buffers: b and x are copied in and out
    if (b64_.size() < (size_t)n_) {
        b64_.alloc(n_);
        x64_.alloc(n_);
    }
    FcgKey k;
    std::memset(&k, 0, sizeof(k));  // padding too: the key is compared as bytes
    FcgArgs &a = k.a;
    a.g = gview(*A_, val32_, dinv_.get());
    a.val64 = val64_;
    a.sgn = sgn_;
    a.b = b64_.get();
    a.x = x64_.get();
    a.r = r32_.get();
    a.z = z32_.get();
    a.p = p32_.get();
    a.q = q32_.get();
    a.e = e32_.get();
    a.fs = fs_.get();
    a.part = part_.get();
    a.inner_tol2 = o.inner_tol * o.inner_tol;
    a.stall_max = stall_max;
    k.b_in = b;
    k.x_out = x;
    k.info = info_dev;
    k.x0_zero = x0_zero ? 1 : 0;
    k.maxit = o.maxit;
    k.use_gnn = use_gnn ? 1 : 0;
    k.chunk = check_every;
    k.gflat = gflat_;
    k.eps = o.eps;
    k.skip = skip;
    k.mg = mg_;
    if (mg_) {
        k.net_level = net_level;
        k.post_level = mg_->post_level;
        k.hook = mg_->post_hook ? 1 : 0;
        k.mg_persistent = mg_->persistent ? 1 : 0;
        k.mg_gamma = mg_->gamma;
    }
    // b, x0 in; the iterations; x and the statistics out
    auto prologue = [&](cudaStream_t s) {
        SYSU_CUDA(cudaMemcpyAsync(b64_.get(), b, sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
        if (!x0_zero) SYSU_CUDA(cudaMemcpyAsync(x64_.get(), x, sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
        if (x0_zero) {
            k_fcg_zero<<<(n_ + FB - 1) / FB, FB, 0, s>>>(n_, a.x);
            ++g_launches;
        }
        k_fcg_init<<<gflat_, FB, 0, s>>>(a, x0_zero ? 1 : 0, o.eps, o.maxit, use_gnn ? 1 : 0);
        ++g_launches;
        SYSU_CUDA(cudaGetLastError());
    };
    auto epilogue = [&](cudaStream_t s) {
        SYSU_CUDA(cudaMemcpyAsync(x, x64_.get(), sizeof(double) * n_, cudaMemcpyDeviceToDevice, s));
        k_fcg_info<<<1, 1, 0, s>>>(fs_.get(), info_dev);
        ++g_launches;
        SYSU_CUDA(cudaGetLastError());
    };
    // the iterations as a WHILE node: check_every a body; the body's last kernel
    // ends the loop once the solve is done, or after maxit / check_every + 8
    // bodies (the solve stops at maxit itself)
    auto enqueue = [&](cudaStream_t s) {
        prologue(s);
        const int bound = o.maxit / std::max(1, check_every) + 8;
        cudaGraphConditionalHandle loop = graph_cond_handle(s, 1);
        graph_cond_node(s, graph_side_stream(), loop, cudaGraphCondTypeWhile, [&](cudaStream_t bs) {
            for (int c = 0; c < check_every; ++c) fcg_iteration(&a, use_gnn, bs);
            graph_loop_tail(loop, &a.fs->done, &a.fs->loops, bound, bs);
        });
        epilogue(s);
    };
    if (stream_capturing(st)) {  // inside the caller's graph: errors surface in the statuses
        enqueue(st);
        return;
    }
    if (!device_loop) {
        // host-driven form, for per-kernel profiling (profilers skip the kernels of
        // graphs with conditional nodes): the same kernels, check_every
        // iterations a captured graph, the host reading `done` after each
        k.chunk = -check_every;  // a different cache entry from the device loop's
        const unsigned char *kc = reinterpret_cast<const unsigned char *>(&k);
        SolveGraph *cg = nullptr;
        for (SolveGraph &g : graphs_)
            if (g.exec && g.key.size() == sizeof(k) && std::memcmp(g.key.data(), kc, sizeof(k)) == 0) cg = &g;
        if (!cg) {
            cg = &graphs_[graph_next_];
            graph_next_ = (graph_next_ + 1) % 4;
            if (cg->exec) cudaGraphExecDestroy(cg->exec);
            *cg = SolveGraph{};
            const long before = g_launches.load();
            cudaGraph_t g;
            SYSU_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            for (int c = 0; c < check_every; ++c) fcg_iteration(&a, use_gnn, st);
            SYSU_CUDA(cudaStreamEndCapture(st, &g));
            cg->launches = g_launches.load() - before;
            g_launches -= cg->launches;
            cudaError_t e = cudaGraphInstantiate(&cg->exec, g, 0);
            cudaGraphDestroy(g);
            SYSU_CUDA(e);
            cg->key.assign(kc, kc + sizeof(k));
        }
        prologue(st);
        int done = 0;
        for (int it = 0; it < o.maxit + check_every && !done; it += check_every) {
            SYSU_CUDA(cudaGraphLaunch(cg->exec, st));
            g_launches += cg->launches;
            SYSU_CUDA(cudaMemcpyAsync(&done, &fs_.get()->done, sizeof(int), cudaMemcpyDeviceToHost, st));
            SYSU_CUDA(cudaStreamSynchronize(st));
        }
        epilogue(st);
        if (use_gnn || (mg_ && mg_->post_hook)) check_err(st);
        return;
    }
    const unsigned char *kb = reinterpret_cast<const unsigned char *>(&k);
    SolveGraph *sg = nullptr;
    for (SolveGraph &g : graphs_)
        if (g.exec && g.key.size() == sizeof(k) && std::memcmp(g.key.data(), kb, sizeof(k)) == 0) sg = &g;
    if (!sg) {
        sg = &graphs_[graph_next_];
        graph_next_ = (graph_next_ + 1) % 4;
        if (sg->exec) cudaGraphExecDestroy(sg->exec);
        *sg = SolveGraph{};
        const long before = g_launches.load();
        cudaGraph_t g;
        SYSU_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
            enqueue(st);
        } catch (...) {
            cudaGraph_t junk = nullptr;
            cudaStreamEndCapture(st, &junk);
            if (junk) cudaGraphDestroy(junk);
            throw;
        }
        SYSU_CUDA(cudaStreamEndCapture(st, &g));
        sg->launches = g_launches.load() - before;
        g_launches -= sg->launches;
        cudaError_t e = cudaGraphInstantiate(&sg->exec, g, 0);
        cudaGraphDestroy(g);
        SYSU_CUDA(e);
        sg->key.assign(kb, kb + sizeof(k));
    }
    SYSU_CUDA(cudaGraphLaunch(sg->exec, st));
    g_launches += sg->launches;
    // a network that timed out on a tensor-core wait (the plain cycle sets nothing)
    if (use_gnn || (mg_ && mg_->post_hook)) check_err(st);
}

GnnPrecond::~GnnPrecond() { drop_graphs(); }

__global__ void k_bf16_to_f32(long n, const uint16_t *a, float *b) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = __uint_as_float((uint32_t)a[i] << 16);
}

void GnnPrecond::hidden(const double *r, int layer, float *host, cudaStream_t st) {
    if (!bound()) throw CaseError{"learned preconditioner: no matrix bound"};
    if (layer < 1 || layer > GNN_LAYERS) throw CaseError{"hidden: layer 1..4"};
    int nb = (n_ + FB - 1) / FB;
    k_to_f32<<<nb, FB, 0, st>>>(n_, r, r32_.get());
    ++g_launches;
    scale_of(r32_.get(), st);
    forward(r32_.get(), z32_.get(), true, nullptr, nullptr, st);
    long nn = (long)n_ * 32;
    DevBuf<float> tmp(nn);
    k_bf16_to_f32<<<(unsigned)((nn + FB - 1) / FB), FB, 0, st>>>(nn, H_.get() + (size_t)layer * nn, tmp.get());
    ++g_launches;
    SYSU_CUDA(cudaGetLastError());
    tmp.download(host, nn, st);
    SYSU_CUDA(cudaStreamSynchronize(st));
    check_err(st);
}

FcgState GnnPrecond::last_state(cudaStream_t st) {
    FcgState f;
    SYSU_CUDA(cudaMemcpyAsync(&f, fs_.get(), sizeof(FcgState), cudaMemcpyDeviceToHost, st));
    SYSU_CUDA(cudaStreamSynchronize(st));
    return f;
}

}  // namespace sysu
