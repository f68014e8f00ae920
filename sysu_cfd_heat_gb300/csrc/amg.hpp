// Aggregation multigrid for the pressure-correction systems: the multilevel
// preconditioner of the flexible CG of the p' equation (its plain form), and
// the cycle whose fine-level post-smoother the learned network replaces (its
// learned form).  The reference solves p' with CG + SSOR (navier_pressure.cpp:29);
// both forms keep that stopping test, ||b - A x|| / ||b|| < eps.
//
// Hierarchy (host, once per matrix pattern): greedy aggregation of the matrix
// graph.  Row i's strong neighbours are the j != i whose coupling, with the
// sign opposite to the diagonal's, is at least theta times the row's largest;
// pass 1 visits rows in order and makes every row whose strong neighbours are
// all unaggregated the seed of a new aggregate {i} + strong(i); pass 2 puts each
// remaining row into the aggregate of its strongest aggregated strong neighbour
// (first in row order on ties); pass 3 makes the rest singletons.  Aggregates
// are numbered in creation order.  The next level is the Galerkin product
// A_c = P^T A P with P the piecewise-constant prolongation (A_c[I,J] = sum of
// a_ij over i in I, j in J), stored SELL-32 with the diagonal first and the
// other entries in order of first appearance over the members of I (ascending)
// and their entries in row order.  Levels are added until a level has at most
// MG_DENSE_MAX rows, which is inverted densely.
//
// Values (device, once per matrix): every coarse entry is the FP64 sum of its
// fine entries in a fixed order (a gather list per coarse position), so the
// coarse operators are bit-identical run to run; each level keeps an FP32 copy
// and w = omega / a_ii.  The coarsest level is inverted in FP32 by Gauss-Jordan
// in one CTA; when its rows sum to zero (the closed-domain p' systems are
// singular with the constant null vector), alpha 1 1^T with alpha = mean(a_ii) / n
// is added first, which leaves the solution of every consistent system unchanged.
//
// Cycle (FP32, V-cycle, one pre- and one post-smoothing step per level):
//   down, level l:  z = w r;  t = r - A z;  r_{l+1}[I] = sum_{i in I} t_i
//   coarsest:       z = A^-1 r
//   up, level l:    z_i = w_i r_i + gamma z_{l+1}[agg(i)];  z += w (r - A z)
// At the finest level the post-smoothing step is either Jacobi (as above) or
// the network applied to t = r - A z:  z += N(t).
#pragma once

#include <functional>
#include <memory>
#include <vector>

#include "krylov.hpp"

namespace sysu {

constexpr int MG_DENSE_MAX = 200;   // coarsest level: dense inverse in one CTA's shared memory
constexpr int MG_MAX_LEVELS = 16;

// One level of the host hierarchy (pattern and maps; values only for strength).
struct MgHostLevel {
    int n = 0;
    SellPattern pat;               // this level's matrix (level 0: the caller's pattern)
    std::vector<double> val;       // values in SELL layout (host, strength of the next aggregation)
    // to the next level (empty on the coarsest)
    std::vector<int> agg;          // coarse row of each row
    std::vector<int> mem_ptr, mem_idx;  // rows of each coarse row, ascending
    std::vector<int> gal_ptr, gal_src;  // per coarse stored position: positions of this level's entries
};

// Build the hierarchy from a SELL pattern and its FP64 values (SELL layout).
std::vector<MgHostLevel> mg_build_hierarchy(const SellPattern &fine, const std::vector<double> &val, double theta,
                                            int dense_max);

struct MgLevelDev {
    int n = 0;
    SellDev A;                     // level >= 1 (level 0 uses the caller's pattern)
    DevBuf<double> val64;          // level >= 1
    DevBuf<float> val32;           // level >= 1
    DevBuf<float> w;               // omega / a_ii
    DevBuf<float> r, z, t;         // cycle vectors
    DevBuf<int> agg, mem_ptr, mem_idx, gal_ptr, gal_src;  // to the next level
    int grow = 1, gagg = 1;        // lanes per row / per aggregate of the cycle kernels
};

// b = a in FP64 (n values on the device)
void mg_to_f64(const float *a, double *b, int n, cudaStream_t st);

class AggMultigrid {
  public:
    AggMultigrid() = default;
    AggMultigrid(const AggMultigrid &) = delete;
    AggMultigrid &operator=(const AggMultigrid &) = delete;

    // Build the hierarchy for the fine pattern A (with host pattern `pat`) from the
    // FP64 values on the device (downloaded once for the strength of connection).
    void setup(const SellDev &A, const SellPattern &pat, const double *val64_dev, double theta, cudaStream_t st);
    bool ready() const { return !lv_.empty(); }
    // New fine values (same pattern): Galerkin values, FP32 copies, w, coarsest inverse.
    // val32_dev: the FP32 copy of the fine values the cycle's fine SpMVs read.
    void refresh(const double *val64_dev, const float *val32_dev, cudaStream_t st);

    // z = M r (whole V-cycle with the Jacobi post-smoother at the finest level).
    // If fs_done != nullptr, every kernel returns at once when *fs_done != 0.
    void apply(const float *r, float *z, const int *fs_done, cudaStream_t st);
    // The fixed part of the cycle at the finest level: z2 = pre-smoothing + coarse
    // correction, t = r - A z2 (the input of the finest post-smoother).
    void apply_fixed(const float *r, float *z2, float *t, const int *fs_done, cudaStream_t st);
    // z2 alone (the caller forms t = r - A z2 itself, fused with what follows).
    void apply_to_fine(const float *r, float *z2, const int *fs_done, cudaStream_t st);
    // true: the coarse levels run as one persistent cooperative launch (grid
    // barriers between phases); false: one launch per phase.  Same results.
    bool persistent = false;
    // Training pair for the post-smoother from a pair (r, e = A^-1 r), in place:
    // r <- r - A z2(r), e <- e - z2(r).
    void smoother_pair(float *r, float *e, cudaStream_t st);

    // The post-smoothing step of one coarse level, post_level (1 <= post_level <
    // levels() - 1), replaced by post_hook: called while the cycle is enqueued,
    // with the level, its right-hand side r, the prolonged correction
    // zp = w r + gamma P z_{l+1}, the output z and the done flag; it enqueues
    // z = zp + (a smoothing step for r - A zp).  Kernels enqueued from it run
    // inside the flexible CG's captured iterations.  The persistent form does
    // not take a hook (the one-launch-per-phase form runs then).
    std::function<void(int, const float *, const float *, float *, const int *, cudaStream_t)> post_hook;
    int post_level = -1;
    // Level l >= 1: its matrix (device pattern, FP64 and FP32 values), host
    // pattern and smoother weights w = omega / a_ii.
    const SellDev &level_matrix(int l) const { return lv_[l]->A; }
    const double *level_val64(int l) const { return lv_[l]->val64.get(); }
    const float *level_val32(int l) const { return lv_[l]->val32.get(); }
    const SellPattern &level_pattern(int l) const { return hpat_[l]; }
    const float *level_w(int l) const { return lv_[l]->w.get(); }
    // The right-hand side the cycle hands level l >= 1 for the finest-level
    // residual r0 (l times pre-smoothing residual and restriction), into out.
    void level_rhs(int l, const float *r0, float *out, cudaStream_t st);

    int levels() const { return (int)lv_.size(); }
    int level_rows(int l) const { return lv_[l]->n; }
    long level_nnz(int l) const { return l == 0 ? A0_->nnz_true : lv_[l]->A.nnz_true; }
    double omega = 0.8;   // Jacobi weight of the smoother at every level
    double gamma = 1.8;   // scale of the prolonged coarse correction (over-correction)
    float sgn() const { return sgn_; }
    const float *w0() const { return lv_[0]->w.get(); }
    int err_flag(cudaStream_t st);  // nonzero if a bounded wait or the inverse failed
    // the same flag in device memory (0 until set), for reading with other results
    const int *err_dev() const { return err_.get(); }

  private:
    struct View;
    void enqueue_down(int l, const float *r, const int *done, cudaStream_t st);
    void enqueue_up(int l, float *zout, const int *done, cudaStream_t st);
    void enqueue_cycle_to_fine(const float *r, float *z, const int *done, cudaStream_t st);

    const SellDev *A0_ = nullptr;
    const float *val0_32_ = nullptr;
    float sgn_ = 1.0f;
    std::vector<std::unique_ptr<MgLevelDev>> lv_;
    std::vector<SellPattern> hpat_;  // host patterns of levels >= 1 (level 0: empty)
    int nd_ = 0;                    // rows of the dense coarsest level
    DevBuf<float> dinv_;            // coarsest inverse, nd_ x nd_
    DevBuf<float> tmpz_;            // fine-level scratch for apply_fixed / smoother_pair
    DevBuf<float> tmpt_;
    DevBuf<int> err_;
    DevBuf<GridBarrier> gb_;
    int pblocks_ = 0;
};

}  // namespace sysu
