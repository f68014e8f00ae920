// Learned preconditioner for the symmetric pressure-correction systems: a small
// message-passing network over the matrix graph (the cell-face graph), BF16
// weights with FP32 accumulation on the tensor cores, used inside flexible CG,
// trained on the GPU from residual/correction pairs that the solver produces.
//
// Network (width 32, four message-passing layers), for a residual r:
//   s      = sqrt(mean((D^-1 r)^2))                       scale (the map is scale-equivariant)
//   u_i    = (D^-1 r)_i / s
//   w_ij   = a_ij / a_ii                                   edge weights (row-scaled off-diagonals)
//   h0_i   = u_i e + c                                     encoder (e, c in R^32)
//   m^l_i  = sum_{j != i} w_ij h^{l-1}_j                  aggregation over the row's neighbours
//   h^l_i  = h^{l-1}_i + relu(W_l^T [h^{l-1}_i ; m^l_i] + b_l)     l = 1..4, W_l 64 x 32
//   z_i    = s (k u_i + w_d . h4_i + b_d)                  decoder (Jacobi plus a learned correction)
// With w_d = b_d = 0 the network is exactly the Jacobi preconditioner (k = 1),
// or the weighted-Jacobi smoothing step of the multigrid cycle (k = omega).
// Activations h, m are stored in BF16; the 64 x 32 dense products run as
// tcgen05 MMAs (M = 128 rows per tile).
//
// Loss of one pair (r, e = A^-1 r): the energy norm of the error,
//   L = (z - e)^T S (z - e) / e^T S e,   S = sgn A positive definite,
// or (loss_kind 1) the residual norm ||S (z - e)||^2 / ||S e||^2.
#pragma once

#include <cstdint>
#include <vector>

#include "amg.hpp"
#include "krylov.hpp"

namespace sysu {

constexpr int GNN_WIDTH = 32;
constexpr int GNN_LAYERS = 4;
constexpr int GNN_LAYER_STRIDE = 64 * 32 + 32;  // W[64 in][32 out], then b[32]
constexpr int GNN_OFF_ENC = 0;                  // e[32], c[32]
constexpr int GNN_OFF_LAYER = 64;
constexpr int GNN_OFF_DEC = GNN_OFF_LAYER + GNN_LAYERS * GNN_LAYER_STRIDE;  // w_d[32], b_d
constexpr int GNN_NPARAM = GNN_OFF_DEC + 33;
constexpr int GNN_NPARAM_PAD = 8448;  // per-CTA gradient record
constexpr int GNN_WBF_LAYER = 4096;   // BF16 copies per layer: Wt[32][64], W[64][32]

// Scalars of one flexible-CG solve (device memory).
struct FcgState {
    double bnorm2, eps2, rr, rr_upd, rr_best, ss;
    double zq, pq, pq_prev, pr, alpha;
    double res;
    int iters, refinements, done, status, use_gnn, stall, restart, need_update, fallback_at, maxit;
    int loops;  // graph loop: bodies run (the loop's bound)
    float inv_s, s;
    float inv_s2, s2;  // multigrid form: scale of the post-smoother's input
    unsigned cnt[4];
};

struct GnnScalars {  // training / apply scalars (device memory)
    double loss_num, loss_den;
    float inv_s, s;
    unsigned cnt[4];
};

class GnnPrecond {
  public:
    GnnPrecond() = default;
    GnnPrecond(const GnnPrecond &) = delete;
    GnnPrecond &operator=(const GnnPrecond &) = delete;
    ~GnnPrecond();
    // Attach to a symmetric SELL matrix (FP64 values and their FP32 copy, both
    // owned by the caller and kept alive); sizes the work buffers for it.
    void bind(const SellDev &A, const double *val64, const float *val32, cudaStream_t st);
    bool bound() const { return A_ != nullptr; }
    // The bound matrix's values changed (same pattern, same buffers): recompute
    // the diagonal inverse the network and the solver use.
    void refresh(cudaStream_t st);
    int n() const { return n_; }

    void init_params(unsigned long long seed, cudaStream_t st);
    void set_params(const float *host, cudaStream_t st);
    void get_params(float *host, cudaStream_t st);
    void reset_adam(cudaStream_t st);

    // z = M(r) (FP64 device vectors, converted to FP32 inside).
    void apply(const double *r, double *z, cudaStream_t st);

    // device time of one network application (ms), averaged over reps
    double time_apply(const double *r, int reps, cudaStream_t st);
    int fwd_per_sm = 0;   // forward CTAs per SM (0: from registers and shared memory); applied at bind
    // Weight of the Jacobi term in the decoder, z = s (skip u + w_d . h4 + b_d):
    // 1 as a whole preconditioner; the smoother's omega as a multigrid
    // post-smoother, so that the untrained network (zero decoder) is exactly the
    // cycle's Jacobi post-smoothing step and training learns a correction to it.
    float skip = 1.0f;

    // Training pairs: a ring of `capacity` FP32 pairs.
    void set_capacity(int pairs) { capacity_ = pairs; }
    void add_pair(const double *r, const double *e, cudaStream_t st);
    // pair of a partial solve x1 of A x = b with solution xs: (b - A x1, xs - x1);
    // x1 == nullptr gives (b, xs)
    void add_pair_from(const double *b, const double *x1, const double *xs, cudaStream_t st);
    int newest_pair() const { return (next_ + capacity_ - 1) % capacity_; }
    int pairs() const { return count_; }
    void clear_pairs() { count_ = 0; next_ = 0; }
    // One Adam step on pair k; the loss lands in losses()[step index] (device).
    void train_step(int k, double lr, cudaStream_t st);
    // Loss and full parameter gradient of pair k without an update.
    void loss_grad(int k, double *loss, float *grad_host, cudaStream_t st);
    int loss_kind = 0;
    int steps() const { return adam_t_; }
    void last_losses(std::vector<double> &out, int count, cudaStream_t st);
    // Forward with stored activations on r (FP64 device vector); h^layer
    // (layer 1..4) as FP32 [n][32] to the host.
    void hidden(const double *r, int layer, float *host, cudaStream_t st);

    // Multigrid form: with a hierarchy attached (built for the bound matrix and
    // refreshed with its values by the caller), the preconditioner of fcg() is
    // the aggregation-multigrid V-cycle, whose finest post-smoothing step is the
    // network applied to the residual t = r - A z2 after pre-smoothing and
    // coarse correction (use_gnn), or Jacobi.  Training pairs added while a
    // hierarchy is attached are turned into pairs of that post-smoother,
    // (r, e) -> (r - A z2(r), e - z2(r)).  nullptr detaches.
    void attach_multigrid(AggMultigrid *mg);
    AggMultigrid *multigrid() const { return mg_; }
    // z = M(r) of the attached cycle once (FP64 device vectors): z2 + N(t) with
    // the network (use_gnn), z2 + w t (Jacobi) without.
    void apply_mg(const double *r, double *z, bool use_gnn, cudaStream_t st);
    // Level of the attached cycle whose post-smoother the network is: 0 the
    // finest (this handle's own network), >= 1 a coarse level, whose network is
    // another handle bound to that level's matrix and called through the
    // cycle's post_hook (this handle's finest post-smoothing is then Jacobi).
    int net_level = 0;
    // As the network of a coarse level (this handle bound to that level's
    // matrix): z = zp + N(r - A zp) while fs->use_gnn, else the Jacobi step
    // zp + w (r - A zp); fs is the finest-level flexible CG's state.
    void post_smooth(const float *r, const float *zp, float *z, FcgState *fs, const float *w, cudaStream_t st);
    FcgState *fcg_state() { return fs_.get(); }
    // r = b - A x1 in FP32 (x1 == nullptr: r = b), FP64 device vectors in
    void residual32(const double *b, const double *x1, float *r, cudaStream_t st);

    // Flexible CG (Notay's FCG(1)) with FP32 recurrences and FP64 reliable
    // updates, preconditioned by the network (use_gnn) or by Jacobi -- or by
    // the multigrid cycle, with or without the network, when one is attached;
    // when the network fails to reduce the residual for `stall_max` iterations,
    // or a direction loses positivity, the same preconditioner without the
    // network takes over for the rest of the solve.
    // Stops on the FP64 residual ||b - A x|| / ||b|| < eps.  The iterations are
    // the body (check_every of them) of a CUDA graph WHILE node, so the solve
    // never waits for the host: on a stream being captured it joins the
    // caller's graph, otherwise it runs as its own graph (graph_loop.hpp).
    void fcg(const double *b, double *x, bool x0_zero, const KrylovOpts &o, bool use_gnn, SolveInfo *info_dev,
             cudaStream_t st);
    int stall_max = 30;
    int check_every = 8;
    // false: the host drives the iterations (a captured chunk of check_every
    // iterations, `done` read after each) -- for per-kernel profiling; profilers
    // skip the kernels of graphs with conditional nodes
    bool device_loop = true;
    FcgState last_state(cudaStream_t st);

  private:
    void forward(const float *r32, float *z32, bool train, FcgState *fs, const float *qprev, cudaStream_t st,
                 const float *zbase = nullptr);
    void backward(const float *r32, cudaStream_t st);
    void refresh_bf16(cudaStream_t st);
    void scale_of(const float *r32, cudaStream_t st);
    void check_err(cudaStream_t st);
    void fcg_iteration(const void *args, bool use_gnn, cudaStream_t st);

    // A whole flexible-CG solve captured as a graph (its iterations a WHILE
    // node, graph_loop.hpp), for streams that are not capturing; the four most
    // recent argument sets (the bytes of everything the capture bakes in) are kept.
    struct SolveGraph {
        cudaGraphExec_t exec = nullptr;
        long launches = 0;
        std::vector<unsigned char> key;
    };
    SolveGraph graphs_[4];
    int graph_next_ = 0;
    void drop_graphs();
    void transform_pair(int k, cudaStream_t st);

    AggMultigrid *mg_ = nullptr;
    DevBuf<float> z2_, t_;      // multigrid form: fixed part of the cycle and its residual

    const SellDev *A_ = nullptr;
    const double *val64_ = nullptr;
    const float *val32_ = nullptr;
    int n_ = 0, ntiles_ = 0, gtiles_ = 0, gfwd_ = 0, gflat_ = 0;
    float sgn_ = 1.0f;
    int capacity_ = 32, count_ = 0, next_ = 0, adam_t_ = 0;

    DevBuf<float> dinv_;
    DevBuf<float> p_, m_, v_;   // FP32 parameters and Adam moments
    DevBuf<uint16_t> wbf_;      // BF16 weights, GNN_WBF_LAYER per layer
    DevBuf<float> rec_;         // per-CTA gradient records
    DevBuf<uint16_t> H_, M_;    // activations [5][n][32], [4][n][32]
    DevBuf<uint32_t> mask_;     // [4][n]
    DevBuf<float> aw_;          // [n][2] layer-1 aggregates
    DevBuf<float> dA_, gA_, dB_, gB_;  // backward ping-pong [n][32]
    DevBuf<float> z32_, y32_, r32_, e32_, p32_, q32_, x32_;
    DevBuf<float> pr_, pe_;     // pair ring [capacity][n]
    DevBuf<double> part_, r64_, b64_, x64_;
    DevBuf<double> losses_;
    DevBuf<GnnScalars> sc_;
    DevBuf<FcgState> fs_;
    DevBuf<int> err_;
};

}  // namespace sysu
