// The GPU SIMPLE solver: one fluid domain (and optionally one solid domain for
// conjugate heat transfer) resident in device memory, advanced one outer
// iteration at a time in the order of NavierStokesSolver::NSSolve
// (navier.cpp:27-76).
#pragma once

#include <map>
#include <string>
#include <vector>

#include "fv.hpp"
#include "gnn.hpp"

namespace sysu {

// Device copy of a Domain plus its matrix pattern.
struct DomainDev {
    DomView view{};
    int nc = 0, nf = 0, F = 0, B = 0, ncb = 0, nv = 0;
    bool has_outlet = false;
    std::vector<int> int2ref;  // internal face id -> reference face id
    std::vector<int> ref2int;
    SellPattern pat;
    SellDev A;
    DevBuf<double> vol, cx, fn, farea, flam, frl, fx, fxpac, fxnac, fd12, bdist, bquirk, bin, bfixed, vx;
    DevBuf<int> cs_ptr, cs_face, cs_k, fc1, fc2, bcell, btype1, btype2, brid, cw_ptr, cw_b, cvert, vc_ptr, vc_cell;
    DevBuf<int> ss_ptr, ss_w, ss_f, ss_n;
    DevBuf<double> lsq_c;   // least-squares gradient coefficients (option "gradient" 1)
    DevBuf<int> d_int2ref;  // internal face -> reference face (field transfers)
    std::vector<int> h_btype1, h_btype2, h_bcell;
    void build(const Domain &d, const Params &p, cudaStream_t st);
};

// Solver choice per equation (the reference hard-codes them per call site).
enum SolverKind { SK_CG = 0, SK_BICGSTAB = 1, SK_GMRES = 2 };

struct EqOpts {
    int kind = SK_BICGSTAB;
    int maxit = 500;
    double eps = 1e-8;
    double omega = 1.2;
    int mixed = 0;            // FP32 recurrences with FP64 residuals (CG; BiCGSTAB: momentum, k, eps, T)
    double inner_tol = 0.1;   // FP32 residual drop between FP64 residual updates
    int precond = PK_JACOBI;  // PrecondKind (SSOR and ILU with CG and GMRES)
    int restart = 10;         // GMRES restart length
    // CG only (the p' equation): learned preconditioner.  The first learn_iters
    // solves run the plain method and train the network on their
    // residual/correction pairs (learn_steps Adam steps each, rate learn_lr);
    // later solves run flexible CG preconditioned by the network (FP32
    // recurrences, FP64 reliable updates, Jacobi fallback).
    int learned = 0;
    int learn_iters = 20;
    int learn_steps = 64;
    double learn_lr = 1e-3;
    int learn_kind = 1;       // loss: 0 energy norm of the error, 1 residual norm
    // precond PK_AMG: strength threshold of the aggregation, Jacobi weight of the
    // smoother, scale of the prolonged coarse correction
    double mg_theta = 0.25;
    double mg_omega = 0.8;
    double mg_gamma = 1.8;
    int mg_persistent = 0;    // 1: the coarse levels as one persistent cooperative launch
    // learned form with precond PK_AMG: the multigrid level whose post-smoother
    // the network is (0 the finest; deeper than the last coarse level clamps)
    int learn_level = 2;
};

struct SolverOptions {
    // defaults: the reference's call sites (navier_velocity.cpp:26,
    // navier_pressure.cpp:29, navier_scalar.cpp:101,143,374,
    // HeatConductionSolver.cpp:90), with GMRES+SSOR running as
    // BiCGSTAB+Jacobi and CG+SSOR as CG+Jacobi
    // momentum: an FP64 residual of its mixed form costs as much as an FP32
    // iteration (an FP64 product for three right-hand sides), so it is taken once
    // the FP32 residual fell by 1e-4 (2M-cell cavity: 3.1 ms per solve, against
    // 3.4 ms at 1e-3 and 5.1 ms at 0.1)
    EqOpts mom{SK_BICGSTAB, 500, 1e-8, 1.2, 0, 1e-4};
    EqOpts p{SK_CG, 1000, 1e-6, 1.3};
    EqOpts ke{SK_BICGSTAB, 500, 1e-8, 1.3};
    EqOpts t{SK_BICGSTAB, 500, 1e-8, 1.3};
    EqOpts ts{SK_CG, 500, 1e-8, 1.3};
    // the reference's own solver mode: GMRES(10) + SSOR for momentum and scalars,
    // CG + SSOR for p' and solid conduction (option "reference_solvers")
    void reference_solvers() {
        for (EqOpts *e : {&mom, &ke, &t}) {
            e->kind = SK_GMRES;
            e->precond = PK_SSOR;
        }
        for (EqOpts *e : {&p, &ts}) {
            e->kind = SK_CG;
            e->precond = PK_SSOR;
            e->mixed = 0;
        }
        mom_batched = false;
        scalars_batched = false;
    }
    // back to the default (fast) mode: BiCGSTAB + Jacobi, CG + Jacobi, batched momentum
    void default_solvers() {
        for (EqOpts *e : {&mom, &ke, &t}) {
            e->kind = SK_BICGSTAB;
            e->precond = PK_JACOBI;
        }
        for (EqOpts *e : {&p, &ts}) {
            e->kind = SK_CG;
            e->precond = PK_JACOBI;
        }
        mom_batched = true;
    }
    bool mom_batched = true;      // u, v, w as one 3-RHS solve
    // the mixed momentum and multigrid p' solves loop on the device (graph WHILE
    // nodes); false: the host drives them, for per-kernel profiling
    bool graph_loops = true;
    int convection = 0;           // convection of momentum and fluid scalars: 0 the reference's upwind + deferred correction, 1 hybrid
    double solid_source = 0.0;    // W/m^3 (extension; the reference has none)
    bool fatal_checks = true;     // the reference's convergence checks
    bool timing = false;          // CUDA events around the p' solve
    bool profile_phases = false;  // %globaltimer stamps at the CG phase boundaries
    bool output = false;          // nssolve writes tec/res####.dat and tot.dat like the reference
    // k, eps and T assembled from the fields at the start of the scalar stage and
    // solved as one batched BiCGSTAB launch (eps's source and T's conductivity lag
    // the k and eps of this iteration by one outer iteration); needs k-epsilon and
    // energy on, BiCGSTAB for ke and t
    bool scalars_batched = false;
};

enum SolveSlot { SLOT_MOM = 0, SLOT_P, SLOT_K, SLOT_EPS, SLOT_T, SLOT_TS, SLOT_N };

struct FieldSet {
    DevBuf<double> U, V, W, P, R, T, TE, ED, VisLam, VisTur, Apr;
    DevBuf<double> dU, dV, dW, dP, dPhi;
    DevBuf<double> RUFace;
    DevBuf<double> BRo, BU, BV, BW, BPre, BTem, BTE, BED, Bq;
    DevBuf<double> Amom, Ap, As;
    DevBuf<double> b3, bp, bs, x3, xp, xs;
    DevBuf<double> fD, fE, fcoef, bapp, bsrc;
    DevBuf<double> Prod, TESrc, EDSrc, VisTE, VisED, ApTE, ApED, kcond, zeros, src;
    DevBuf<double> tmp3, tmpv;
    DevBuf<double> diff;  // solid conductivity
    DevBuf<double> Unp, Vnp, Wnp, Tnp, TEp, EDp, tapp;  // transient: last step's fields, time-term diagonal
    DevBuf<float> Ap32, As32;  // FP32 copies for mixed-precision solves
    DevBuf<double> As2, As3, bs2, bs3, xs2, xs3;  // eps and T systems of the batched scalar form
};

class SimpleSolver {
  public:
    explicit SimpleSolver(const std::string &param_path);
    ~SimpleSolver();

    Case cs;
    SolverOptions opt;
    cudaStream_t st = nullptr;
    DomainDev fd, sd;
    FieldSet f, s;
    KrylovWork kw;
    GnnPrecond gnn;             // learned p' preconditioner (option p.learned); flexible CG driver
    AggMultigrid mg;            // p' multigrid hierarchy (option p.precond 4)
    double mg_theta_built = 0.0;
    // learned multigrid form with the network on a coarse level: the network
    // bound to that level's matrix, the hierarchy below that level (for the
    // level's own solves that give its training pairs), scratch
    Bicg3Mixed mom3;            // momentum with FP32 recurrences (options mom.mixed + mom_batched)
    bool mom_split = false;     // the last momentum solve left per-component statistics (SLOT_N + c)
    GnnPrecond gnn_c;
    AggMultigrid mg_c;
    int learn_level_built = -1;
    DevBuf<float> mg_r32, mg_rl32;
    DevBuf<double> mg_rl64, mg_el64;
    DevBuf<SolveInfo> mg_info;
    int p_solves = 0;           // p' solves so far (training window of the learned form)
    DevBuf<double> gnn_x1;      // partial solution of a training solve
    DevBuf<double> io_stage;    // staging for reordered field transfers
    DevBuf<SolveInfo> infos;
    DevBuf<double> red_partials, red_out;
    DevBuf<unsigned int> red_ticket;
    DevBuf<int> flags;
    DevBuf<unsigned long long> phase_ts;
    RedScratch rs{};
    int red_blocks = 0;

    double Residual[10] = {0};
    int iter_done = 0;
    SolveInfo last_info[SLOT_N]{};
    double last_p_ms = 0.0;       // CUDA-event time of the last p' solve (opt.timing)
    double last_mom_ms = 0.0;
    cudaEvent_t ev[6]{};

    // NavierStokesSolver::InitFlowField (navier.cpp:113-188) + solid module init
    void init_flow_field();
    // pieces of one outer iteration (enqueued on st, no host sync)
    void calculate_velocity();
    void calculate_pressure();
    void update_ke();
    void update_energy();
    void update_scalars_batched();
    void energy_sources(ScalarArgs &sa);
    // the device work of one outer iteration, enqueued on st without any host
    // synchronisation (capturable into a CUDA graph); outer_iteration() is this
    // plus check_iteration()
    void enqueue_iteration();
    void solid_solve();
    // SaveTransientOldData (navier.cpp:190-240, HeatConductionSolver.cpp:306-327)
    void save_transient_old_data();
    int tscheme() const { return cs.params.steady ? 0 : cs.params.time_scheme; }
    // one NSSolve loop body; syncs once, updates Residual and the solve infos,
    // returns a non-empty message when a reference convergence check fails
    std::string outer_iteration();
    std::string check_iteration();  // read back infos + residuals (one sync)
    // field I/O by reference name (host buffers, reference ordering)
    long field_size(const std::string &name) const;
    int gradient_scheme = 0;  // 0 Green-Gauss (the reference's), 1 least squares
    void set_gradient_scheme(int scheme);
    void get_field(const std::string &name, double *out, long n);
    void set_field(const std::string &name, const double *in, long n);
    void sync();
    // back to the state after InitFlowField (fields, residuals, counters)
    void reset();
    // One application of the p' multigrid cycle as the last p' solve left it
    // (hierarchy, values, the network on its level when use_net), host vectors
    void p_cycle(const double *r, double *z, bool use_net);
    // CUDA events on the solver's stream around a region of work
    void timer_start();
    double timer_stop();  // ms; synchronises
    // Output(): tec/res%04lu.dat in `dir` (numbered by output_counter), and
    // VolumnAverage(t, out_iter): one line of `dir`/tot.dat.
    void output(const std::string &dir);
    void volume_average(const std::string &dir, double t, int out_iter);
    std::string case_dir;       // directory of param.in
    unsigned long output_counter = 0;
    // Standalone SpMV sweep on an assembled matrix ("mom", "p", "scalar", "solid"):
    // mean device time (ms) of one y = A x over `reps` products, FP64 or FP32
    // values, L2 flushed (256 MB write) before each product.
    // Mean device ms of one y = A x of an assembled matrix by the current kernel
    // form: L2 flushed before each of `reps` timed products, or (steady) products
    // back to back alternating between two full copies of the operands
    double spmv_timing(const std::string &which, bool fp32, int reps, bool steady = false);

  private:
    void alloc_fields(FieldSet &fs, const DomainDev &d, bool solid);
    void solve_learned(const EqOpts &o, const double *val, const double *b, double *x, bool x0_zero, SolveInfo *info);

    void solve(int slot, const EqOpts &o, const SellDev &A, const double *val, int nrhs, const double *const *b,
               double *const *x, bool x0_zero);
    void grad_limited(DomainDev &d, FieldSet &fs, int nfield, const double *const *phi, const double *const *Bphi,
                      double *const *grad);
    DevBuf<double> *field_ptr(const std::string &name, int &kind, bool &solid);
};

}  // namespace sysu
