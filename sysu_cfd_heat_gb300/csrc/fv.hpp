// Device views of one finite-volume domain and the kernel launchers that
// implement the SIMPLE hot path.  Views are plain structs of device pointers
// passed by value to kernels.
//
// Face numbering on the device ("internal" order): interior faces first, in
// the reference's relative order, then one face per boundary record, in
// boundary-record order (face F+b belongs to record b).  The permutation to
// the reference's face ids is kept for field input/output.
//
// Vectors of 3-vectors are stored structure-of-arrays: component c of item i
// at [c*n + i].
#pragma once

#include "krylov.hpp"

namespace sysu {

struct DomView {
    int nc, nf, F, B, ncb;       // cells, faces, interior faces, boundary records, first coupled record
    // cells
    const double *vol, *cx;      // cx: 3*nc
    const int *cs_ptr;           // nc+1 (slots = reference Cell[i].face[j] order)
    const int *cs_face;          // internal face id of each slot
    const int *cs_k;             // interior slot: position k >= 1 in the matrix row; boundary slot: record b
    // the same slots in SELL-32 layout (slice of 32 cells, column-major, padded
    // to the slice's widest cell): slot j of cell i at ss_ptr[i/32] + 32 j + i%32.
    // ss_f: internal face id (-1 = padding); ss_n: neighbour cell (bit 31 set when
    // the cell is the face's cell2) or, for a boundary slot, SS_BND | record
    const int *ss_ptr, *ss_w, *ss_f, *ss_n;
    int ss_tot;                  // slots stored (the component stride of lsq_c)
    // least-squares gradients (option "gradient" 1; null: Green-Gauss): per slot
    // the vector c_j = M^-1 w_j d_j (3 * ss_tot, SoA), so grad = sum_j c_j (phi_j - phi_c)
    const double *lsq_c;
    // faces
    const int *fc1, *fc2;        // fc2 < 0 on boundary faces
    const double *fn, *farea, *flam, *frl, *fx;  // fn, fx: 3*nf
    const double *fxpac, *fxnac; // 3*F
    const double *fd12;          // F: |Xnac - Xpac| (geometric, precomputed: saves an FP64 sqrt per face)
    // boundary records
    const int *bcell, *btype1, *btype2, *brid;
    const double *bdist;
    const double *bquirk_area;   // area of reference face id b (navier_bc.cpp:72 reads Face[i])
    // per-record inlet values (region initvalues) and fixed values
    const double *bin;           // 8*B: u v w p r t te ed (SoA)
    const double *bfixed;        // B
    // cell -> wall boundary records (type1 == 1), ascending record order
    const int *cw_ptr, *cw_b;
    // vertices (limiters)
    int nv;
    const double *vx;            // 3*nv
    const int *cvert;            // 8*nc (SoA: [k*nc + i])
    const int *vc_ptr, *vc_cell; // vertex -> cells
    // matrix pattern
    SellView A;                  // val filled per equation
};

constexpr int SS_C2 = (int)0x80000000u;
constexpr int SS_BND = 0x40000000;

// Launch configuration shared by the FV kernels.
constexpr int FV_BLOCK = 256;

// Reduction scratch: per-block partials and the final values, plus a ticket.
struct RedScratch {
    double *partials;   // NSLOT * max_blocks
    double *out;        // NSLOT
    unsigned int *ticket;
    int max_blocks;
};

enum RedSlotId {
    RED_MASS_IN = 0, RED_MASS_OUT, RED_AREA_OUT,   // SetBCVelocity sums
    RED_RES0, RED_RES1, RED_RES2, RED_RES3,        // Residual[0..3]
    RED_HEAT_F, RED_HEAT_S,                        // interface heat balance
    RED_MISC0, RED_MISC1, RED_MISC2,
    RED_NSLOT
};

// ---- kernels (fv.cu) ------------------------------------------------------
// SetBCVelocity, navier_bc.cpp:8-108 (density model 0: outlet mass rescaling)
void launch_bc_velocity(const DomView &d, const double *R, const double *U, const double *V, const double *W,
                        double *BRo, double *BU, double *BV, double *BW, bool has_outlet, RedScratch rs,
                        cudaStream_t st);
// Green-Gauss gradient (BasicSolver.cpp:29-63) of 1, 3 or 4 fields with
// boundary values Bphi[k].
// Coefficients of the least-squares gradient (lsq_c of DomView) from the geometry:
// d_j = x_j - x_c (x_j the neighbour's centroid, or the boundary face's), w_j =
// 1 / |d_j|^2, M = sum_j w_j d_j d_j^T, c_j = M^-1 w_j d_j; cells whose M is
// singular get c_j = 0 (zero gradient).
void launch_lsq_setup(const DomView &d, double *lsq_c, cudaStream_t st);
void launch_gradient(const DomView &d, int nfield, const double *const *phi, const double *const *Bphi,
                     double *const *grad, cudaStream_t st);
// Limiters (BasicSolver.cpp:118-288) applied in place to grad of phi.
void launch_limiter(const DomView &d, int limiter, const double *phi, double *grad, double *tmp3,
                    double *tmp_v, cudaStream_t st);

struct MomArgs {
    const double *U, *V, *W, *R, *VisLam, *VisTur, *RUFace, *dU, *dV, *dW, *dP;
    const double *BU, *BV, *BW;
    double urf;
    double g[3];
    double *fD, *fE;       // per interior face: D, E (3*F)
    double *bapp, *bsrc;   // per boundary record: diag part, explicit source (3*B)
    double *val;           // matrix values (SELL)
    double *bu, *bv, *bw;  // right-hand sides
    double *Apr;
    int *flags;            // error flags (e.g. unknown boundary type)
    // transient terms (navier_velocity.cpp:103-118): tscheme 0 steady, 1 Euler,
    // 2 "Dual" (BDF2 with the reference's old levels, both equal to the last step)
    const double *Unp = nullptr, *Vnp = nullptr, *Wnp = nullptr;
    double dt = 0.0;
    int tscheme = 0;
    // convection of interior faces: 0 the reference's implicit upwind with deferred
    // correction to linear upwind (navier_velocity.cpp:255-295); 1 hybrid (Spalding):
    // a_nb = max(-F, D - F/2, 0) with F the face's outward mass flux, no deferred
    // correction (an option; the reference has no hybrid scheme)
    int hybrid = 0;
};
// BuildVelocityMatrix, navier_velocity.cpp:77-357
void launch_momentum(const DomView &d, const MomArgs &a, cudaStream_t st);

// L1 change residual and commit: res += sum |old - new| * vol, old = new
// (navier_velocity.cpp:31-34).  3 fields at once (slots RED_RES0..2).
void launch_commit3(const DomView &d, double *U, double *V, double *W, const double *x3, RedScratch rs,
                    cudaStream_t st);

struct PresArgs {
    const double *U, *V, *W, *R, *P, *dP, *Apr;
    const double *BRo, *BU, *BV, *BW;
    double *RUFace;        // out: Rhie-Chow flux (internal face order)
    double *fcoef;         // out: (rho Apr)_f vol_f rlencos per interior face
    double *val, *bp;      // p' matrix (full storage) and right-hand side
    // density model 1 (perfect gas, navier_pressure.cpp:96-100,118-133,165-181):
    // compressibility terms; the matrix is then not symmetric
    int density_model;
    const double *T;
    double rcpcv;
    int transient;
    double dt;
};
// CalRUFace2 (navier_velocity.cpp:389-442) + BuildPressureMatrix (navier_pressure.cpp:78-198)
void launch_pressure_assembly(const DomView &d, const PresArgs &a, cudaStream_t st);

struct CorrArgs {
    const double *dp, *dPdp;   // p' and its gradient
    const double *Apr;
    double *R;                 // corrected for density model 1 (navier_pressure.cpp:45-48)
    double *P, *U, *V, *W;
    double urf_p;
    int cell_ref;
    int density_model;
    const double *T;
    double rcpcv;
};
// navier_pressure.cpp:38-56: Residual[3], pressure and velocity correction
void launch_correct_cells(const DomView &d, const CorrArgs &a, RedScratch rs, cudaStream_t st);
// CorrectRUFace2, navier_pressure.cpp:200-242 (density model 0)
// (the face coefficient of the p' assembly, fcoef, is reused: Apr and rho are unchanged)
// Density model 1: the face coefficient is recomputed from the corrected density
// and the flux gains the rho' u term (navier_pressure.cpp:225-234).
void launch_correct_faces(const DomView &d, const double *dp, const double *dPdp, const double *R,
                          const double *Apr, const double *BRo, const double *BU, const double *BV,
                          const double *BW, double urf_p, double *RUFace, const double *fcoef, int density_model,
                          const double *T, double rcpcv, cudaStream_t st);
// Viscous work source of the energy equation for density model 1
// (navier_scalar.cpp:277-338): src[i] += sum over i's faces of +-fvis_f.
void launch_energy_viscous(const DomView &d, const double *VisLam, const double *VisTur, const double *dU,
                           const double *dV, const double *dW, const double *U, const double *V, const double *W,
                           double cp, double *src, cudaStream_t st);
// Field transfer helpers: dst[i] = src[idx[i]] / dst[idx[i]] = src[i], and the
// [k*n + i] <-> [3 i + k] reshuffle of the gradient fields.
void launch_gather(double *dst, const double *src, const int *idx, int n, cudaStream_t st);
void launch_scatter(double *dst, const double *src, const int *idx, int n, cudaStream_t st);
void launch_aos3_to_soa3(double *dst, const double *src, int n, cudaStream_t st);
void launch_soa3_to_aos3(double *dst, const double *src, int n, cudaStream_t st);
// Bphi[b] = phi(cell of b) for every record: SetBCPressure / SetBCDeltaP (navier_bc.cpp:110-162)
void launch_bnd_from_cell(const DomView &d, const double *phi, double *Bphi, cudaStream_t st);

// Generic scalar transport assembly (navier_scalar.cpp:466-647,
// HeatConductionSolver.cpp:175-288).
enum ScalarBc { SC_FLUID_PLAIN = 0, SC_FLUID_ENERGY = 1, SC_SOLID = 2 };
struct ScalarArgs {
    const double *phi, *Bphi, *diff, *src, *app0, *grad, *RUFace, *Bq;
    double urf;
    int bc_mode;           // ScalarBc
    double *fD, *fE;       // interior face scratch (fE: F)
    double *bapp, *bsrc;   // boundary scratch
    double *val, *b;
    int *flags;
    int hybrid = 0;        // convection of interior faces: see MomArgs::hybrid
};
void launch_scalar(const DomView &d, const ScalarArgs &a, cudaStream_t st);

// k-epsilon pieces (navier_scalar.cpp:36-67,116-161; navier_bc.cpp:209-296)
struct KeArgs {
    const double *dU, *dV, *dW, *R, *VisLam, *U, *V, *W;
    double *TE, *ED, *VisTur;
    double *Prod, *TESrc, *EDSrc, *VisTE, *VisED, *ApTE, *ApED;
    double *BTE, *BED;
};
void launch_ke_sources(const DomView &d, const KeArgs &a, cudaStream_t st);      // per cell + wall functions
void launch_ke_bnd_values(const DomView &d, const KeArgs &a, cudaStream_t st);   // inlet/outlet/sym BTE, BED
void launch_ke_eps_sources(const DomView &d, const KeArgs &a, cudaStream_t st);  // after k is solved
void launch_ke_eps_wall_rows(const DomView &d, const double *ED, double *val, double *b, cudaStream_t st);
void launch_clip_max(double *dst, const double *src, double lo, int n, cudaStream_t st);
void launch_visc_tur(int n, const double *R, const double *TE, const double *ED, double *VisTur, cudaStream_t st);

// energy (navier_scalar.cpp:257-397, navier_bc.cpp:164-203, HeatConductionSolver.cpp:13-44,373-427)
void launch_kcond(int n, const double *VisLam, const double *VisTur, double cp, double prl, double prte,
                  double *kcond, cudaStream_t st);
void launch_bc_temperature_fluid(const DomView &d, const double *T, double *BTem, cudaStream_t st);
void launch_bc_temperature_solid(const DomView &d, const double *T, const double *diff, const double *Bq,
                                 double *BTem, cudaStream_t st);
// solid -> fluid: fluid BTem of coupled record k = T_s + grad T_s . (x_f - x_c)
void launch_cht_solid2fluid(const DomView &s, const double *Ts, const double *gTs, const DomView &f,
                            double *BTem_f, cudaStream_t st);
// fluid -> solid: q_f = -k grad T_f . n / |S|, q_s = -q_f
void launch_cht_fluid2solid(const DomView &f, const double *gTf, const double *kcond, double *Bq_f,
                            const DomView &s, double *Bq_s, cudaStream_t st);

void launch_fill(double *x, double v, int n, cudaStream_t st);
// Transient term of a cell equation (navier_scalar.cpp:72-89,350-366,
// HeatConductionSolver.cpp:66-80): coef = R/dt * vol; Euler: app += coef,
// src += coef phi_old; scheme 2: app += 1.5 coef, src += coef (2 phi_old - 0.5 phi_old2)
// with phi_old2 = phi_old (SaveTransientOldData sets both levels to the last step).
void launch_time_term(int n, const double *R, const double *vol, double dt, int scheme, const double *phi_old,
                      double *app, double *src, cudaStream_t st);
void launch_copy(double *dst, const double *src, int n, cudaStream_t st);
void launch_scale_src(double *dst, const double *vol, double q, int n, cudaStream_t st);  // dst = q*vol

// Reset the reduction slots and tickets.
void red_reset(RedScratch rs, cudaStream_t st);

}  // namespace sysu
