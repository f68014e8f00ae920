/*
 * laspack/laspack.h -- LASPack-compatible C ABI backed by the GPU Krylov
 * solvers of libsysucfd.so.
 *
 * A drop-in for the reference's `extern "C" { #include "laspack/laspack.h" }`
 * (reference src/BasicType.h:11-13, src/navier.h:6-8, src/tools.h:10-12,
 * src/navier_velocity.cpp:5-7).  It declares exactly the subset of LASPack
 * (T. Skalicky, TU Dresden; the reference does not pin a version) that the
 * reference calls; signatures follow those call sites:
 *   Q_Constr / Q_SetLen / Q_SetEntry / Q_Destr   navier_velocity.cpp:19,340-345,73;
 *       navier_pressure.cpp:15-18,186-191; navier_scalar.cpp:95,126,135-136,262;
 *       HeatConductionSolver.cpp:52,275-280
 *   V_Constr / V_Destr / V_SetAllCmp, Vector::Cmp[1..Dim]   navier.cpp:568-573,
 *       navier_pressure.cpp:21, navier_velocity.cpp:25,33
 *   SetRTCAccuracy / GetLastNoIter / GetLastAccuracy        tools.cpp:56-64
 *   CGIter / GMRESIter / BiCGSTABIter, SSORPrecond / JacobiPrecond / ILUPrecond
 *
 * Semantics kept from LASPack as the reference uses it: 1-based rows, columns
 * and vector components; a symmetric matrix receives its upper triangle only;
 * Q_SetLen on an assembled row replaces the row; the iterators stop when
 * ||b - A x||_2 / ||b||_2 < eps (SetRTCAccuracy) or after MaxIter iterations,
 * and GetLastNoIter / GetLastAccuracy report the last solve.
 *
 * GPU specifics: vectors stay in host memory (the caller reads and writes
 * Cmp[] directly); each iterator call uploads A (values only when the pattern
 * is unchanged), b and x, runs one persistent GPU solve and downloads x.
 * CGIter, BiCGSTABIter and GMRESIter (restarted, SetGMRESRestart, default 10,
 * at most 30) run those methods; JacobiPrecond, SSORPrecond and ILUPrecond
 * (ILU(0)) run as given, the triangular sweeps level-scheduled in natural row
 * order, except that BiCGSTABIter applies Jacobi in place of SSOR/ILU.
 * laspack_gpu_set_mode() can substitute BiCGSTAB for GMRES and Jacobi for
 * SSOR/ILU (faster, same solution to the tolerance); a substitution is reported
 * once on stderr.  Any other preconditioner function is refused.  The environment variable SYSU_LASPACK_RTC, when set, replaces
 * the tolerance of every solve (for tight-tolerance comparisons).  Nothing here falls back to the CPU: without a GPU an iterator
 * leaves x unchanged and reports accuracy +inf, which the reference's own
 * checks treat as a failed solve.
 */
#ifndef SYSU_LASPACK_GPU_H
#define SYSU_LASPACK_GPU_H

#include <stddef.h>
/* the reference reaches sqrt/fabs through this header (BasicSolver.cpp:304,313) */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double Real;
typedef enum { False = 0, True = 1 } Boolean;
typedef enum { Rowws, Clmws } ElOrderType;
typedef enum { Normal, Tempor } InstanceType;

typedef struct {
    char *Name;
    size_t Dim;
    InstanceType Instance;
    Boolean OwnData;
    Real *Cmp; /* Cmp[1..Dim] */
} Vector;

typedef struct {
    size_t Pos;
    Real Val;
} ElType;

typedef struct {
    char *Name;
    size_t Dim;
    Boolean Symmetry;
    ElOrderType ElOrder;
    InstanceType Instance;
    Boolean OwnData;
    size_t *Len;
    ElType **El;
    void *Priv; /* device-side cache */
} QMatrix;

typedef Vector *(*PrecondProcType)(QMatrix *, Vector *, Vector *, double);

void Q_Constr(QMatrix *Q, const char *Name, size_t Dim, Boolean Symmetry, ElOrderType ElOrder,
              InstanceType Instance, Boolean OwnData);
void Q_Destr(QMatrix *Q);
void Q_SetLen(QMatrix *Q, size_t RoC, size_t Len);
void Q_SetEntry(QMatrix *Q, size_t RoC, size_t Entry, size_t Pos, Real Val);

void V_Constr(Vector *V, const char *Name, size_t Dim, InstanceType Instance, Boolean OwnData);
void V_Destr(Vector *V);
void V_SetAllCmp(Vector *V, Real C);

void SetRTCAccuracy(double NewEps);
int GetLastNoIter(void);
double GetLastAccuracy(void);
void SetGMRESRestart(int MaxSteps);

Vector *CGIter(QMatrix *A, Vector *x, Vector *b, int MaxIter, PrecondProcType Precond, double Omega);
Vector *BiCGSTABIter(QMatrix *A, Vector *x, Vector *b, int MaxIter, PrecondProcType Precond, double Omega);
Vector *GMRESIter(QMatrix *A, Vector *x, Vector *b, int MaxIter, PrecondProcType Precond, double Omega);

/* Apply y = M^-1 c on the host (for callers that use a preconditioner
 * directly); the iterators recognise these addresses and run the GPU kernels. */
Vector *JacobiPrecond(QMatrix *A, Vector *y, Vector *c, double Omega);
Vector *SSORPrecond(QMatrix *A, Vector *y, Vector *c, double Omega);
Vector *ILUPrecond(QMatrix *A, Vector *y, Vector *c, double Omega);

/* ---- extensions (not LASPack) ------------------------------------------- */
/* gmres_as: 0 = GMRES (default), 1 = BiCGSTAB; ssor_as: 0 = SSOR/ILU as named
 * (default), 1 = Jacobi.  Returns 0. */
int laspack_gpu_set_mode(int gmres_as, int ssor_as);
/* solves run through this ABI and the GPU iterations they took */
long laspack_gpu_solves(void);
long laspack_gpu_iterations(void);

#ifdef __cplusplus
}
#endif

#endif
