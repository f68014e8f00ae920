/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the subset of the LASPack C API (T. Skalicky, TU Dresden;
 * version unpinned: the library is neither vendored with the reference nor
 * installed here) that the reference solver calls.  It exists so that the
 * reference's own C++ sources can be compiled unmodified into a CPU oracle
 * binary, and it is never linked into the product library.
 *
 * Call sites this header must satisfy (reference file:line):
 *   Q_Constr      navier_velocity.cpp:19, navier_pressure.cpp:15,18,
 *                 navier_scalar.cpp:95,126,262,448, HeatConductionSolver.cpp:52
 *   Q_SetLen / Q_SetEntry   navier_velocity.cpp:340-345, navier_pressure.cpp:186-191,
 *                 navier_scalar.cpp:135-136,634-639, HeatConductionSolver.cpp:275-280
 *   Q_Destr       navier_velocity.cpp:73 and the matching sites above
 *   V_Constr / V_Destr / V_SetAllCmp   navier.cpp:568-573,484-489, navier_pressure.cpp:21
 *   Vector::Cmp[1..Dim]   navier_velocity.cpp:25,33 (1-based component array)
 *   SetRTCAccuracy / GetLastNoIter / GetLastAccuracy   tools.cpp:56-64
 *   CGIter / GMRESIter / SSORPrecond   navier_velocity.cpp:26, navier_pressure.cpp:29,31
 *
 * The algorithms behind these entry points are textbook restatements:
 * CG and BiCGSTAB follow Barrett et al., "Templates for the Solution of
 * Linear Systems" (SIAM 1994), Figs. 2.5 and 2.10; GMRES(m) with right
 * preconditioning and Givens rotations, SSOR and ILU(0) follow Saad,
 * "Iterative Methods for Sparse Linear Systems" (2nd ed., 2003), Algs. 9.5,
 * 4.x and 10.4.  The stopping test is ||b - A x||_2 / ||b||_2 < eps on the
 * unpreconditioned residual recurrence, which is what the reference assumes
 * when it compares GetLastAccuracy() against its tolerance.
 */
#ifndef SYSU_ORACLE_LASPACK_H
#define SYSU_ORACLE_LASPACK_H

#include <stddef.h>
/* BasicSolver.cpp:304,313,382 call sqrt/fabs without including <math.h>;
 * they reach it through this header, so it must be included here. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

typedef double Real;
typedef enum { False = 0, True = 1 } Boolean;
typedef enum { Rowws, Clmws } ElOrderType;
typedef enum { Normal, Tempor } InstanceType;

typedef struct {
    char *Name;
    size_t Dim;
    InstanceType Instance;
    Boolean OwnData;
    Real *Cmp; /* Cmp[1..Dim]; Cmp[0] unused */
} Vector;

typedef struct {
    size_t Pos; /* 1-based column */
    Real Val;
} ElType;

typedef struct {
    char *Name;
    size_t Dim;
    Boolean Symmetry; /* True: only entries with column >= row are given */
    ElOrderType ElOrder;
    InstanceType Instance;
    Boolean OwnData;
    size_t *Len;  /* Len[1..Dim] */
    ElType **El;  /* El[1..Dim][0..Len-1] */
    void *Priv;   /* cached full-CSR view and preconditioner data */
} QMatrix;

typedef Vector *(*PrecondProcType)(QMatrix *, Vector *, Vector *, double);
typedef Vector *(*IterProcType)(QMatrix *, Vector *, Vector *, int, PrecondProcType, double);

void Q_Constr(QMatrix *Q, const char *Name, size_t Dim, Boolean Symmetry,
              ElOrderType ElOrder, InstanceType Instance, Boolean OwnData);
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

Vector *JacobiPrecond(QMatrix *A, Vector *y, Vector *c, double Omega);
Vector *SSORPrecond(QMatrix *A, Vector *y, Vector *c, double Omega);
Vector *ILUPrecond(QMatrix *A, Vector *y, Vector *c, double Omega);

/* ---- oracle-only instrumentation (not part of the LASPack API) ---------- */
typedef struct {
    long calls[3];      /* CG, BiCGSTAB, GMRES */
    long iters[3];
    double seconds[3];  /* wall time spent inside each iterator */
} LaspackOracleStats;
const LaspackOracleStats *laspack_oracle_stats(void);
void laspack_oracle_reset_stats(void);

#endif
