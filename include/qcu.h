/*
 * qcu.h -- drop-in C ABI of the GB300 MRHS Wilson library (libqcu.so).
 *
 * Same symbols, argument meaning and numeric enum values as the reference's
 * include/qcu.h:1-34 (and include/qcu_enum.h:4-12 for the enum values).
 * Every pointer argument is a DEVICE pointer owned by the caller, in the
 * reference's caller layouts (complex double, interleaved re/im):
 *   gauge    [mu=4][parity=2][Vh][N][N], row-major U_ab
 *   fermion  one parity, [Vh][Ns=4][N] spin-major  (Vh = X*Y*Z*T/2)
 *   full fermion (cg_inverter) [2][Vh][4][N], even half first
 * Half-lattice site index i = ((t*Lz + z)*Ly + y)*(Lx/2) + X/2.
 *
 * Errors never terminate the process (the reference calls exit(1),
 * include/qcu_macro.cuh:16-40): the message is printed to stderr in the
 * reference's wording and recorded for qcuGetLastError() (qcu_gb300.h).
 * Setting QCU_ABORT_ON_ERROR=1 in the environment restores exit(1).
 */
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

/* include/qcu.h:7-9 of the reference: lattice extents in X, Y, Z, T order */
typedef struct QcuParam_s {
  int lattice_size[4];
} QcuParam;

/* include/qcu.h:11-15: process grid; every entry must be 1 (one GPU) */
typedef struct QcuGrid_t {
  int grid_size[4];
} QcuGrid_t;

typedef QcuGrid_t QcuGrid;

/* Replaces include/qcu.h:19 / src/qcu.cu:127-135: (re)create the session for
 * one lattice and colour number N (3..8).  Drops any loaded gauge. */
void initGridSize(QcuGrid_t *grid, QcuParam *p_param, int nColors);

/* Replaces include/qcu.h:20 / src/qcu.cu:137-142: queue one RHS pair.
 * fermionIn has parity 1-p and fermionOut parity p of the next startDslash.
 * Nothing is copied until startDslash (no per-RHS allocation). */
void pushBackFermions(void *fermionOut, void *fermionIn);

/* Replaces include/qcu.h:21 / src/qcu.cu:144-149 (Qcu::startDslash at
 * :58-86): apply the hopping term D_parity^f (f = +1, or -1 when daggerFlag
 * is 1) to every queued RHS in one MRHS launch, write each result to its
 * fermionOut, clear the queue.  Synchronous on return. */
void startDslash(int parity, int daggerFlag);

/* Replaces include/qcu.h:22 / src/qcu.cu:162-167 (Qcu::loadGauge :102-109):
 * copy the caller's gauge field into the library's resident layout. */
void loadQcuGauge(void *gauge);

/* Replaces include/qcu.h:24 / src/qcu.cu:152-160: choose the operator.
 * dslashType: 0 = Wilson (1 = clover is rejected, as in the reference);
 * mass -> kappa = 1/(2(4+mass)); floatPrecision: 0 half (FP16 storage with
 * per-site FP32 scales), 1 single, 2 double, 4 bf16 (extension).  Caller
 * buffers stay complex double in every precision. nInputs is a hint. */
void getDslash(int dslashType, double mass, int nColors, int nInputs, int floatPrecision);

/* include/qcu.h:27 (a no-op stub in the reference, src/qcu.cu:170): one
 * even-odd hop, out(parity) = D in(1-parity), SU(3) complex double, with the
 * caller's gauge in caller layout. */
void dslashQcu(void *fermion_out, void *fermion_in, void *gauge, QcuParam *param, int parity);

/* include/qcu.h:28 (a no-op stub in the reference, src/qcu.cu:171): the
 * hopping term on a full even-odd field [2][Vh][4][3]:
 * out_e = D_eo in_o, out_o = D_oe in_e, dagger as in startDslash. */
void fullDslashQcu(void *fermion_out, void *fermion_in, void *gauge, QcuParam *param, int dagger_flag);

/* include/qcu.h:30 (an empty stub in the reference, src/qcu.cu:173): solve
 * M x = b, M = 1 - kappa D, for a full even-odd field (one RHS) to relative
 * true residual p_max_prec, by even-odd preconditioned mixed-precision CG
 * (FP32 inner iterations, FP64 reliable updates).  N is the session's colour
 * number when a session exists, else 3; the boundary condition is the
 * session's (periodic by default). */
void cg_inverter(void *x_vector, void *b_vector, void *gauge, QcuParam *param, double p_max_prec, double p_kappa);

#ifdef __cplusplus
}
#endif
