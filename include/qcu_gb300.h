/*
 * qcu_gb300.h -- extensions of the drop-in ABI in qcu.h.
 *
 * None of these has a counterpart in the reference unless a line says so;
 * they expose what the reference's C ABI hides or lacks: an error status, the
 * boundary condition, explicit streams, device-resident MRHS fields (no
 * per-call layout transform), the layout transforms themselves, the Krylov
 * solvers and the kernel autotuner.
 *
 * Every function returns 0 (QCU_OK) or one of the QCU_ERR_* codes below and
 * records the error for qcuGetLastError().  Pointers are device pointers.
 *
 * Internal MRHS field of one parity (for the session lattice and N):
 *   data  [4N][Vh][nrhs] complex in the field precision (component-major,
 *         RHS innermost)
 *   norm  [Vh][nrhs] float, present only for FP16 storage; stored values
 *         are component / norm(site, rhs).  BF16 has the FP32 exponent range
 *         and is stored unscaled (no norm array; norm pointers are ignored).
 * Sizes come from qcuFieldBytes.  Buffers must be 16-byte aligned.
 */
#pragma once

#include <stddef.h>

#include "qcu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
typedef enum QcuStatus_e {
  QCU_OK = 0,
  QCU_ERR_NOT_INITIALIZED = 1,
  QCU_ERR_INVALID_ARGUMENT = 2,
  QCU_ERR_UNSUPPORTED = 3,
  QCU_ERR_CUDA = 4,
  QCU_ERR_NO_GAUGE = 5,
  QCU_ERR_NO_OPERATOR = 6,
  QCU_ERR_NOT_CONVERGED = 7,
  QCU_ERR_BREAKDOWN = 8,
  QCU_ERR_DEVICE_TIMEOUT = 9,
  QCU_ERR_OUT_OF_MEMORY = 10,
  QCU_ERR_CAPACITY = 11
} QcuStatus;

/* precision codes: the reference's QCU_PRECISION values
 * (include/qcu_enum.h:4 of the reference) plus BF16 */
#ifndef QCU_ENUM_H_INCLUDED /* C++ callers of qcu_enum.h have these as enumerators */
#define QCU_HALF_PRECISION 0
#define QCU_SINGLE_PRECISION 1
#define QCU_DOUBLE_PRECISION 2
#endif
#define QCU_BF16_PRECISION 4
/* BF16 storage in the site-major layout: resident fields [Vh][4N][nrhs]
 * (every other code is component-major, [4N][Vh][nrhs]).  The dslash on
 * these fields is the tensor-core kernel, which copies one site's whole
 * block as one contiguous operand tile: nrhs a multiple of 4, N = 2..8, no
 * clover term.  Accepted by pack/unpack, qcuDslashMRHS / qcuDslashXpayMRHS,
 * qcuTuneDslash, qcuDslashKernels and as a solver inner precision. */
#define QCU_BF16_SITE_PRECISION 5

/* caller fermion address modes for pack/unpack */
#define QCU_SRC_EO_HALF 0 /* one parity [Vh][4][N] */
#define QCU_SRC_EO_FULL 1 /* [2][Vh][4][N]; parity selects the half */
#define QCU_SRC_LEX 2     /* lexicographic full field [V][4][N] */

/* solvers */
#define QCU_SOLVER_CG 0       /* CG on Mhat^dag Mhat, Mhat = 1 - kappa^2 D_eo D_oe */
#define QCU_SOLVER_BICGSTAB 1 /* BiCGStab on Mhat */

int qcuGetLastError(void);
const char *qcuGetLastErrorString(void);
void qcuClearError(void);
const char *qcuVersion(void);

/* 1 = antiperiodic time boundaries (every hop across t = Lt-1 <-> 0 is
 * multiplied by -1), 0 = periodic (the reference's only mode). */
int qcuSetAntiperiodicT(int flag);
/* Run library work on this cudaStream_t (NULL: the library's own stream).
 * ABI calls still synchronise before returning. */
int qcuSetStream(void *stream);
int qcuSynchronize(void);

/* bytes of one internal MRHS field of one parity */
int qcuFieldBytes(int precision, int nrhs, size_t *data_bytes, size_t *norm_bytes);

/* caller FP64 fermions -> internal MRHS field (one launch for all RHS) */
int qcuPackFermions(void *dst, void *dst_norm, void *const *src, int nrhs, int src_mode, int parity, int precision);
/* internal MRHS field -> caller FP64 fermions */
int qcuUnpackFermions(void *const *dst, const void *src, const void *src_norm, int nrhs, int dst_mode, int parity,
                      int precision);

/* load a lexicographic gauge field [4][V][N][N] (complex double) */
int qcuLoadGaugeLex(void *gauge_lex);
/* lexicographic [V][ncomp] <-> even-odd [2][Vh][ncomp] complex double */
int qcuLexToEo(void *eo_out, const void *lex_in, int ncomp);
int qcuEoToLex(void *lex_out, const void *eo_in, int ncomp);

/* out = D_parity^f in on resident MRHS fields; precision as in getDslash
 * (the session gauge is converted to it once).  Asynchronous on the
 * library stream. */
int qcuDslashMRHS(void *out, void *out_norm, const void *in, const void *in_norm, int nrhs, int parity, int dagger,
                  int precision);
/* out = a * D_parity^f in + b * x  (the reference's DslashXpay stub,
 * include/qcu_dirac.h:49) */
int qcuDslashXpayMRHS(void *out, void *out_norm, const void *in, const void *in_norm, const void *x,
                      const void *x_norm, int nrhs, int parity, int dagger, int precision, double a, double b);

/* Clover term A of the Wilson-clover operator M = A - kappa D.  The
 * reference reserves DSLASH_CLOVER (include/qcu_enum.h:12) and the per-site
 * storage of (Nc*Ns)^2/2 complex (include/basic_data/qcu_point.cuh:98-101)
 * but has no clover code; this layout follows that storage:
 *   clover [parity=2][Vh][block=2][2N][2N] complex double (device), block 0
 *   acting on spins 0, 1 and block 1 on spins 2, 3, row / column index =
 *   local spin * N + colour; the blocks must be Hermitian.
 * qcuLoadClover copies it and inverts every block once (FP64); a singular
 * block returns QCU_ERR_INVALID_ARGUMENT.  The solvers use it when
 * QcuSolverParam.use_clover = 1. */
int qcuLoadClover(void *clover);
/* out = A_parity in (inverse = 1: A_parity^-1 in) on resident MRHS fields */
int qcuCloverMRHS(void *out, void *out_norm, const void *in, const void *in_norm, int nrhs, int parity, int inverse,
                  int precision);

/* out[r] = |field_r|^2 (FP64 accumulation, deterministic order) for each RHS
 * of a resident MRHS field of the session lattice, precision FP32 or FP64.
 * out is a device array of nrhs doubles.  The block partial sums live in the
 * session's workspace (allocated on first use).  Asynchronous on the library
 * stream. */
int qcuNorm2MRHS(double *out, const void *field, int precision, int nrhs);

/* BLAS-1 on MRHS fields (no counterpart in the reference, which has no linear
 * algebra): the operations the solvers are built from, for callers composing
 * their own iterations.  Fields hold n_elements complex values, RHS innermost
 * (element e belongs to RHS e % nrhs; n_elements a multiple of nrhs), in
 * FP32 or FP64 (x_precision, ...).  a, b, c are device arrays of nrhs
 * complex doubles (re, im) or NULL for 1; out is a device array.
 *   QCU_BLAS_AXPBY       y = a x + b y
 *   QCU_BLAS_AXPBYPCZ    z = a x + b y + c z        (one precision)
 *   QCU_BLAS_AXPBY_NORM  y = a x + b y, out[r] = |y_r|^2 (doubles)
 *   QCU_BLAS_NORM2       out[r] = |x_r|^2, every product in FP64
 *   QCU_BLAS_NORM2_FP32  the same with FP32 products for FP32 fields
 *   QCU_BLAS_CDOT        out[r] = sum conj(x_r) y_r (complex doubles)
 *   QCU_BLAS_ADD_TO      y += x (any precisions)
 *   QCU_BLAS_COPY        y = x (with precision conversion)
 * Reductions accumulate in FP64 in a fixed order (bitwise reproducible).
 * Needs an initialised session (its workspace holds the block partial sums);
 * asynchronous on the library stream. */
#define QCU_BLAS_AXPBY 0
#define QCU_BLAS_AXPBYPCZ 1
#define QCU_BLAS_AXPBY_NORM 2
#define QCU_BLAS_NORM2 3
#define QCU_BLAS_NORM2_FP32 4
#define QCU_BLAS_CDOT 5
#define QCU_BLAS_ADD_TO 6
#define QCU_BLAS_COPY 7
int qcuBlasMRHS(int op, const void *a, const void *b, const void *c, const void *x, int x_precision, void *y,
                int y_precision, void *z, int z_precision, size_t n_elements, int nrhs, void *out);

/* No counterpart in the reference.  The same per-RHS norm for callers that
 * cannot allocate device memory: host callbacks and graph nodes, real-time
 * loops that cannot absorb cudaFree's device-wide synchronisation, processes
 * whose device memory another allocator already owns.  It needs no session
 * and allocates nothing.  The block partial sums live in a fixed 512 KiB
 * array inside libqcu.so, held on every GPU that loads the library until the
 * process exits.
 *   field:      n_elements complex values, RHS innermost (element e belongs
 *               to RHS e % nrhs), FP32 or FP64
 *   out:        device array of nrhs doubles
 *   limit:      nrhs <= 64; larger requests return QCU_ERR_CAPACITY
 *   stream:     cudaStream_t (NULL: the legacy default stream), asynchronous
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress) and keeps it for the life of the process; make that
 * first call before any stream capture, and do not use the library on a
 * device after cudaDeviceReset (which destroys the array).  Every call
 * shares the one array: calls whose work overlaps on the GPU race, so
 * serialise them (one stream, or events). */
int qcuNorm2MRHSNoAlloc(double *out, const void *field, int precision, size_t n_elements, int nrhs, void *stream);

/* One segment of qcuDslashSegments: the hop term on one lattice, with its
 * own gauge and fields (no counterpart in the reference, which launches one
 * kernel per operator call). */
typedef struct QcuHopSegment_s {
  int lattice[4];              /* X, Y, Z, T of this segment's lattice (X even) */
  const void *gauge;           /* [4][2][N*N][Vh] complex, the coalesced gauge layout, in `precision` */
  const void *gauge_two_row;   /* SU(3) only: the first two rows of every link in groups of 32
                                  sites, [4][2][Vp/32][6][32] with Vp = Vh rounded up to a multiple
                                  of 32 (component k of site s of a (mu, parity) block at
                                  (s / 32) * 192 + 32 k + s % 32), or NULL */
  const void *in;              /* resident MRHS field [4N][Vh][nrhs] (parity 1 - parity) */
  void *out;                   /* resident MRHS field, output parity; not the same memory as in or x */
  const void *x;               /* optional xpay field (output parity), or NULL */
  double a, b;                 /* out = a * D in + b * x (a = 1, b = 0: the plain hop) */
  int nrhs, parity, dagger, antiperiodic_t;
} QcuHopSegment;

/* The hop term on `count` segments of different lattices, gauges and RHS
 * counts in one kernel launch per 16 segments: a work list of (segment,
 * block) pairs, so small lattices share the GPU instead of each paying a
 * launch and a tail.  All segments share one kernel shape (same nColors and
 * precision, FP32, FP64 or BF16): the one QCU_DSLASH_CONFIG pins, else the
 * fastest work-list shape for this list of (volume, nrhs), timed on the first
 * call with it and cached (one segment: the lattice's own tuned shape, as
 * qcuDslashMRHS uses); each result is bit-identical to launching that shape
 * on the segment alone.  When the
 * shape has no work-list form the segments run one launch each, and a
 * segment whose nrhs is not a multiple of the shape's RHS per thread runs
 * alone with its own shape.  Asynchronous on `stream` (a cudaStream_t, NULL
 * for the legacy default stream). */
int qcuDslashSegments(const QcuHopSegment *segments, int count, int nColors, int precision, void *stream);

/* The kernel shape the dslash uses for (N, nrhs, volume, precision): the
 * shape pinned by QCU_DSLASH_CONFIG, else the cached choice (this process's,
 * or the file named by QCU_TUNE_CACHE), else the fastest shape, timed now and
 * cached.  Returns the chosen RHS-per-thread, block size, register-cap variant
 * (registers per thread: 1 no cap, 2 = 128, 3 = 85, 4 = 112, 5 = 96,
 * 6 = 104), whether the packed FP32x2 arithmetic variant was chosen, and the
 * ring depth of the TMA-staged kernel (0: the register kernel was chosen;
 * -v: tensor-core variant v, see qcuDslashKernels), whether the kernel
 * reads two-row SU(3) links (recon = 1), and whether its links are staged by
 * TMA per x-row (linktma = 1).  Any output pointer may be NULL. */
int qcuTuneDslash(int nrhs, int precision, int *rhs_per_thread, int *block, int *reg_cap, int *packed, int *stages,
                  int *recon, int *linktma);

/* No counterpart in the reference.  The kernel shape that the last
 * single-lattice dslash launched by the calling thread ran, after the dispatcher's fallbacks (a
 * pinned or tuned shape whose kernel cannot take the arguments runs the
 * register kernel): shape[0..5] = (RHS per thread, register-cap variant,
 * packed, stages, recon, linktma) as in qcuDslashKernels; all zero before the
 * thread's first dslash. */
int qcuLastDslashShape(int *shape);

/* No counterpart in the reference.  FMA throughput of the current GPU in
 * TFLOP/s (2 flop per FMA), precision QCU_DOUBLE_PRECISION or
 * QCU_SINGLE_PRECISION: the peak that bounds compute-bound kernels such as
 * the FP64 dslash.  Synchronous; takes a few milliseconds. */
int qcuMeasureFmaRate(int precision, double *tflops);

/* The compiled dslash kernel shapes for (precision, nColors): *count 6-tuples
 * (RHS per thread, register-cap variant, packed, stages, recon, linktma) are
 * available; the first max_shapes are written to shapes[6 * i .. 6 * i + 5].
 * stages > 0 is the TMA-staged kernel with that many ring buffers, stages < 0
 * a tensor-core (tcgen05) kernel, BF16 only: -1 projected half-spinor
 * operands with direct loads, -2 / -3 the same with a TMA ring of that depth,
 * -4 / -5 / -6 the neighbour spinor block as the MMA operand (warp-specialised,
 * TMA and B rings of different depths; nrhs a multiple of 4), -7 / -8 the
 * same with deeper rings of half-size stages (tiles of at most 32 RHS);
 * recon = 1 reads
 * SU(3) links as two rows and reconstructs the third (used only when the
 * loaded gauge is SU(3) to the precision's rounding); linktma = 1 is the
 * register kernel with one CTA per x-row whose links are staged by TMA into
 * shared memory (used when X/2 x the complex size is a multiple of 16 bytes
 * and X/2 x nrhs / R <= 512).  Any shape can be pinned with
 * QCU_DSLASH_CONFIG="R,block,reg_cap,packed,stages,rcta,tensor,recon,linktma"
 * (tensor = 1..8 for the tensor-core variants).  Where whole t-slices of the
 * fields overflow L2, the register kernels walk the lattice in slabs of
 * z-planes (t slowest within a slab); QCU_DSLASH_ZSLAB=<planes> overrides the
 * slab height (0: the field's own order). */
int qcuDslashKernels(int precision, int nColors, int *shapes, int max_shapes, int *count);

typedef struct QcuSolverParam_s {
  int solver;          /* QCU_SOLVER_CG or QCU_SOLVER_BICGSTAB */
  int inner_precision; /* operator precision of the inner iterations */
  double kappa;
  double tol;          /* target |b - M x| / |b| per RHS (FP64 true residual) */
  int max_iter;
  double delta;        /* reliable-update trigger: |r| < delta * max|r| since the last update */
  int use_graph;       /* capture inner iterations in CUDA graphs */
  int src_mode;        /* QCU_SRC_EO_FULL or QCU_SRC_LEX for x and b */
  int use_clover;      /* 1: M = A - kappa D with the clover field of qcuLoadClover */
  /* outputs */
  int iterations;
  int reliable_updates;
  double seconds;
  double true_residual[256]; /* per RHS, FP64 */
  int converged[256];
} QcuSolverParam;

/* ---- solve server: resident gauges, continuous MRHS batching ------------
 * A server keeps gauge fields resident (one lane each, with its own stream
 * and worker thread, so lanes overlap on the device), admits requests into
 * free RHS slots between iteration chunks of the running batch, and reports
 * latency percentiles.  A lane's slot capacity is fixed when its gauge is
 * added, from the HBM budget.  Requests carry their own kappa and tolerance;
 * x and b are device arrays of nrhs full even-odd fields [2][Vh][4][N]
 * (complex double) that must stay valid until the request is done.  The
 * server calls are thread-safe and do not use the qcu.h session.  Lanes run
 * on non-blocking streams of their own; work queued on the legacy default
 * stream before qcuServerAddGauge / qcuServerSubmit is ordered before the
 * server reads the gauge / the sources, and a request's solution is in
 * memory when qcuServerWait reports it done. */
typedef struct QcuRequestInfo_s {
  int done, status, nrhs, iterations;
  double latency_s; /* submit -> solution written */
  double queue_s;   /* submit -> admitted */
  double max_true_residual;
  int all_converged;
} QcuRequestInfo;

typedef struct QcuServerStats_s {
  long long submitted, completed;
  double p50_s, p99_s, mean_s;
  double solves_per_s, rhs_per_s;
  size_t hbm_used;
} QcuServerStats;

int qcuServerCreate(void **server, size_t hbm_budget_bytes, int max_slots_per_gauge, int inner_precision,
                    int solver);
int qcuServerAddGauge(void *server, int gauge_id, const int lattice[4], int nColors, const void *gauge,
                      int antiperiodic_t);
int qcuServerSubmit(void *server, int gauge_id, double kappa, double tol, int nrhs, void *const *x,
                    void *const *b, long long *request_id);
/* timeout < 0 waits forever; returns QCU_OK whether or not the request is done
 * (see info->done and info->status) */
int qcuServerWait(void *server, long long request_id, double timeout_s, QcuRequestInfo *info);
int qcuServerStats(void *server, QcuServerStats *stats);
int qcuServerDestroy(void *server);

void qcuSolverParamDefaults(QcuSolverParam *p);
/* Solve M x_r = b_r for nrhs right-hand sides with the loaded gauge.
 * Returns QCU_ERR_NOT_CONVERGED when some RHS did not reach tol within
 * max_iter (p->converged[r] and p->true_residual[r] say which), and
 * QCU_ERR_INVALID_ARGUMENT when a source holds NaN or Inf: such a source is
 * not solved (its x is not meaningful) while the others are.  The server
 * reports the same two conditions in QcuRequestInfo.status. */
int qcuInvert(void *const *x, void *const *b, int nrhs, QcuSolverParam *p);

/* Diagnostic of the device-side wait bound (no counterpart in the
 * reference).  The staged and tensor-core dslash kernels wait on mbarriers
 * with a bound of about one second; when a wait runs out, the kernel sets a
 * device flag and returns, and the next synchronising call reports
 * QCU_ERR_DEVICE_TIMEOUT with the context still usable.  This runs one
 * kernel that waits, with the same bounded wait, on a barrier that nothing
 * completes, with the bound set to limit_seconds (0 < limit_seconds <= 1),
 * and reports through the same path: the expected result is
 * QCU_ERR_DEVICE_TIMEOUT.  Synchronous. */
int qcuCheckWaitTimeout(double limit_seconds);

#ifdef __cplusplus
}
#endif
