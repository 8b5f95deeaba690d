// Host side of the TMA-staged dslash (dslash_tma.cuh): tensor maps, the
// tile plan, the launcher template used by the instantiation units, and the
// device timeout flag of its bounded waits.
#pragma once

#include <cuda.h>

#include "dslash.h"
#include "dslash_tma.cuh"

namespace qcu {

// device address of the timeout flag (zero-initialised, one per device)
int* tma_error_flag();
// true once per timeout: reads and clears the flag if a staged kernel ran
// since the last check (synchronises the stream first)
bool tma_check_timeout(cudaStream_t st);
void tma_note_launch();
// One kernel whose bounded wait (limit_s seconds) is on an mbarrier that
// nothing completes: the timeout path of the staged kernels, without any
// copy in flight.  Returns whether the device reported the timeout.
bool wait_timeout_selftest(double limit_s, cudaStream_t st);

// tensor maps in 4-byte units: field [4N][Vh][nrhs] with box {rcta, hx, 4N};
// gauge [8][N*N][Vh] with box {hx, N*N, 1}
void tma_encode_field(CUtensorMap* m, const void* ptr, int ebytes, int nrhs, int vh, int ncomp, int rcta, int hx);
void tma_encode_gauge(CUtensorMap* m, const void* ptr, int ebytes, int vh, int nn, int hx);
// the two-row gauge in groups of 32 sites, [8][vhp/32][6][32] (vhp: Vh padded
// to 32), as {32 sites, 6 components, 8 vhp / 32 groups}, box {hx, 6, 1}
void tma_encode_gauge_groups(CUtensorMap* m, const void* ptr, int ebytes, int vhp, int hx);
// 16-bit storage scales [Vh][nrhs] float with box {rcta, hx}
void tma_encode_norm(CUtensorMap* m, const float* ptr, int nrhs, int vh, int rcta, int hx);
// the MRHS field of a tensor-core operand: [site][spin 4][colour N][RHS] of
// 4-byte complex BF16 in the component- or site-major layout, box (32 RHS,
// 8 colours, 4 spins, 1 site), 128-byte swizzle, colours N..7 zero-filled;
// false when the driver rejects the map
bool tma_encode_field_swizzled(CUtensorMap* m, const void* ptr, int nrhs, int vh, int N, bool site_major);
// the same field with the RHS index split as 32 x (nrhs / 32) (nrhs a multiple
// of 32): dims (RHS 32, colour, spin, half, site), box (32, 8, 4, 2, 1), so
// that one copy lands two 32-RHS halves 4 KB apart in shared memory
bool tma_encode_field_swizzled_halves(CUtensorMap* m, const void* ptr, int nrhs, int vh, int N, bool site_major);

// Tile plan for (precision, N, geometry, nrhs, R, stages); rcta = 0 picks the
// largest RHS chunk that fits.  False when the staged kernel cannot run these
// arguments (alignment, box or shared-memory limits, 16-bit storage).
bool tma_plan(int prec, int N, const Geometry& geo, int nrhs, int R, int nst, int rcta, TmaDslashArgs* T,
              int* threads, size_t* smem);
bool tma_pointers_ok(const DslashArgs& A);
int tma_grid(const void* kernel, int threads, size_t smem, int ntiles);

template <int P, int N, int R, int NST>
void launch_wilson_tma(const DslashArgs& A, int rcta, cudaStream_t st) {
  using E = typename Store<P>::elem;
  TmaDslashArgs T;
  int threads = 0;
  size_t smem = 0;
  QCU_REQUIRE(tma_plan(P, N, A.geo, A.nrhs, R, NST, rcta, &T, &threads, &smem) && tma_pointers_ok(A),
              QCU_ERR_UNSUPPORTED, "staged dslash: arguments outside the kernel's limits");
  T.A = A;
  T.err = tma_error_flag();
  CUtensorMap mi, mg;
  tma_encode_field(&mi, A.in, (int)sizeof(E), A.nrhs, A.geo.vh, 4 * N, T.rcta, A.geo.hx);
  tma_encode_gauge(&mg, A.gauge, (int)sizeof(E), A.geo.vh, N * N, A.geo.hx);
  CUtensorMap mn;
  if constexpr (Store<P>::has_norm)
    tma_encode_norm(&mn, A.in_norm, A.nrhs, A.geo.vh, T.rcta, A.geo.hx);
  else
    mn = mg;  // not read
  const void* k = reinterpret_cast<const void*>(&wilson_tma_kernel<P, N, R, NST>);
  static size_t smem_set = 0;  // the attribute only grows; set outside graph capture by the first launch
  if (smem > smem_set) {
    QCU_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    smem_set = smem;
  }
  const int grid = tma_grid(k, threads, smem, T.ntiles);
  wilson_tma_kernel<P, N, R, NST><<<grid, threads, smem, st>>>(T, mi, mg, mn);
  tma_note_launch();
}

using TmaLauncher = void (*)(const DslashArgs&, int rcta, cudaStream_t);
void register_tma(int prec, int N, int R, int nst, TmaLauncher fn);
TmaLauncher find_tma(int prec, int N, int R, int nst);
// compiled (R, stages) pairs for (prec, N)
int tma_options(int prec, int N, int* R, int* nst, int max);

}  // namespace qcu
