// Host side of the tensor-core dslash (dslash_tc.cuh): tile plan, launcher,
// registry.
#pragma once

#include <cstring>

#include "dslash.h"
#include "dslash_tc.cuh"
#include "dslash_tcs.cuh"
#include "dslash_tma.h"

namespace qcu {

// Tile plan for (precision, N, geometry, nrhs) and ring depth nst (0: no
// ring): false when the tensor-core kernel cannot run these arguments (BF16
// storage and N = 4..8 only; the ring also needs nrhs and the tile's RHS
// count to be multiples of 4 for its TMA boxes).  *smem: dynamic shared bytes.
bool tc_plan(int prec, int N, const Geometry& geo, int nrhs, int nst, TcDslashArgs* T, size_t* smem);
// grid of a persistent tensor-core kernel: CTAs per SM from registers and
// shared memory, capped so that their tensor memory (tmem_cols each) fits
int tc_grid(const void* kernel, int ntiles, size_t smem, int tmem_cols = 32, int threads = 128);

// Tile plan of the spinor-operand kernel (dslash_tcs.cuh); false when it
// cannot run these arguments (BF16, N = 2..8, nrhs a multiple of 4, the
// site-major links present, 16-byte aligned field and links, 32-bit element
// offsets, and a field map the driver accepts).
bool tcs_plan(const DslashArgs& A, int N, TcsDslashArgs* T, CUtensorMap* map_in);

// ring depths of the spinor-operand variants 4-8: (TMA stages, B buffers, A
// halves of 32 RHS per stage).  Variants 7 and 8 hold one half per stage, so
// their deeper rings fit the same shared memory; they take tiles of at most
// 32 RHS (nrhs <= 32, or RHS counts that split into such tiles).
constexpr int tcs_stages(int variant) { return variant == 5 ? 6 : variant == 6 ? 5 : variant == 7 ? 8 : variant == 8 ? 6 : 4; }
constexpr int tcs_bbufs(int variant) { return (variant == 6 || variant == 7 || variant == 8) ? 2 : 3; }
constexpr int tcs_halves(int variant) { return variant >= 7 ? 1 : 2; }

// Variants 4 and 6-8 are sized so that 4 CTAs share an SM (228 KB of shared
// memory, 1 KB reserved per CTA; tensor memory 4 x 128 columns); variant 5
// trades the fourth CTA for six stages.
constexpr bool tcs_fits_4_ctas(int v) {
  return 4 * (tcs::smem_bytes(tcs_stages(v), tcs_bbufs(v), tcs_halves(v)) + 1024) <= 228 * 1024;
}
static_assert(tcs_fits_4_ctas(4) && tcs_fits_4_ctas(6) && tcs_fits_4_ctas(7) && tcs_fits_4_ctas(8),
              "a spinor-operand variant no longer fits 4 CTAs per SM");

template <int N, int V>
void launch_wilson_tcs(const DslashArgs& A, cudaStream_t st) {
  constexpr int NST = tcs_stages(V), NB = tcs_bbufs(V), HV = tcs_halves(V);
  TcsDslashArgs T;
  CUtensorMap mi;
  QCU_REQUIRE(tcs_plan(A, N, &T, &mi) && T.halves <= HV, QCU_ERR_UNSUPPORTED,
              "tensor-core dslash: arguments outside the kernel's limits");
  T.A = A;
  T.err = tma_error_flag();
  const size_t smem = tcs::smem_bytes(NST, NB, HV);
  const void* k = reinterpret_cast<const void*>(&wilson_tcs_kernel<N, NST, NB, HV>);
  static size_t smem_set = 0;
  if (smem > 48 * 1024 && smem > smem_set) {
    QCU_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    smem_set = smem;
  }
  const int grid = tc_grid(k, T.ntiles, smem, (int)tcs::kTmemCols, tcs::kThreads);
  wilson_tcs_kernel<N, NST, NB, HV><<<grid, tcs::kThreads, smem, st>>>(T, mi);
  tma_note_launch();
}

template <int N, int NST>
void launch_wilson_tc(const DslashArgs& A, cudaStream_t st) {
  TcDslashArgs T;
  size_t smem = 0;
  QCU_REQUIRE(tc_plan(PREC_BF16, N, A.geo, A.nrhs, NST, &T, &smem), QCU_ERR_UNSUPPORTED,
              "tensor-core dslash: arguments outside the kernel's limits");
  T.A = A;
  T.err = tma_error_flag();
  CUtensorMap mi;
  if constexpr (NST > 0)
    tma_encode_field(&mi, A.in, 4, A.nrhs, A.geo.vh, 4 * N, T.rt, 1);
  else
    memset(&mi, 0, sizeof(mi));  // not read
  const void* k = reinterpret_cast<const void*>(&wilson_tc_kernel<N, NST>);
  static size_t smem_set = 0;
  if (smem > 48 * 1024 && smem > smem_set) {
    QCU_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    smem_set = smem;
  }
  const int grid = tc_grid(k, T.ntiles, smem);
  wilson_tc_kernel<N, NST><<<grid, 128, smem, st>>>(T, mi);
  tma_note_launch();
}

// variant: 1 = direct loads, 2 / 3 = TMA ring of 2 / 3 stages (projected
// half-spinor operands, dslash_tc.cuh); 4 / 5 / 6 = the spinor-operand kernel
// (dslash_tcs.cuh) with (TMA stages, B buffers) = (4, 3) / (6, 3) / (5, 2);
// 7 / 8 = the same with one 32-RHS half per stage, (8, 2) / (6, 2)
constexpr int kTcVariants = 8;  // <= 15 (registry keys)
using TcLauncher = void (*)(const DslashArgs&, cudaStream_t);
void register_tc(int prec, int N, int variant, TcLauncher fn);
TcLauncher find_tc(int prec, int N, int variant = 1);
int tc_ring_stages(int variant);

}  // namespace qcu
