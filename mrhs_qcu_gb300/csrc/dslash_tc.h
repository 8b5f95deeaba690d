// Host side of the tensor-core dslash (dslash_tc.cuh): tile plan, launcher,
// registry.
#pragma once

#include "dslash.h"
#include "dslash_tc.cuh"
#include "dslash_tma.h"

namespace qcu {

// Tile plan for (precision, N, geometry, nrhs): false when the tensor-core
// kernel cannot run these arguments (BF16 storage and N = 4..8 only).
bool tc_plan(int prec, int N, const Geometry& geo, int nrhs, TcDslashArgs* T);
int tc_grid(const void* kernel, int ntiles);

template <int N>
void launch_wilson_tc(const DslashArgs& A, cudaStream_t st) {
  TcDslashArgs T;
  QCU_REQUIRE(tc_plan(PREC_BF16, N, A.geo, A.nrhs, &T), QCU_ERR_UNSUPPORTED,
              "tensor-core dslash: arguments outside the kernel's limits");
  T.A = A;
  T.err = tma_error_flag();
  const void* k = reinterpret_cast<const void*>(&wilson_tc_kernel<N>);
  const int grid = tc_grid(k, T.ntiles);
  wilson_tc_kernel<N><<<grid, 128, tc::kSmemBytes, st>>>(T);
  tma_note_launch();
}

using TcLauncher = void (*)(const DslashArgs&, cudaStream_t);
void register_tc(int prec, int N, TcLauncher fn);
TcLauncher find_tc(int prec, int N);

}  // namespace qcu
