// FMA pipe throughput of this GPU (qcuMeasureFmaRate): the denominator for
// kernels that the FP64 pipe bounds rather than HBM (the FP64 dslash: 1320
// flop per site and RHS against 480 bytes).  No counterpart in the
// reference.
//
// Every thread runs 8 independent FMA chains (enough in flight to cover the
// pipe latency at full occupancy) for `iters` steps; the grid fills every SM.
// A data-dependent store keeps the chains live.
#include <cuda_runtime.h>

#pragma GCC visibility push(default)  // the public header: exported
#include "../../include/qcu_gb300.h"
#pragma GCC visibility pop
#include "qcu_common.cuh"

extern "C" void qcu_record_error(int code, const char* msg);

namespace qcu {
namespace {

template <typename T>
__global__ void __launch_bounds__(256) fma_chains_kernel(T* sink, int iters, T a, T b) {
  T v[8];
#pragma unroll
  for (int k = 0; k < 8; k++) v[k] = (T)(threadIdx.x + k);
  for (int i = 0; i < iters; i++)
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = v[k] * a + b;
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += v[k];
  if (s == (T)-1.2345) sink[blockIdx.x] = s;  // never true for these inputs; keeps the work
}

template <typename T>
double measure(int iters) {
  int dev = 0, sms = 0;
  QCU_CHECK_CUDA(cudaGetDevice(&dev));
  QCU_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int grid = sms * 8, block = 256;
  T* sink = nullptr;
  QCU_CHECK_CUDA(cudaMalloc(&sink, sizeof(T) * grid));
  cudaEvent_t e0, e1;
  QCU_CHECK_CUDA(cudaEventCreate(&e0));
  QCU_CHECK_CUDA(cudaEventCreate(&e1));
  // a = 1 - 2^-20, b = 2^-20: the chains stay bounded and never reach -1.2345
  const T a = (T)(1.0 - 1.0 / 1048576.0), b = (T)(1.0 / 1048576.0);
  fma_chains_kernel<T><<<grid, block>>>(sink, iters / 8, a, b);  // warm-up
  QCU_CHECK_CUDA(cudaEventRecord(e0));
  fma_chains_kernel<T><<<grid, block>>>(sink, iters, a, b);
  QCU_CHECK_CUDA(cudaEventRecord(e1));
  QCU_CHECK_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  QCU_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  const double flops = 2.0 * 8.0 * (double)iters * grid * block;
  return flops / (ms * 1e-3) / 1e12;
}

}  // namespace
}  // namespace qcu

extern "C" int qcuMeasureFmaRate(int precision, double* tflops) {
  try {
    QCU_REQUIRE(tflops != nullptr, QCU_ERR_INVALID_ARGUMENT, "qcuMeasureFmaRate: null output");
    QCU_REQUIRE(precision == QCU_DOUBLE_PRECISION || precision == QCU_SINGLE_PRECISION, QCU_ERR_INVALID_ARGUMENT,
                "qcuMeasureFmaRate: precision must be single or double");
    *tflops = precision == QCU_DOUBLE_PRECISION ? qcu::measure<double>(1 << 14) : qcu::measure<float>(1 << 16);
    return QCU_OK;
  } catch (const qcu::Error& e) {
    qcu_record_error(e.code, e.what());
    return e.code;
  }
}
