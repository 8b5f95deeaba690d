// Launch shims around the reference's own device code, used ONLY to pin the
// oracle against the reference (tests/golden/make_golden.py runs them on a
// GPU through the CUDA driver API).  Built by oracle/build_ref.sh from the
// reference headers where they lie; the output goes to oracle/_ref/.
//
// The reference's dslash kernel is a `static __global__` template
// (include/kernels/wilson_dslash_4d.cuh:303-322), so its symbol is internal
// to its translation unit.  The shims below call the reference's
// `applyWilson` device function (wilson_dslash_4d.cuh:25-301) for one output
// site per thread, which is what dslashKernel does when launched, as the
// reference launches it, with grid = Vh/256 and block = 256
// (src/qcd/qcu_wilson.cu:9-18,25): its loop (wilson_dslash_4d.cuh:318-321)
// then runs once per thread.  A `tid < Vh` guard is added so lattices whose
// half volume is not a multiple of 256 stay in bounds.
//
// The storage (layout) kernels are ordinary __global__ templates; they are
// explicitly instantiated here and looked up by their mangled names.
#include "kernels/storage/storage_kernels.cuh"
#include "kernels/wilson_dslash_4d.cuh"

namespace {
template <typename T, int N, int n>
__device__ __forceinline__ void ref_dslash_site(qcu::MrhsInput<n>& out, qcu::MrhsInput<n>& in, void* gauge, T flag,
                                                int Lx, int Ly, int Lz, int Lt, int parity) {
  const int tid = threadIdx.x + blockIdx.x * blockDim.x;
  if (tid >= Lx * Ly * Lz * Lt / 2) return;
  qcu::Complex<T> src[Ns * N];
  qcu::Complex<T> dst[Ns * N * n];
  qcu::Complex<T> u[N * N];
  qcu::kernel::applyWilson<T, N, n>(out, in, gauge, dst, src, u, flag, Lx, Ly, Lz, Lt, 1, 1, 1, 1, parity, tid);
}
}  // namespace

#define QCUREF_DSLASH(T, TAG, N, n)                                                                              \
  extern "C" __global__ void qcuref_dslash_##TAG##_##N##_##n(qcu::MrhsInput<n> out, qcu::MrhsInput<n> in,       \
                                                               void* gauge, T flag, int Lx, int Ly, int Lz,     \
                                                               int Lt, int parity) {                            \
    ref_dslash_site<T, N, n>(out, in, gauge, flag, Lx, Ly, Lz, Lt, parity);                                     \
  }

QCUREF_DSLASH(double, d, 3, 1)
QCUREF_DSLASH(double, d, 3, 2)
QCUREF_DSLASH(double, d, 3, 3)
QCUREF_DSLASH(double, d, 3, 4)
QCUREF_DSLASH(double, d, 3, 5)
QCUREF_DSLASH(float, f, 3, 1)
QCUREF_DSLASH(float, f, 3, 4)
QCUREF_DSLASH(double, d, 4, 2)
QCUREF_DSLASH(float, f, 4, 2)
QCUREF_DSLASH(double, d, 5, 1)
QCUREF_DSLASH(float, f, 5, 1)

template __global__ void qcu::kernel::storeVectorCoalesced<double, 3>(void*, void*, int, int, int, int);
template __global__ void qcu::kernel::storeVectorNonCoalesced<double, 3>(void*, void*, int, int, int, int);
template __global__ void qcu::kernel::storeGaugeCoalesced<double, 3>(void*, void*, int, int, int, int);
template __global__ void qcu::kernel::storeGaugeNonCoalesced<double, 3>(void*, void*, int, int, int, int);
