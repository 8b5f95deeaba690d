// qcuNorm2MRHSNoAlloc: the per-RHS norm reduction of qcuNorm2MRHS for
// callers that cannot allocate device memory.
//
// Who cannot allocate: code that runs where cudaMalloc / cudaFree are not
// allowed or not acceptable:
//  * a host callback (cudaLaunchHostFunc) or a CUDA-graph node;
//  * a real-time loop, where cudaFree's device-wide synchronisation would stall
//    every stream;
//  * a process whose device memory is reserved up front by another allocator
//    (a framework's caching allocator, a fixed memory pool).
// qcuNorm2MRHS keeps its block partial sums in the session workspace, which
// is allocated on first use.  This entry point takes no session and
// allocates nothing.  Its partial sums live in the file-scope device array
// g_noalloc_partials: 1024 blocks x 64 RHS doubles = 512 KiB, held on every
// GPU that loads the library until the process exits.
#include <mutex>
#include <new>
#include <stdexcept>

#pragma GCC visibility push(default)  // the public header: exported
#include "../../include/qcu_gb300.h"
#pragma GCC visibility pop
#include "blas.h"

extern "C" void qcu_record_error(int code, const char* msg);

namespace {

constexpr int kNoAllocMaxRhs = 64;
constexpr int kNoAllocBlocks = 1024;
constexpr int kMaxDevices = 64;

// Shared by every call on a device: each call overwrites every partial it
// reads (one value per launched block and RHS), so nothing needs clearing,
// and calls that overlap on the GPU race on this array.
static __device__ __align__(256) double g_noalloc_partials[kNoAllocBlocks * kNoAllocMaxRhs];

std::mutex g_addr_mutex;
void* g_addr[kMaxDevices] = {};

// Device address of g_noalloc_partials on the current device.  In host code
// the array's name is only a host-side stand-in, never a device address, so
// the address is queried once per device, with that device current, and
// cached for the life of the process.  cudaDeviceReset destroys the module
// that holds the array (and every other resource of this library on that
// device), so the library is not used on a device after resetting it.
double* partials_address() {
  int dev = -1;
  QCU_CHECK_CUDA(cudaGetDevice(&dev));
  QCU_REQUIRE(dev >= 0 && dev < kMaxDevices, QCU_ERR_UNSUPPORTED, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_addr_mutex);
  if (!g_addr[dev]) {
    void* a = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&a, g_noalloc_partials);
    QCU_REQUIRE(e == cudaSuccess && a != nullptr, QCU_ERR_CUDA,
                std::string("cudaGetSymbolAddress(g_noalloc_partials) failed: ") + cudaGetErrorString(e));
    g_addr[dev] = a;
  }
  return static_cast<double*>(g_addr[dev]);
}

}  // namespace

extern "C" int qcuNorm2MRHSNoAlloc(double* out, const void* field, int precision, size_t n_elements, int nrhs,
                                   void* stream) {
  try {
    QCU_REQUIRE(out && field, QCU_ERR_INVALID_ARGUMENT, "qcuNorm2MRHSNoAlloc: null pointer");
    QCU_REQUIRE(precision == QCU_SINGLE_PRECISION || precision == QCU_DOUBLE_PRECISION, QCU_ERR_UNSUPPORTED,
                "qcuNorm2MRHSNoAlloc: the field must be FP32 or FP64");
    QCU_REQUIRE(nrhs >= 1, QCU_ERR_INVALID_ARGUMENT, "qcuNorm2MRHSNoAlloc: nrhs must be positive");
    QCU_REQUIRE(nrhs <= kNoAllocMaxRhs, QCU_ERR_CAPACITY,
                "qcuNorm2MRHSNoAlloc: nrhs " + std::to_string(nrhs) + " exceeds the fixed scratch limit of " +
                    std::to_string(kNoAllocMaxRhs) + " RHS (use qcuNorm2MRHS)");
    QCU_REQUIRE(n_elements > 0 && n_elements % (size_t)nrhs == 0, QCU_ERR_INVALID_ARGUMENT,
                "qcuNorm2MRHSNoAlloc: n_elements must be a positive multiple of nrhs");
    QCU_REQUIRE(qcu::Blas::blocks_for((int64_t)n_elements) <= kNoAllocBlocks, QCU_ERR_CAPACITY,
                "qcuNorm2MRHSNoAlloc: reduction grid exceeds the fixed scratch array");
    qcu::Blas blas(partials_address(), kNoAllocBlocks);
    qcu::FieldRef f;
    f.data = const_cast<void*>(field);
    f.prec = precision;
    f.n = (int64_t)n_elements;
    f.nrhs = nrhs;
    blas.norm2(f, out, static_cast<cudaStream_t>(stream));
    return QCU_OK;
  } catch (const qcu::Error& e) {
    qcu_record_error(e.code, e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    qcu_record_error(QCU_ERR_OUT_OF_MEMORY, "host allocation failed");
    return QCU_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    qcu_record_error(QCU_ERR_CUDA, e.what());
    return QCU_ERR_CUDA;
  }
}
