// Host side of the TMA-staged dslash (see dslash_tma.h).
#include <cudaTypedefs.h>

#include <atomic>
#include <map>
#include <mutex>

#include "dslash_tma.h"

namespace qcu {
namespace {

__device__ int g_tma_timeout = 0;
constexpr int kMaxDevices = 64;
int* g_flag_addr[kMaxDevices] = {};
std::mutex g_flag_mutex;
std::atomic<bool> g_launched{false};

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  QCU_REQUIRE(fn != nullptr, QCU_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available from the driver");
  return fn;
}

void encode(CUtensorMap* m, const void* ptr, const cuuint64_t dims[3], const cuuint64_t strides[2],
            const cuuint32_t box[3], cuuint32_t rank = 3) {
  const cuuint32_t es[3] = {1, 1, 1};
  const CUresult r = encode_fn()(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, rank, const_cast<void*>(ptr), dims, strides,
                                 box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  QCU_REQUIRE(r == CUDA_SUCCESS, QCU_ERR_CUDA, "cuTensorMapEncodeTiled failed with code " + std::to_string((int)r));
}

uint32_t align128(size_t b) { return (uint32_t)((b + 127) / 128 * 128); }

std::map<int, TmaLauncher>& registry() {
  static std::map<int, TmaLauncher> r;
  return r;
}
std::mutex& registry_mutex() {
  static std::mutex m;
  return m;
}
int key(int prec, int N, int R, int nst) { return ((prec * 16 + N) * 16 + R) * 8 + nst; }

}  // namespace

int* tma_error_flag() {
  int dev = 0;
  QCU_CHECK_CUDA(cudaGetDevice(&dev));
  QCU_REQUIRE(dev >= 0 && dev < kMaxDevices, QCU_ERR_UNSUPPORTED, "device index out of range");
  std::lock_guard<std::mutex> lk(g_flag_mutex);
  if (!g_flag_addr[dev]) {
    void* p = nullptr;
    QCU_CHECK_CUDA(cudaGetSymbolAddress(&p, g_tma_timeout));
    g_flag_addr[dev] = static_cast<int*>(p);
  }
  return g_flag_addr[dev];
}

void tma_note_launch() { g_launched.store(true, std::memory_order_relaxed); }

namespace {
// one warp; lane 0 waits on phase 0 of a barrier that expects one arrival
// and never gets it, so the bounded wait runs out, sets the flag and returns
__global__ void wait_selftest_kernel(int* err, uint64_t limit_ns) {
  __shared__ __align__(8) uint64_t bar;
  const uint32_t b = tma::smem_u32(&bar);
  if (threadIdx.x == 0) {
    tma::mbar_init(b, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  if (threadIdx.x == 0) {
    tma::mbar_wait(b, 0, err, limit_ns);
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(b) : "memory");
  }
}
}  // namespace

bool wait_timeout_selftest(double limit_s, cudaStream_t st) {
  int* flag = tma_error_flag();
  wait_selftest_kernel<<<1, 32, 0, st>>>(flag, (uint64_t)(limit_s * 1e9));
  QCU_CHECK_CUDA(cudaGetLastError());
  tma_note_launch();
  QCU_CHECK_CUDA(cudaStreamSynchronize(st));
  return tma_check_timeout(st);
}

bool tma_check_timeout(cudaStream_t st) {
  if (!g_launched.exchange(false)) return false;
  int* flag = tma_error_flag();
  int v = 0;
  QCU_CHECK_CUDA(cudaMemcpyAsync(&v, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
  QCU_CHECK_CUDA(cudaStreamSynchronize(st));
  if (!v) return false;
  const int zero = 0;
  QCU_CHECK_CUDA(cudaMemcpyAsync(flag, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
  QCU_CHECK_CUDA(cudaStreamSynchronize(st));
  return true;
}

void tma_encode_field(CUtensorMap* m, const void* ptr, int ebytes, int nrhs, int vh, int ncomp, int rcta, int hx) {
  const cuuint64_t dims[3] = {(cuuint64_t)nrhs * ebytes / 4, (cuuint64_t)vh, (cuuint64_t)ncomp};
  const cuuint64_t strides[2] = {(cuuint64_t)nrhs * ebytes, (cuuint64_t)vh * nrhs * ebytes};
  const cuuint32_t box[3] = {(cuuint32_t)(rcta * ebytes / 4), (cuuint32_t)hx, (cuuint32_t)ncomp};
  encode(m, ptr, dims, strides, box);
}

void tma_encode_gauge(CUtensorMap* m, const void* ptr, int ebytes, int vh, int nn, int hx) {
  const cuuint64_t dims[3] = {(cuuint64_t)vh * ebytes / 4, (cuuint64_t)nn, 8};
  const cuuint64_t strides[2] = {(cuuint64_t)vh * ebytes, (cuuint64_t)nn * vh * ebytes};
  const cuuint32_t box[3] = {(cuuint32_t)(hx * ebytes / 4), (cuuint32_t)nn, 1};
  encode(m, ptr, dims, strides, box);
}

void tma_encode_gauge_groups(CUtensorMap* m, const void* ptr, int ebytes, int vhp, int hx) {
  const cuuint64_t dims[3] = {(cuuint64_t)32 * ebytes / 4, 6, (cuuint64_t)8 * vhp / 32};
  const cuuint64_t strides[2] = {(cuuint64_t)32 * ebytes, (cuuint64_t)6 * 32 * ebytes};
  const cuuint32_t box[3] = {(cuuint32_t)(hx * ebytes / 4), 6, 1};
  encode(m, ptr, dims, strides, box);
}

bool tma_encode_field_swizzled(CUtensorMap* m, const void* ptr, int nrhs, int vh, int N, bool site_major) {
  // byte strides of colour, spin and site
  const cuuint64_t cs = site_major ? (cuuint64_t)nrhs * 4 : (cuuint64_t)vh * nrhs * 4;
  const cuuint64_t ss = site_major ? (cuuint64_t)4 * N * nrhs * 4 : (cuuint64_t)nrhs * 4;
  const cuuint64_t dims[4] = {(cuuint64_t)nrhs, (cuuint64_t)N, 4, (cuuint64_t)vh};
  const cuuint64_t strides[3] = {cs, (cuuint64_t)N * cs, ss};
  const cuuint32_t box[4] = {32, 8, 4, 1};
  const cuuint32_t es[4] = {1, 1, 1, 1};
  return encode_fn()(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<void*>(ptr), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool tma_encode_field_swizzled_halves(CUtensorMap* m, const void* ptr, int nrhs, int vh, int N, bool site_major) {
  if (nrhs % 32) return false;
  // byte strides of colour, spin, half (32 RHS) and site
  const cuuint64_t cs = site_major ? (cuuint64_t)nrhs * 4 : (cuuint64_t)vh * nrhs * 4;
  const cuuint64_t ss = site_major ? (cuuint64_t)4 * N * nrhs * 4 : (cuuint64_t)nrhs * 4;
  const cuuint64_t dims[5] = {32, (cuuint64_t)N, 4, (cuuint64_t)nrhs / 32, (cuuint64_t)vh};
  const cuuint64_t strides[4] = {cs, (cuuint64_t)N * cs, 128, ss};
  const cuuint32_t box[5] = {32, 8, 4, 2, 1};
  const cuuint32_t es[5] = {1, 1, 1, 1, 1};
  return encode_fn()(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 5, const_cast<void*>(ptr), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

void tma_encode_norm(CUtensorMap* m, const float* ptr, int nrhs, int vh, int rcta, int hx) {
  const cuuint64_t dims[3] = {(cuuint64_t)nrhs, (cuuint64_t)vh, 1};
  const cuuint64_t strides[2] = {(cuuint64_t)nrhs * 4, (cuuint64_t)vh * nrhs * 4};
  const cuuint32_t box[3] = {(cuuint32_t)rcta, (cuuint32_t)hx, 1};
  encode(m, ptr, dims, strides, box, 2);
}

bool tma_plan(int prec, int N, const Geometry& geo, int nrhs, int R, int nst, int rcta, TmaDslashArgs* T,
              int* threads, size_t* smem) {
  if (N < 1 || nst < 1) return false;
  const bool norm = prec_has_norm(prec);
  const int E = prec_complex_bytes(prec);
  const int hx = geo.hx;
  // TMA: 16-byte aligned row starts and strides, box extents <= 256
  if ((nrhs * E) % 16 || (hx * E) % 16 || hx > 256 || 4 * N > 256 || N * N > 256) return false;
  if ((int64_t)geo.vh * nrhs * E / 4 >= (1ll << 32) || (int64_t)geo.vh * E / 4 >= (1ll << 32)) return false;
  static int smem_max = 0;
  if (!smem_max) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
      return false;
  }
  for (int c = (rcta > 0 ? rcta : nrhs); c >= R; c--) {
    if (nrhs % c || c % R || (c * E) % 16 || c * E / 4 > 256) {
      if (rcta > 0) return false;
      continue;
    }
    const int cons = (hx * (c / R) + 31) / 32 * 32;
    const size_t spin = (size_t)c * E * hx * 4 * N, link = (size_t)hx * N * N * E;
    const size_t nb = norm ? (size_t)c * 4 * hx : 0;  // c * 4 is a multiple of 16 here
    const size_t stage = align128(spin) + (nb ? align128(nb) : 0) + 2 * (size_t)align128(link);
    const size_t need = (size_t)nst * stage + 16 * (size_t)nst;
    if (cons + 32 > 512 || need > (size_t)smem_max) {
      if (rcta > 0) return false;
      continue;
    }
    T->rcta = c;
    T->chunks = nrhs / c;
    T->rows = geo.vh / hx;
    T->ntiles = T->rows * T->chunks;
    T->spin_bytes = (uint32_t)spin;
    T->norm_bytes = (uint32_t)nb;
    T->link_bytes = (uint32_t)link;
    T->spin_stride = align128(spin);
    T->norm_stride = nb ? align128(nb) : 0;
    T->link_stride = align128(link);
    T->stage_bytes = (uint32_t)stage;
    *threads = cons + 32;
    *smem = need;
    return true;
  }
  return false;
}

bool tma_pointers_ok(const DslashArgs& A) {
  return (reinterpret_cast<uintptr_t>(A.in) % 16) == 0 && (reinterpret_cast<uintptr_t>(A.gauge) % 16) == 0 &&
         (reinterpret_cast<uintptr_t>(A.in_norm) % 16) == 0;
}

int tma_grid(const void* kernel, int threads, size_t smem, int ntiles) {
  static std::mutex m;
  static std::map<std::pair<const void*, std::pair<int, size_t>>, int> cache;
  static int sms = 0;
  std::lock_guard<std::mutex> lk(m);
  if (!sms) {
    int dev = 0;
    QCU_CHECK_CUDA(cudaGetDevice(&dev));
    QCU_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  }
  auto k = std::make_pair(kernel, std::make_pair(threads, smem));
  auto it = cache.find(k);
  int occ = 0;
  if (it == cache.end()) {
    QCU_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, smem));
    cache[k] = occ;
  } else {
    occ = it->second;
  }
  QCU_REQUIRE(occ >= 1, QCU_ERR_UNSUPPORTED, "staged dslash does not fit on an SM");
  return std::min(ntiles, occ * sms);
}

void register_tma(int prec, int N, int R, int nst, TmaLauncher fn) {
  std::lock_guard<std::mutex> lk(registry_mutex());
  registry()[key(prec, N, R, nst)] = fn;
}

TmaLauncher find_tma(int prec, int N, int R, int nst) {
  std::lock_guard<std::mutex> lk(registry_mutex());
  auto it = registry().find(key(prec, N, R, nst));
  return it == registry().end() ? nullptr : it->second;
}

int tma_options(int prec, int N, int* R, int* nst, int max) {
  int n = 0;
  for (int r = 1; r <= 8; r++)
    for (int s = 1; s <= 6; s++)
      if (n < max && find_tma(prec, N, r, s)) {
        R[n] = r;
        nst[n] = s;
        n++;
      }
  return n;
}

}  // namespace qcu
