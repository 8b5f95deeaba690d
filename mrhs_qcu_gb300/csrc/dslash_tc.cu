// Host side of the tensor-core dslash (see dslash_tc.h) and its instances.
#include <algorithm>
#include <map>
#include <mutex>

#include "dslash_tc.h"

namespace qcu {
namespace {

std::map<int, TcLauncher>& registry() {
  static std::map<int, TcLauncher> r;
  return r;
}
std::mutex& registry_mutex() {
  static std::mutex m;
  return m;
}

struct RegisterTc {
  RegisterTc() {
    register_tc(PREC_BF16, 4, 1, &launch_wilson_tc<4, 0>);
    register_tc(PREC_BF16, 5, 1, &launch_wilson_tc<5, 0>);
    register_tc(PREC_BF16, 6, 1, &launch_wilson_tc<6, 0>);
    register_tc(PREC_BF16, 7, 1, &launch_wilson_tc<7, 0>);
    register_tc(PREC_BF16, 8, 1, &launch_wilson_tc<8, 0>);
    register_tc(PREC_BF16, 4, 2, &launch_wilson_tc<4, 2>);
    register_tc(PREC_BF16, 6, 2, &launch_wilson_tc<6, 2>);
    register_tc(PREC_BF16, 8, 2, &launch_wilson_tc<8, 2>);
    register_tc(PREC_BF16, 4, 3, &launch_wilson_tc<4, 3>);
    register_tc(PREC_BF16, 6, 3, &launch_wilson_tc<6, 3>);
    register_tc(PREC_BF16, 8, 3, &launch_wilson_tc<8, 3>);
  }
} register_tc_instances;

}  // namespace

bool tc_plan(int prec, int N, const Geometry& geo, int nrhs, int nst, TcDslashArgs* T, size_t* smem) {
  if (prec != PREC_BF16 || N < 4 || N > 8 || nrhs < 1 || nst < 0) return false;
  // 32-bit element offsets into the field and the gauge
  if ((int64_t)4 * N * geo.vh * nrhs >= (1ll << 32) || (int64_t)8 * N * N * geo.vh >= (1ll << 32)) return false;
  int rt = 64;
  while (nrhs % rt) rt--;
  if (nst > 0 && (nrhs % 4 || rt % 4)) return false;  // 16-byte TMA rows
  const int64_t ntiles = (int64_t)geo.vh * (nrhs / rt);
  if (ntiles >= (1ll << 31)) return false;
  T->rt = rt;
  T->chunks = nrhs / rt;
  T->ntiles = (int)ntiles;
  T->spin_bytes = T->stage_bytes = 0;
  *smem = tc::kSmemBytes;
  if (nst > 0) {
    T->spin_bytes = (uint32_t)(4 * N * rt * 4);
    T->stage_bytes = (T->spin_bytes + 127u) / 128u * 128u;
    *smem = (size_t)tc::kRingOffset + (size_t)nst * T->stage_bytes;
  }
  return true;
}

int tc_ring_stages(int variant) { return variant >= 2 && variant <= 3 ? variant : 0; }

bool tcs_plan(const DslashArgs& A, int N, TcsDslashArgs* T, CUtensorMap* map_in) {
  const Geometry& geo = A.geo;
  const int nrhs = A.nrhs;
  if (N < 2 || N > 8 || nrhs < 1 || nrhs % 4 || !A.gauge_tc) return false;
  if (((uintptr_t)A.in | (uintptr_t)A.gauge_tc) % 16) return false;
  // 32-bit BF16 scalar offsets into the field (2 per complex) and element offsets into the gauge
  if ((int64_t)8 * N * geo.vh * nrhs >= (1ll << 32) || (int64_t)8 * N * N * geo.vh >= (1ll << 32)) return false;
  int rt = 64;
  while (nrhs % rt || rt % 4) rt--;
  const int64_t ntiles = (int64_t)geo.vh * (nrhs / rt);
  if (ntiles >= (1ll << 31)) return false;
  // tiles of 64 RHS: one copy per hop brings both halves (5-D map), else one per half
  T->fused = rt == 64 && tma_encode_field_swizzled_halves(map_in, A.in, nrhs, geo.vh, N, A.site_major != 0);
  if (!T->fused && !tma_encode_field_swizzled(map_in, A.in, nrhs, geo.vh, N, A.site_major != 0)) return false;
  T->cstr = (uint32_t)(A.site_major ? nrhs : geo.vh * nrhs);
  T->sstr = (uint32_t)(A.site_major ? 4 * N * nrhs : nrhs);
  T->rt = rt;
  T->chunks = nrhs / rt;
  T->ntiles = (int)ntiles;
  T->halves = rt > 32 ? 2 : 1;
  return true;
}

// CTAs per SM from the kernel's registers and shared memory (the runtime's
// occupancy query reports 1 for kernels that allocate tensor memory), capped
// by the 512 tensor-memory columns.
int tc_grid(const void* kernel, int ntiles, size_t smem, int tmem_cols, int threads) {
  static std::mutex m;
  static std::map<std::pair<const void*, size_t>, int> cache;
  static int sms = 0, smem_sm = 0, reserved = 0, regs_sm = 0, thr_sm = 0;
  std::lock_guard<std::mutex> lk(m);
  if (!sms) {
    int dev = 0;
    QCU_CHECK_CUDA(cudaGetDevice(&dev));
    QCU_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    QCU_CHECK_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    QCU_CHECK_CUDA(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev));
    QCU_CHECK_CUDA(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev));
    QCU_CHECK_CUDA(cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev));
  }
  auto it = cache.find(std::make_pair(kernel, smem));
  int occ = 0;
  if (it == cache.end()) {
    cudaFuncAttributes fa;
    QCU_CHECK_CUDA(cudaFuncGetAttributes(&fa, kernel));
    const int regs = (fa.numRegs + 7) / 8 * 8;  // allocation granularity
    const int by_smem = smem_sm / ((int)smem + (int)fa.sharedSizeBytes + reserved);
    const int by_regs = regs_sm / (std::max(regs, 1) * threads);
    const int by_thr = thr_sm / threads;
    occ = std::min(std::min(by_smem, by_regs), std::min(by_thr, 512 / std::max(tmem_cols, 32)));
    cache[std::make_pair(kernel, smem)] = occ;
  } else {
    occ = it->second;
  }
  QCU_REQUIRE(occ >= 1, QCU_ERR_UNSUPPORTED, "tensor-core dslash does not fit on an SM");
  return std::min(ntiles, occ * sms);
}

// one key per (precision, N <= 15, variant <= 15)
static int tc_key(int prec, int N, int variant) { return (prec * 16 + N) * 16 + variant; }

void register_tc(int prec, int N, int variant, TcLauncher fn) {
  std::lock_guard<std::mutex> lk(registry_mutex());
  registry()[tc_key(prec, N, variant)] = fn;
}

TcLauncher find_tc(int prec, int N, int variant) {
  std::lock_guard<std::mutex> lk(registry_mutex());
  auto it = registry().find(tc_key(prec, N, variant));
  return it == registry().end() ? nullptr : it->second;
}

}  // namespace qcu
