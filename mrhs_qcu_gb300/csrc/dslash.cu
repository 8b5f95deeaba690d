// Dslash registry and launch (see dslash.h).
#include <map>
#include <mutex>

#include "dslash.h"
#include "dslash_tc.h"
#include "dslash_tma.h"

namespace qcu {
namespace {
std::map<int, DslashLauncher>& registry() {
  static std::map<int, DslashLauncher> r;
  return r;
}
std::mutex& registry_mutex() {
  static std::mutex m;
  return m;
}
int key(int prec, int N, int R, int minb, int pk, int rc) {
  return ((((prec * 16 + N) * 16 + R) * 8 + minb) * 2 + pk) * 2 + rc;
}
}  // namespace

void register_dslash(int prec, int N, int R, int minb, int pk, int rc, DslashLauncher fn) {
  std::lock_guard<std::mutex> lk(registry_mutex());
  registry()[key(prec, N, R, minb, pk, rc)] = fn;
}

void register_dslash(int prec, int N, int R, int minb, int pk, DslashLauncher fn) {
  register_dslash(prec, N, R, minb, pk, 0, fn);
}

DslashLauncher find_dslash(int prec, int N, int R, int minb, int pk, int rc) {
  std::lock_guard<std::mutex> lk(registry_mutex());
  auto it = registry().find(key(prec, N, R, minb, pk, rc));
  return it == registry().end() ? nullptr : it->second;
}

int dslash_r_options(int prec, int N, int* out, int max) {
  int n = 0;
  for (int R = 8; R >= 1 && n < max; R--)
    if (find_dslash(prec, N, R)) out[n++] = R;
  return n;
}

int dslash_minb_options(int prec, int N, int R, int pk, int* out, int max, int rc) {
  int n = 0;
  for (int m = 1; m <= 7 && n < max; m++)
    if (find_dslash(prec, N, R, m, pk, rc)) out[n++] = m;
  return n;
}

bool tma_runs(const DslashArgs& A, int prec, int N, const DslashConfig& cfg) {
  if (cfg.tma <= 0 || A.nrhs % cfg.R || !find_tma(prec, N, cfg.R, cfg.tma) || !tma_pointers_ok(A)) return false;
  TmaDslashArgs T;
  int threads = 0;
  size_t smem = 0;
  return tma_plan(prec, N, A.geo, A.nrhs, cfg.R, cfg.tma, cfg.rcta, &T, &threads, &smem);
}

bool tc_runs(const DslashArgs& A, int prec, int N, int variant) {
  TcDslashArgs T;
  size_t smem = 0;
  if (!find_tc(prec, N, variant)) return false;
  if (variant >= 4) {
    TcsDslashArgs T4;
    CUtensorMap m;
    return tcs_plan(A, N, &T4, &m);
  }
  return (variant < 2 || (uintptr_t)A.in % 16 == 0) &&
         tc_plan(prec, N, A.geo, A.nrhs, tc_ring_stages(variant), &T, &smem);
}

void launch_dslash(const DslashArgs& A, int prec, int N, const DslashConfig& cfg_in, cudaStream_t st) {
  DslashConfig cfg = cfg_in;
  if (cfg.tc && tc_runs(A, prec, N, cfg.tc)) {
    DslashArgs B = A;
    B.af = (float)A.a;
    B.bf = (float)A.b;
    find_tc(prec, N, cfg.tc)(B, st);
    QCU_CHECK_CUDA(cudaGetLastError());
    return;
  }
  if (cfg.tc) {  // arguments the tensor-core kernel cannot take: register kernel
    cfg = DslashConfig{};
    int opts[8];
    const int n = dslash_r_options(prec, N, opts, 8);
    for (int i = 0; i < n; i++)
      if (A.nrhs % opts[i] == 0 && opts[i] <= 2) {
        cfg.R = opts[i];
        break;
      }
  }
  if (cfg.tma > 0) {
    if (tma_runs(A, prec, N, cfg)) {
      QCU_REQUIRE((int64_t)A.geo.vh * A.nrhs * prec_complex_bytes(prec) < (1ll << 32), QCU_ERR_INVALID_ARGUMENT,
                  "field component stride must stay below 4 GB");
      DslashArgs B = A;
      B.af = (float)A.a;
      B.bf = (float)A.b;
      find_tma(prec, N, cfg.R, cfg.tma)(B, cfg.rcta, st);
      QCU_CHECK_CUDA(cudaGetLastError());
      return;
    }
    // arguments the staged kernel cannot take (e.g. a misaligned caller buffer): register kernel
    cfg = DslashConfig{};
    int opts[8];
    const int n = dslash_r_options(prec, N, opts, 8);
    for (int i = 0; i < n; i++)
      if (A.nrhs % opts[i] == 0 && opts[i] <= 2) {
        cfg.R = opts[i];
        break;
      }
  }
  if (cfg.rc && (!A.gauge12 || !find_dslash(prec, N, cfg.R, cfg.minb, cfg.pk, 1))) {
    // no two-row gauge for this field (not SU(3) to rounding): the full links
    cfg.rc = 0;
    if (!find_dslash(prec, N, cfg.R, cfg.minb, cfg.pk, 0)) cfg.minb = 1, cfg.pk = 0;
  }
  DslashLauncher fn = find_dslash(prec, N, cfg.R, cfg.minb, cfg.pk, cfg.rc);
  QCU_REQUIRE(fn != nullptr, QCU_ERR_UNSUPPORTED,
              std::string("no dslash kernel for precision ") + prec_name(prec) + ", N=" + std::to_string(N) +
                  ", R=" + std::to_string(cfg.R) + ", minb=" + std::to_string(cfg.minb) +
                  ", pk=" + std::to_string(cfg.pk));
  QCU_REQUIRE(cfg.block >= 32 && cfg.block <= 256 && cfg.block % 32 == 0, QCU_ERR_INVALID_ARGUMENT,
              "dslash block size must be a multiple of 32 in 32..256");
  QCU_REQUIRE(A.nrhs % cfg.R == 0, QCU_ERR_INVALID_ARGUMENT, "nrhs not a multiple of R");
  QCU_REQUIRE((int64_t)A.geo.vh * (A.nrhs / cfg.R) < (1ll << 31), QCU_ERR_INVALID_ARGUMENT,
              "lattice x nrhs too large for one launch");
  // the kernels index fields and links with 32-bit element offsets
  QCU_REQUIRE((int64_t)4 * N * A.geo.vh * A.nrhs < (1ll << 32) && (int64_t)8 * N * N * A.geo.vh < (1ll << 32),
              QCU_ERR_INVALID_ARGUMENT, "field too large for 32-bit element offsets");
  QCU_REQUIRE((int64_t)A.geo.vh * A.nrhs * prec_complex_bytes(prec) < (1ll << 32), QCU_ERR_INVALID_ARGUMENT,
              "field component stride must stay below 4 GB");
  DslashArgs B = A;
  B.div_groups = FastDiv((uint32_t)(A.nrhs / cfg.R));
  B.af = (float)A.a;
  B.bf = (float)A.b;
  fn(B, cfg.block, st);
  QCU_CHECK_CUDA(cudaGetLastError());
}

}  // namespace qcu
