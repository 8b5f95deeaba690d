// Dslash registry and launch (see dslash.h).
#include <algorithm>
#include <cstdlib>
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
int key(int prec, int N, int R, int minb, int pk, int rc, int lt = 0) {
  return (((((prec * 16 + N) * 16 + R) * 8 + minb) * 2 + pk) * 2 + rc) * 2 + lt;
}
std::map<int, SegmentsLauncher>& seg_registry() {
  static std::map<int, SegmentsLauncher> r;
  return r;
}
}  // namespace

void register_segments(int prec, int N, int R, int minb, int pk, int rc, SegmentsLauncher fn) {
  std::lock_guard<std::mutex> lk(registry_mutex());
  seg_registry()[key(prec, N, R, minb, pk, rc)] = fn;
}

SegmentsLauncher find_segments(int prec, int N, int R, int minb, int pk, int rc) {
  std::lock_guard<std::mutex> lk(registry_mutex());
  auto it = seg_registry().find(key(prec, N, R, minb, pk, rc));
  return it == seg_registry().end() ? nullptr : it->second;
}

int segments_options(int prec, int N, int* out, int max) {
  int n = 0;
  for (int R = 1; R <= 8; R++)
    for (int m = 1; m <= 7; m++)
      for (int pk = 0; pk < 2; pk++)
        for (int rc = 0; rc < 2; rc++)
          if (n < max && find_segments(prec, N, R, m, pk, rc)) {
            out[4 * n] = R;
            out[4 * n + 1] = m;
            out[4 * n + 2] = pk;
            out[4 * n + 3] = rc;
            n++;
          }
  return n;
}

void register_dslash(int prec, int N, int R, int minb, int pk, int rc, int lt, DslashLauncher fn) {
  std::lock_guard<std::mutex> lk(registry_mutex());
  registry()[key(prec, N, R, minb, pk, rc, lt)] = fn;
}

void register_dslash(int prec, int N, int R, int minb, int pk, int rc, DslashLauncher fn) {
  register_dslash(prec, N, R, minb, pk, rc, 0, fn);
}

void register_dslash(int prec, int N, int R, int minb, int pk, DslashLauncher fn) {
  register_dslash(prec, N, R, minb, pk, 0, fn);
}

DslashLauncher find_dslash(int prec, int N, int R, int minb, int pk, int rc, int lt) {
  std::lock_guard<std::mutex> lk(registry_mutex());
  auto it = registry().find(key(prec, N, R, minb, pk, rc, lt));
  return it == registry().end() ? nullptr : it->second;
}

int dslash_r_options(int prec, int N, int* out, int max) {
  int n = 0;
  for (int R = 8; R >= 1 && n < max; R--)
    if (find_dslash(prec, N, R)) out[n++] = R;
  return n;
}

int dslash_minb_options(int prec, int N, int R, int pk, int* out, int max, int rc, int lt) {
  int n = 0;
  for (int m = 1; m <= 7 && n < max; m++)
    if (find_dslash(prec, N, R, m, pk, rc, lt)) out[n++] = m;
  return n;
}

bool tma_runs(const DslashArgs& A, int prec, int N, const DslashConfig& cfg) {
  if (cfg.tma <= 0 || A.nrhs % cfg.R || !find_tma(prec, N, cfg.R, cfg.tma) || !tma_pointers_ok(A)) return false;
  TmaDslashArgs T;
  int threads = 0;
  size_t smem = 0;
  return tma_plan(prec, N, A.geo, A.nrhs, cfg.R, cfg.tma, cfg.rcta, &T, &threads, &smem);
}

bool tc_runs(const DslashArgs& A_in, int prec, int N, int variant) {
  TcDslashArgs T;
  size_t smem = 0;
  if (!find_tc(prec, N, variant)) return false;
  DslashArgs A = A_in;
  A.site_major = prec_site_major(prec) ? 1 : 0;
  if (variant >= 4) {
    TcsDslashArgs T4;
    CUtensorMap m;
    return tcs_plan(A, N, &T4, &m) && T4.halves <= tcs_halves(variant);
  }
  return (variant < 2 || (uintptr_t)A.in % 16 == 0) &&
         tc_plan(prec, N, A.geo, A.nrhs, tc_ring_stages(variant), &T, &smem);
}

void plan_site_order(DslashArgs& B, int prec, int N) {
  // Measured at 32^3x64 FP32 SU(3) (register kernel, G site*RHS/s): nrhs 12
  // field order 17.8, slabs of 16 / 8 / 4 planes 19.0 / 19.0 / 18.5; nrhs 24
  // 15.9, 17.8 / 19.1 / 18.8.  The best slab keeps three slab-slices of input
  // and output within 28-57 MB; thinner slabs re-read more of their z faces.
  const Geometry& g = B.geo;
  const int64_t site_bytes = (int64_t)2 * 4 * N * B.nrhs * prec_complex_bytes(prec);  // in + out
  const int64_t field_bytes = site_bytes * g.vh;
  B.zb = 0;
  B.stream_out = field_bytes > ((int64_t)96 << 20) ? 1 : 0;  // larger than L2: the output is not re-read from it
  if (field_bytes <= ((int64_t)96 << 20)) return;
  int zb = g.L[2];
  while (zb > 1 && (int64_t)3 * g.plane * zb * site_bytes > ((int64_t)64 << 20)) {
    int d = zb - 1;
    while (d > 1 && g.L[2] % d) d--;  // the next smaller divisor of Lz
    zb = d;
  }
  // slabs thinner than 4 planes re-read more of their z faces than the field
  // order loses to L2 (2 / zb of the input per launch)
  if (zb < 4) zb = g.L[2];
  // QCU_DSLASH_ZSLAB=<planes> overrides the choice (0: the field's order)
  if (const char* e = getenv("QCU_DSLASH_ZSLAB")) {
    const int v = atoi(e);
    zb = (v > 0 && g.L[2] % v == 0) ? v : g.L[2];
  }
  if (zb >= g.L[2]) return;  // whole t-slices already fit
  B.zb = (uint32_t)zb;
  B.div_plane = FastDiv((uint32_t)g.plane);
  B.div_zb = FastDiv((uint32_t)zb);
  B.div_lt = FastDiv((uint32_t)g.L[3]);
}

namespace {
DslashConfig no_launch() {
  DslashConfig c;
  c.R = c.block = c.minb = 0;
  return c;
}
thread_local DslashConfig g_last_launched = no_launch();  // the shape last launched on this thread
}

DslashConfig last_launched_dslash() { return g_last_launched; }

void launch_dslash(const DslashArgs& A_in, int prec, int N, const DslashConfig& cfg_in, cudaStream_t st) {
  DslashConfig cfg = cfg_in;
  DslashArgs A = A_in;
  A.site_major = prec_site_major(prec) ? 1 : 0;
  if (A.site_major && !(cfg.tc >= 4 && tc_runs(A, prec, N, cfg.tc))) {
    // site-major fields have only the spinor-operand tensor-core kernels: the first that runs
    cfg = DslashConfig{};
    for (int v = 4; v <= kTcVariants && !cfg.tc; v++)
      if (tc_runs(A, prec, N, v)) cfg.tc = v;
    QCU_REQUIRE(cfg.tc, QCU_ERR_UNSUPPORTED,
                "site-major BF16 fields need the tensor-core dslash: nrhs a multiple of 4, N = 2..8, 16-byte "
                "aligned fields");
  }
  if (cfg.tc && tc_runs(A, prec, N, cfg.tc)) {
    DslashArgs B = A;
    B.af = (float)A.a;
    B.bf = (float)A.b;
    find_tc(prec, N, cfg.tc)(B, st);
    QCU_CHECK_CUDA(cudaGetLastError());
    g_last_launched = DslashConfig{};
    g_last_launched.R = 1, g_last_launched.tc = cfg.tc;
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
      g_last_launched = DslashConfig{};
      g_last_launched.R = cfg.R, g_last_launched.tma = cfg.tma, g_last_launched.rcta = cfg.rcta;
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
  if (cfg.rc && (!A.gauge12 || !find_dslash(prec, N, cfg.R, cfg.minb, cfg.pk, 1, cfg.lt))) {
    // no two-row gauge for this field (not SU(3) to rounding): the full links
    cfg.rc = 0;
    if (!find_dslash(prec, N, cfg.R, cfg.minb, cfg.pk, 0, cfg.lt)) cfg.minb = 1, cfg.pk = 0, cfg.lt = 0;
  }
  if (cfg.lt && !tmalink_runs(A, cfg.R, prec_complex_bytes(prec), cfg.rc ? (N - 1) * N : N * N)) {
    cfg.lt = 0;  // arguments the link-staged kernel cannot take: the register kernel of the same shape
    if (!find_dslash(prec, N, cfg.R, cfg.minb, cfg.pk, cfg.rc)) cfg.minb = 1, cfg.pk = 0;
  }
  DslashLauncher fn = find_dslash(prec, N, cfg.R, cfg.minb, cfg.pk, cfg.rc, cfg.lt);
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
  if (!cfg.lt) plan_site_order(B, prec, N);  // the link-staged kernel walks x-rows in its own order
  fn(B, cfg.block, st);
  QCU_CHECK_CUDA(cudaGetLastError());
  cfg.tma = cfg.rcta = cfg.tc = 0;
  g_last_launched = cfg;
}

int launch_dslash_segments(const std::vector<DslashArgs>& all, int prec, int N, const DslashConfig& cfg_in,
                           cudaStream_t st, std::vector<int>* misfits) {
  DslashConfig cfg = cfg_in;
  const int R = (cfg.tc || cfg.tma > 0) ? 1 : cfg.R;  // the staged and tensor-core kernels take any nrhs here
  std::vector<DslashArgs> segs;
  bool all_rc = true;
  for (size_t i = 0; i < all.size(); i++) {
    if (all[i].nrhs % R) {
      misfits->push_back((int)i);
      continue;
    }
    segs.push_back(all[i]);
    all_rc &= all[i].gauge12 != nullptr;
  }
  if (segs.empty()) return 0;
  if (cfg.rc && !all_rc) cfg.rc = 0;
  SegmentsLauncher fn = (cfg.tma <= 0 && cfg.tc == 0) ? find_segments(prec, N, cfg.R, cfg.minb, cfg.pk, cfg.rc)
                                                      : nullptr;
  if (!fn) {  // no work-list form of this shape: one launch per segment
    for (const DslashArgs& A : segs) launch_dslash(A, prec, N, cfg, st);
    return (int)segs.size();
  }
  QCU_REQUIRE(cfg.block >= 32 && cfg.block <= 256 && cfg.block % 32 == 0, QCU_ERR_INVALID_ARGUMENT,
              "dslash block size must be a multiple of 32 in 32..256");
  int launches = 0;
  for (size_t base = 0; base < segs.size(); base += kMaxHopSegments) {
    HopSegments S;
    S.count = (int)std::min<size_t>(kMaxHopSegments, segs.size() - base);
    int64_t blocks = 0;
    for (int i = 0; i < S.count; i++) {
      DslashArgs B = segs[base + i];
      QCU_REQUIRE((int64_t)B.geo.vh * (B.nrhs / cfg.R) < (1ll << 31), QCU_ERR_INVALID_ARGUMENT,
                  "lattice x nrhs too large for one launch");
      QCU_REQUIRE((int64_t)4 * N * B.geo.vh * B.nrhs < (1ll << 32) && (int64_t)8 * N * N * B.geo.vh < (1ll << 32),
                  QCU_ERR_INVALID_ARGUMENT, "field too large for 32-bit element offsets");
      QCU_REQUIRE((int64_t)B.geo.vh * B.nrhs * prec_complex_bytes(prec) < (1ll << 32), QCU_ERR_INVALID_ARGUMENT,
                  "field component stride must stay below 4 GB");
      B.div_groups = FastDiv((uint32_t)(B.nrhs / cfg.R));
      B.af = (float)B.a;
      B.bf = (float)B.b;
      plan_site_order(B, prec, N);
      S.A[i] = B;
      blocks += ((int64_t)B.geo.vh * (B.nrhs / cfg.R) + cfg.block - 1) / cfg.block;
    }
    QCU_REQUIRE(blocks < (1ll << 31), QCU_ERR_INVALID_ARGUMENT, "work list too large for one launch");
    fn(S, cfg.block, st);
    QCU_CHECK_CUDA(cudaGetLastError());
    launches++;
  }
  return launches;
}

}  // namespace qcu
