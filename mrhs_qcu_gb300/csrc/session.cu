// Session, hop operator and autotuner implementation (see session.h).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <new>
#include <sstream>

#include "session.h"
#include "clover.h"
#include "dslash_tc.h"
#include "dslash_tma.h"

namespace qcu {

// ---------------------------------------------------------------------------
void* DeviceBuffer::ensure(size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (bytes > bytes_) {
    release();
    const cudaError_t e = cudaMalloc(&p_, bytes);
    if (e != cudaSuccess) {
      p_ = nullptr;
      // clear the runtime's last error, so the next launch check does not report this failure again
      (void)cudaGetLastError();
      QCU_CHECK_CUDA(e);
    }
    bytes_ = bytes;
  }
  return p_;
}

void DeviceBuffer::release() {
  if (p_) cudaFree(p_);
  p_ = nullptr;
  bytes_ = 0;
}

size_t Workspace::total_bytes() const {
  size_t s = 0;
  for (auto& kv : bufs_) s += kv.second.bytes();
  return s;
}

void inject_failure(const char* site) {
  const char* e = getenv("QCU_INJECT_FAILURE");
  if (e && strcmp(e, site) == 0) throw std::bad_alloc();
}

// ---------------------------------------------------------------------------
Autotuner& global_tuner() {
  static Autotuner t;
  return t;
}

bool Autotuner::enabled() const {
  const char* e = getenv("QCU_TUNE");
  return !(e && e[0] == '0');
}

std::string Autotuner::key(int prec, int N, int nrhs, int vh) const {
  std::ostringstream o;
  o << prec << ":" << N << ":" << nrhs << ":" << vh;
  return o.str();
}

void Autotuner::load_file() {
  file_loaded_ = true;
  const char* path = getenv("QCU_TUNE_CACHE");
  if (!path) return;
  std::ifstream in(path);
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    std::string k;
    DslashConfig c;
    if (!(ls >> k >> c.R >> c.block >> c.minb >> c.pk)) continue;
    if (!(ls >> c.tma >> c.rcta)) c.tma = c.rcta = 0;
    if (!(ls >> c.tc)) c.tc = 0;
    if (!(ls >> c.rc)) c.rc = 0;
    if (!(ls >> c.lt)) c.lt = 0;
    cache_[k] = c;
  }
}

void Autotuner::save_file() {
  const char* path = getenv("QCU_TUNE_CACHE");
  if (!path) return;
  std::ofstream out(path);
  for (auto& kv : cache_)
    out << kv.first << " " << kv.second.R << " " << kv.second.block << " " << kv.second.minb << " " << kv.second.pk
        << " " << kv.second.tma << " " << kv.second.rcta << " " << kv.second.tc << " " << kv.second.rc << " "
        << kv.second.lt << "\n";
}

DslashConfig Autotuner::lookup(int prec, int N, int nrhs, int vh, bool* found) {
  std::lock_guard<std::mutex> lk(m_);
  // QCU_DSLASH_CONFIG="R,block[,reg_cap[,packed[,stages[,rcta[,tensor[,recon[,linktma]]]]]]]" pins the
  // kernel shape (profiling, sweeps); stages > 0 selects the TMA-staged kernel, tensor = 1 the tensor-core
  // kernel (the other fields are then ignored); recon = 1 the register kernel on two-row SU(3) links;
  // linktma = 1 the register kernel with its links staged by TMA
  if (const char* f = getenv("QCU_DSLASH_CONFIG")) {
    DslashConfig c;
    const int got = sscanf(f, "%d,%d,%d,%d,%d,%d,%d,%d,%d", &c.R, &c.block, &c.minb, &c.pk, &c.tma, &c.rcta, &c.tc,
                           &c.rc, &c.lt);
    if (got < 8) c.rc = 0;
    if (got < 9) c.lt = 0;
    const bool tensor = got >= 7 && c.tc >= 1 && find_tc(prec, N, c.tc);
    const bool staged = !tensor && got >= 5 && c.tma > 0 && c.R >= 1 && nrhs % c.R == 0 &&
                        find_tma(prec, N, c.R, c.tma);
    const bool plain = !tensor && got >= 2 && c.tma <= 0 && c.R >= 1 && nrhs % c.R == 0 &&
                       find_dslash(prec, N, c.R, c.minb, c.pk, c.rc, c.lt) && c.block >= 32 && c.block <= 256 &&
                       c.block % 32 == 0;
    if (tensor || staged || plain) {
      if (!staged) c.tma = c.rcta = 0;
      if (!tensor) c.tc = 0;
      if (!plain) c.rc = c.lt = 0;
      *found = true;
      return c;
    }
  }
  if (!file_loaded_) load_file();
  auto it = cache_.find(key(prec, N, nrhs, vh));
  *found = it != cache_.end();
  return *found ? it->second : heuristic(prec, N, nrhs);
}

void Autotuner::store(int prec, int N, int nrhs, int vh, const DslashConfig& c) {
  std::lock_guard<std::mutex> lk(m_);
  cache_[key(prec, N, nrhs, vh)] = c;
  save_file();
}

bool Autotuner::layout_site_major(int N, int nrhs, int vh, bool* known) {
  std::lock_guard<std::mutex> lk(m_);
  auto it = layout_.find(key(PREC_BF16S, N, nrhs, vh));
  *known = it != layout_.end();
  return *known && it->second;
}

void Autotuner::store_layout(int N, int nrhs, int vh, bool site_major) {
  std::lock_guard<std::mutex> lk(m_);
  layout_[key(PREC_BF16S, N, nrhs, vh)] = site_major;
}

DslashConfig Autotuner::heuristic(int prec, int N, int nrhs) {
  DslashConfig c;
  if (prec_site_major(prec)) {  // only the spinor-operand tensor-core kernels take site-major fields
    c.tc = 4;
    return c;
  }
  int opts[8];
  const int n = dslash_r_options(prec, N, opts, 8);
  int want = prec == PREC_DOUBLE ? 1 : (prec == PREC_SINGLE ? 2 : 4);
  if (N > 4) want = 1;
  c.R = 1;
  for (int i = 0; i < n; i++)
    if (opts[i] <= want && nrhs % opts[i] == 0) {
      c.R = opts[i];
      break;
    }
  c.block = 128;
  return c;
}

DslashConfig Autotuner::tune(const DslashArgs& A, int prec, int N, cudaStream_t st) {
  if (getenv("QCU_DSLASH_CONFIG")) {
    bool pinned = false;
    DslashConfig c = lookup(prec, N, A.nrhs, A.geo.vh, &pinned);
    if (pinned) return c;
  }
  int opts[8];
  const int n = dslash_r_options(prec, N, opts, 8);
  const int blocks[] = {32, 64, 128, 256};
  cudaEvent_t e0, e1;
  QCU_CHECK_CUDA(cudaEventCreate(&e0));
  QCU_CHECK_CUDA(cudaEventCreate(&e1));
  DslashConfig best = heuristic(prec, N, A.nrhs);
  float best_ms = 1e30f;
  for (int i = 0; i < n; i++) {
    if (A.nrhs % opts[i]) continue;
    // scalar / packed FP32x2 arithmetic x full / two-row links x links from L1 / staged by TMA
    for (int v = 0; v < 8; v++) {
    const int pk = v & 1, rc = (v >> 1) & 1, lt = v >> 2;
    if (rc && !A.gauge12) continue;
    if (lt && !tmalink_runs(A, opts[i], prec_complex_bytes(prec), rc ? (N - 1) * N : N * N)) continue;
    int minbs[8];
    const int nm = dslash_minb_options(prec, N, opts[i], pk, minbs, 8, rc, lt);
    for (int j = 0; j < nm; j++)
      for (int b : blocks) {
        if (lt && b != blocks[0]) continue;  // the link-staged kernel's CTA is one x-row, whatever the block
        DslashConfig c;
        c.R = opts[i];
        c.block = b;
        c.minb = minbs[j];
        c.pk = pk;
        c.rc = rc;
        c.lt = lt;
        launch_dslash(A, prec, N, c, st);  // warm-up
        QCU_CHECK_CUDA(cudaEventRecord(e0, st));
        const int reps = 3;
        for (int k = 0; k < reps; k++) launch_dslash(A, prec, N, c, st);
        QCU_CHECK_CUDA(cudaEventRecord(e1, st));
        QCU_CHECK_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        QCU_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) {
          best_ms = ms;
          best = c;
        }
      }
    }
  }
  // the TMA-staged kernel, where these arguments fit it
  int tr[16], ts[16];
  const int nt = tma_options(prec, N, tr, ts, 16);
  for (int i = 0; i < nt; i++) {
    DslashConfig c;
    c.R = tr[i];
    c.tma = ts[i];
    if (!tma_runs(A, prec, N, c)) continue;
    launch_dslash(A, prec, N, c, st);  // warm-up
    QCU_CHECK_CUDA(cudaEventRecord(e0, st));
    const int reps = 3;
    for (int k = 0; k < reps; k++) launch_dslash(A, prec, N, c, st);
    QCU_CHECK_CUDA(cudaEventRecord(e1, st));
    QCU_CHECK_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    QCU_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best_ms) {
      best_ms = ms;
      best = c;
    }
  }
  // the tensor-core kernel, where these arguments fit it; at N <= 4 the
  // CUDA-core kernels were faster at every RHS count measured (16^3x32, nrhs
  // 16-64), so component-major fields do not time them there
  for (int variant = 1; variant <= kTcVariants; variant++) {
    if (!tc_runs(A, prec, N, variant)) continue;
    if (N <= 4 && !prec_site_major(prec)) continue;
    DslashConfig c;
    c.tc = variant;
    launch_dslash(A, prec, N, c, st);  // warm-up
    QCU_CHECK_CUDA(cudaEventRecord(e0, st));
    const int reps = 3;
    for (int k = 0; k < reps; k++) launch_dslash(A, prec, N, c, st);
    QCU_CHECK_CUDA(cudaEventRecord(e1, st));
    QCU_CHECK_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    QCU_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best_ms) {
      best_ms = ms;
      best = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  store(prec, N, A.nrhs, A.geo.vh, best);
  return best;
}

// ---------------------------------------------------------------------------
void WilsonHopOperator::Dslash(FieldView out, FieldView in, int parity, int dagger, int nInputs) {
  QCU_REQUIRE(out.nrhs == nInputs && in.nrhs == nInputs, QCU_ERR_INVALID_ARGUMENT, "Dslash: nInputs mismatch");
  s_.hop(out, in, FieldView{}, parity, dagger, 1.0, 0.0);
}

void WilsonHopOperator::DslashXpay(FieldView out, FieldView in, FieldView x, int parity, int dagger, int nInputs, double a,
                             double b) {
  QCU_REQUIRE(out.nrhs == nInputs && in.nrhs == nInputs && x.nrhs == nInputs, QCU_ERR_INVALID_ARGUMENT,
              "DslashXpay: nInputs mismatch");
  s_.hop(out, in, x, parity, dagger, a, b);
}

// ---------------------------------------------------------------------------
Session::Session(const int L[4], const int grid[4], int nColors) : tuner(global_tuner()) {
  inject_failure("session");
  for (int i = 0; i < 4; i++) {
    latt.dim[i] = L[i];
    proc.dim[i] = grid ? grid[i] : 1;
  }
  N = nColors;
  geo = make_geometry(L);
}

Session::~Session() {
  if (own_stream_) cudaStreamDestroy(own_stream_);
}

cudaStream_t Session::stream() {
  if (user_stream_) return user_stream_;
  if (!own_stream_)
    QCU_CHECK_CUDA(
        cudaStreamCreateWithFlags(&own_stream_, nonblocking_stream ? cudaStreamNonBlocking : cudaStreamDefault));
  return own_stream_;
}

void Session::sync() {
  QCU_CHECK_CUDA(cudaStreamSynchronize(stream()));
  QCU_REQUIRE(!tma_check_timeout(stream()), QCU_ERR_DEVICE_TIMEOUT,
              "a staged dslash kernel timed out waiting for its copies (results invalid)");
}

void Session::load_gauge(const void* caller_gauge, int lex) {
  QCU_REQUIRE(caller_gauge != nullptr, QCU_ERR_INVALID_ARGUMENT, "gauge pointer is null");
  const size_t bytes = (size_t)8 * geo.vh * N * N * 16;
  void* d = gauge_[PREC_DOUBLE].ensure(bytes);
  pack_gauge(PREC_DOUBLE, N, caller_gauge, lex, d, geo, stream());
  for (int p = 0; p < 5; p++) gauge_valid_[p] = gauge12_valid_[p] = false;
  gauge_tc_valid_ = false;
  gauge_valid_[PREC_DOUBLE] = true;
  su3_dev_ = -1.0;
  gauge_loaded_ = true;
}

const void* Session::gauge(int prec) {
  QCU_REQUIRE(gauge_loaded_, QCU_ERR_NO_GAUGE, "localGauge_ is nullptr, not loaded.\n");
  QCU_REQUIRE(prec_valid(prec), QCU_ERR_INVALID_ARGUMENT, "bad precision");
  if (prec == PREC_BF16S) prec = PREC_BF16;  // the field layout does not apply to links
  if (!gauge_valid_[prec]) {
    const int64_t count = (int64_t)8 * geo.vh * N * N;
    void* d = gauge_[prec].ensure((size_t)count * prec_complex_bytes(prec));
    // links are bounded by 1 in modulus, so 16-bit links carry no scale
    convert_gauge(gauge_[PREC_DOUBLE].get(), prec, d, count, stream());
    gauge_valid_[prec] = true;
  }
  return gauge_[prec].get();
}

const void* Session::gauge12(int prec) {
  QCU_REQUIRE(gauge_loaded_, QCU_ERR_NO_GAUGE, "localGauge_ is nullptr, not loaded.\n");
  QCU_REQUIRE(prec_valid(prec), QCU_ERR_INVALID_ARGUMENT, "bad precision");
  if (prec == PREC_BF16S) prec = PREC_BF16;
  if (N != 3) return nullptr;
  if (su3_dev_ < 0) {
    unsigned* scratch = static_cast<unsigned*>(su3_scratch_.ensure(16));
    su3_dev_ = su3_row_deviation(gauge_[PREC_DOUBLE].get(), geo.vh, scratch, stream());
  }
  // a reconstructed row must agree with the stored one to the rounding of the precision
  const double tol = prec == PREC_DOUBLE ? 1e-13 : (prec == PREC_SINGLE ? 1e-7 : 1e-4);
  if (!(su3_dev_ < tol)) return nullptr;
  if (!gauge12_valid_[prec]) {
    const size_t vhp = ((size_t)geo.vh + 31) / 32 * 32;  // the two-row layout's groups of 32 sites
    void* d = gauge12_[prec].ensure(48 * vhp * prec_complex_bytes(prec));
    compress_gauge_su3(gauge_[PREC_DOUBLE].get(), prec, d, geo.vh, stream());
    gauge12_valid_[prec] = true;
  }
  return gauge12_[prec].get();
}

const void* Session::gauge_tc() {
  QCU_REQUIRE(gauge_loaded_, QCU_ERR_NO_GAUGE, "localGauge_ is nullptr, not loaded.\n");
  if (!gauge_tc_valid_) {
    void* d = gauge_tc_.ensure(tc_links_bytes(geo.vh));
    gauge_tc_records_bf16(N, gauge_[PREC_DOUBLE].get(), d, geo, stream());
    gauge_tc_valid_ = true;
  }
  return gauge_tc_.get();
}

void Session::load_clover(const void* caller_clover) {
  QCU_REQUIRE(caller_clover != nullptr, QCU_ERR_INVALID_ARGUMENT, "clover pointer is null");
  const size_t bytes = (size_t)16 * geo.vh * N * N * 16;  // 2 parities x 2 blocks x (2N)^2 complex double
  void* d = clover_[PREC_DOUBLE].ensure(bytes);
  pack_clover(N, caller_clover, d, geo.vh, stream());
  void* di = cloverinv_[PREC_DOUBLE].ensure(bytes);
  int* flag = static_cast<int*>(clover_flag_.ensure(16));
  const bool ok = invert_clover(N, d, di, geo.vh, flag, stream());
  for (int p = 0; p < 5; p++) clover_valid_[p] = cloverinv_valid_[p] = false;
  clover_valid_[PREC_DOUBLE] = cloverinv_valid_[PREC_DOUBLE] = true;
  clover_loaded_ = ok;
  QCU_REQUIRE(ok, QCU_ERR_INVALID_ARGUMENT, "clover field has a singular block");
}

const void* Session::clover(int prec, bool inverse) {
  QCU_REQUIRE(clover_loaded_, QCU_ERR_NO_OPERATOR, "no clover field loaded");
  QCU_REQUIRE(prec_valid(prec), QCU_ERR_INVALID_ARGUMENT, "bad precision");
  QCU_REQUIRE(!prec_site_major(prec), QCU_ERR_UNSUPPORTED, "clover: site-major BF16 fields are not supported");
  DeviceBuffer* buf = inverse ? cloverinv_ : clover_;
  bool* valid = inverse ? cloverinv_valid_ : clover_valid_;
  if (!valid[prec]) {
    const int64_t count = (int64_t)16 * geo.vh * N * N;
    void* d = buf[prec].ensure((size_t)count * prec_complex_bytes(prec));
    convert_gauge(buf[PREC_DOUBLE].get(), prec, d, count, stream());
    valid[prec] = true;
  }
  return buf[prec].get();
}

void Session::clover_apply(FieldView out, FieldView in, FieldView x, int parity, bool inverse, double a, double b,
                           const int* mask, const float* a_rhs_f, const double* a_rhs_d) {
  QCU_REQUIRE(parity == 0 || parity == 1, QCU_ERR_INVALID_ARGUMENT, "parity must be 0 or 1");
  QCU_REQUIRE(out.prec == in.prec && (!x.data || x.prec == in.prec) && out.nrhs == in.nrhs,
              QCU_ERR_INVALID_ARGUMENT, "clover operands must share precision and nrhs");
  DslashArgs A;
  A.gauge = nullptr;
  A.in = in.data;
  A.in_norm = in.norm;
  A.out = out.data;
  A.out_norm = out.norm;
  A.x = x.data;
  A.x_norm = x.norm;
  A.mask = mask;
  A.a_rhs_f = a_rhs_f;
  A.a_rhs_d = a_rhs_d;
  A.a = a;
  A.b = b;
  A.geo = geo;
  A.nrhs = in.nrhs;
  A.parity = parity;
  A.dagger = 0;
  A.antiperiodic_t = 0;
  qcu::clover_apply(in.prec, N, A, clover(in.prec, inverse), stream());
}

FieldView Session::alloc_field(const std::string& name, int prec, int nrhs) {
  FieldView f;
  f.prec = prec;
  f.nrhs = nrhs;
  f.data = ws.get(name, field_bytes(prec, nrhs));
  if (prec_has_norm(prec)) f.norm = static_cast<float*>(ws.get(name + ".norm", norm_bytes(prec, nrhs)));
  return f;
}

bool Session::prefer_site_major(FieldView a, FieldView b) {
  const int nrhs = a.nrhs;
  if (!prec_bf16(a.prec) || b.nrhs != nrhs || nrhs % 4 || !tuner.enabled()) return false;
  bool known = false;
  const bool cached = tuner.layout_site_major(N, nrhs, geo.vh, &known);
  if (known) return cached;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  QCU_CHECK_CUDA(cudaStreamIsCapturing(stream(), &cs));
  if (cs != cudaStreamCaptureStatusNone) return false;
  // zero input (the bytes are the same in both layouts), then each layout's
  // tuned dslash: one untimed application (tunes it), three timed
  QCU_CHECK_CUDA(cudaMemsetAsync(a.data, 0, field_bytes(PREC_BF16, nrhs), stream()));
  cudaEvent_t e0, e1;
  QCU_CHECK_CUDA(cudaEventCreate(&e0));
  QCU_CHECK_CUDA(cudaEventCreate(&e1));
  float ms[2] = {0.f, 0.f};
  bool ok = true;
  for (int i = 0; i < 2 && ok; i++) {
    a.prec = b.prec = i ? PREC_BF16S : PREC_BF16;
    try {
      hop(b, a, FieldView{}, 0, 0, 1.0, 0.0);
      QCU_CHECK_CUDA(cudaEventRecord(e0, stream()));
      for (int k = 0; k < 3; k++) hop(b, a, FieldView{}, 0, 0, 1.0, 0.0);
      QCU_CHECK_CUDA(cudaEventRecord(e1, stream()));
      QCU_CHECK_CUDA(cudaEventSynchronize(e1));
      QCU_CHECK_CUDA(cudaEventElapsedTime(&ms[i], e0, e1));
    } catch (const Error& e) {
      if (e.code != QCU_ERR_UNSUPPORTED) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
      }
      ok = false;  // the site-major kernel cannot take these arguments
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const bool site = ok && ms[1] < 0.95f * ms[0];
  tuner.store_layout(N, nrhs, geo.vh, site);
  return site;
}

void Session::hop(FieldView out, FieldView in, FieldView x, int parity, int dagger, double a, double b,
                  const int* mask, const float* a_rhs_f, const double* a_rhs_d) {
  QCU_REQUIRE(parity == 0 || parity == 1, QCU_ERR_INVALID_ARGUMENT, "parity must be 0 or 1");
  QCU_REQUIRE(dagger == 0 || dagger == 1, QCU_ERR_INVALID_ARGUMENT, "daggerFlag must be 0 or 1");
  QCU_REQUIRE(out.prec == in.prec && (!x.data || x.prec == in.prec), QCU_ERR_INVALID_ARGUMENT,
              "dslash operands must share one precision");
  QCU_REQUIRE(out.nrhs == in.nrhs && (!x.data || x.nrhs == in.nrhs), QCU_ERR_INVALID_ARGUMENT,
              "dslash operands must share nrhs");
  DslashArgs A;
  A.gauge = gauge(in.prec);
  A.gauge12 = gauge12(in.prec);
  // BF16 RHS counts the spinor-operand tensor-core kernel takes
  if (prec_bf16(in.prec) && in.nrhs % 4 == 0) A.gauge_tc = gauge_tc();
  A.in = in.data;
  A.in_norm = in.norm;
  A.out = out.data;
  A.out_norm = out.norm;
  A.x = x.data;
  A.x_norm = x.norm;
  A.mask = mask;
  A.a_rhs_f = a_rhs_f;
  A.a_rhs_d = a_rhs_d;
  A.a = a;
  A.b = b;
  A.geo = geo;
  A.nrhs = in.nrhs;
  A.parity = parity;
  A.dagger = dagger;
  A.antiperiodic_t = antiperiodic_t ? 1 : 0;
  bool found = false;
  DslashConfig c = tuner.lookup(in.prec, N, in.nrhs, geo.vh, &found);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  QCU_CHECK_CUDA(cudaStreamIsCapturing(stream(), &cs));
  if (!found && tuner.enabled() && cs == cudaStreamCaptureStatusNone) c = tuner.tune(A, in.prec, N, stream());
  launch_dslash(A, in.prec, N, c, stream());
}

Blas& Session::blas() {
  if (!blas_) {
    const int max_blocks = 1024;
    double* p = static_cast<double*>(partials_.ensure((size_t)max_blocks * QCU_MAX_RHS * 2 * sizeof(double)));
    blas_.reset(new Blas(p, max_blocks));
  }
  return *blas_;
}

double* Session::scalars(size_t count) { return static_cast<double*>(scalars_.ensure(count * sizeof(double))); }

}  // namespace qcu
