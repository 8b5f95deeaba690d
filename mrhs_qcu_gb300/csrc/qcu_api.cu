// C ABI of libqcu.so: the reference's qcu.h entry points (src/qcu.cu:125-181
// of the reference) plus the extensions in qcu_gb300.h.
//
// The reference keeps one global Qcu object (src/qcu.cu:125); so does this
// library (g_session), guarded by a mutex.  Errors are recorded and printed
// instead of terminating the process (the reference's errorQcu / CHECK_CUDA
// call exit(1), include/qcu_macro.cuh:16-40); QCU_ABORT_ON_ERROR=1 restores
// that behaviour.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>

#pragma GCC visibility push(default)  // the public headers: exported
#include "../../include/qcu.h"
#include "../../include/qcu_gb300.h"
#pragma GCC visibility pop
#include "dslash_tc.h"
#include "dslash_tma.h"
#include "serve.h"
#include "session.h"

using qcu::Error;
using qcu::Session;

namespace {

std::mutex g_mutex;
std::unique_ptr<Session> g_session;
std::unique_ptr<Session> g_solver_session;  // private session of cg_inverter
cudaStream_t g_user_stream = nullptr;
int g_antiperiodic = 0;
thread_local int g_last_error = 0;
thread_local std::string g_last_message;

void record(int code, const std::string& msg) {
  g_last_error = code;
  g_last_message = msg;
  fprintf(stderr, "%s", msg.c_str());
  if (msg.empty() || msg.back() != '\n') fprintf(stderr, "\n");
  fprintf(stderr, "Error happened in libqcu (code %d)\n", code);
  const char* e = getenv("QCU_ABORT_ON_ERROR");
  if (e && e[0] == '1') exit(1);
}

template <typename F>
int guarded(F&& f) {
  std::lock_guard<std::mutex> lk(g_mutex);
  try {
    f();
    return QCU_OK;
  } catch (const Error& e) {
    record(e.code, e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    record(QCU_ERR_OUT_OF_MEMORY, "host allocation failed");
    return QCU_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    record(QCU_ERR_CUDA, e.what());
    return QCU_ERR_CUDA;
  }
}

// the same error handling without the global session lock (server calls,
// which block or run concurrently with the session API)
template <typename F>
int guarded_unlocked(F&& f) {
  try {
    f();
    return QCU_OK;
  } catch (const Error& e) {
    std::lock_guard<std::mutex> lk(g_mutex);
    record(e.code, e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    std::lock_guard<std::mutex> lk(g_mutex);
    record(QCU_ERR_OUT_OF_MEMORY, "host allocation failed");
    return QCU_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    std::lock_guard<std::mutex> lk(g_mutex);
    record(QCU_ERR_CUDA, e.what());
    return QCU_ERR_CUDA;
  }
}

Session& session() {
  QCU_REQUIRE(g_session != nullptr, QCU_ERR_NOT_INITIALIZED, "Qcu is not initialized.\n");
  return *g_session;
}

void check_lattice(const QcuParam* p) {
  QCU_REQUIRE(p != nullptr, QCU_ERR_INVALID_ARGUMENT, "QcuParam is null");
  for (int i = 0; i < 4; i++)
    QCU_REQUIRE(p->lattice_size[i] > 0, QCU_ERR_INVALID_ARGUMENT, "lattice sizes must be positive");
  QCU_REQUIRE(p->lattice_size[0] % 2 == 0, QCU_ERR_INVALID_ARGUMENT, "lattice X extent must be even");
  const long long v = (long long)p->lattice_size[0] * p->lattice_size[1] * p->lattice_size[2] * p->lattice_size[3];
  QCU_REQUIRE(v / 2 < (1ll << 30), QCU_ERR_INVALID_ARGUMENT, "lattice too large");
}

void apply_settings(Session& s) {
  s.antiperiodic_t = g_antiperiodic != 0;
  s.set_user_stream(g_user_stream);
}

// run the hopping term on caller-layout fermions through the session
void caller_dslash(Session& s, int prec, void* const* outs, void* const* ins, int n, int in_mode, int out_mode,
                   int parity, int dagger) {
  using namespace qcu;
  for (int base = 0; base < n; base += QCU_MAX_RHS) {
    const int m = std::min(QCU_MAX_RHS, n - base);
    PtrArray pin{}, pout{};
    for (int r = 0; r < m; r++) {
      pin.p[r] = ins[base + r];
      pout.p[r] = outs[base + r];
    }
    FieldView fin = s.alloc_field("abi.in", prec, m);
    FieldView fout = s.alloc_field("abi.out", prec, m);
    pack_fermions(prec, s.N, pin, in_mode, 1 - parity, fin.data, fin.norm, s.geo, m, s.stream());
    s.hop(fout, fin, FieldView{}, parity, dagger, 1.0, 0.0);
    unpack_fermions(prec, s.N, pout, out_mode, parity, fout.data, fout.norm, s.geo, m, s.stream());
  }
  s.sync();
}

}  // namespace

extern "C" {

// used by the C++ storage API (storage_api.cu) to report through the same channel
void qcu_record_error(int code, const char* msg) {
  std::lock_guard<std::mutex> lk(g_mutex);
  record(code, msg);
}

// ---- drop-in ABI (include/qcu.h) -------------------------------------------
void initGridSize(QcuGrid_t* grid, QcuParam* p_param, int nColors) {
  guarded([&] {
    check_lattice(p_param);
    QCU_REQUIRE(nColors >= 3 && nColors <= 8, QCU_ERR_UNSUPPORTED, "Now we only support 3-8 colors.\n");
    int g[4] = {1, 1, 1, 1};
    if (grid)
      for (int i = 0; i < 4; i++) g[i] = grid->grid_size[i];
    for (int i = 0; i < 4; i++)
      QCU_REQUIRE(g[i] == 1, QCU_ERR_UNSUPPORTED,
                  "process grids other than 1x1x1x1 are not supported (one GPU per process)");
    g_session.reset();
    g_session.reset(new Session(p_param->lattice_size, g, nColors));
    apply_settings(*g_session);
  });
}

void pushBackFermions(void* fermionOut, void* fermionIn) {
  guarded([&] {
    Session& s = session();
    QCU_REQUIRE(fermionOut && fermionIn, QCU_ERR_INVALID_ARGUMENT, "fermion pointers must not be null");
    s.queue.emplace_back(fermionOut, fermionIn);
  });
}

void startDslash(int parity, int daggerFlag) {
  guarded([&] {
    Session& s = session();
    QCU_REQUIRE(s.dirac != nullptr, QCU_ERR_NO_OPERATOR, "getDslash has not been called");
    QCU_REQUIRE(parity == 0 || parity == 1, QCU_ERR_INVALID_ARGUMENT, "parity must be 0 or 1");
    QCU_REQUIRE(daggerFlag == 0 || daggerFlag == 1, QCU_ERR_INVALID_ARGUMENT, "daggerFlag must be 0 or 1");
    std::vector<void*> outs, ins;
    for (auto& pr : s.queue) {
      outs.push_back(pr.first);
      ins.push_back(pr.second);
    }
    s.queue.clear();
    if (outs.empty()) return;
    caller_dslash(s, s.dirac->precision(), outs.data(), ins.data(), (int)outs.size(), qcu::SRC_EO_HALF,
                  qcu::SRC_EO_HALF, parity, daggerFlag);
  });
}

void loadQcuGauge(void* gauge) {
  guarded([&] {
    Session& s = session();
    s.load_gauge(gauge, 0);
    s.sync();
  });
}

void getDslash(int dslashType, double mass, int nColors, int nInputs, int floatPrecision) {
  guarded([&] {
    Session& s = session();
    QCU_REQUIRE(s.gauge_loaded(), QCU_ERR_NO_GAUGE, "localGauge_ is nullptr, not loaded.\n");
    QCU_REQUIRE(dslashType == 0, QCU_ERR_UNSUPPORTED, "Now we only support Wilson dslash.\n");
    QCU_REQUIRE(nColors == s.N, QCU_ERR_INVALID_ARGUMENT, "nColors differs from initGridSize");
    QCU_REQUIRE(qcu::prec_valid(floatPrecision), QCU_ERR_UNSUPPORTED,
                "floatPrecision must be 0 (half), 1 (single), 2 (double) or 4 (bf16)");
    QCU_REQUIRE(nInputs >= 0, QCU_ERR_INVALID_ARGUMENT, "nInputs must not be negative");
    s.dirac.reset(new qcu::WilsonHopOperator(s, mass, nColors, floatPrecision, dslashType));
    s.gauge(floatPrecision);  // convert the resident gauge once
    s.sync();
  });
}

void dslashQcu(void* fermion_out, void* fermion_in, void* gauge, QcuParam* param, int parity) {
  guarded([&] {
    check_lattice(param);
    QCU_REQUIRE(fermion_out && fermion_in && gauge, QCU_ERR_INVALID_ARGUMENT, "null pointer");
    int g[4] = {1, 1, 1, 1};
    Session s(param->lattice_size, g, 3);
    apply_settings(s);
    s.load_gauge(gauge, 0);
    caller_dslash(s, qcu::PREC_DOUBLE, &fermion_out, &fermion_in, 1, qcu::SRC_EO_HALF, qcu::SRC_EO_HALF, parity, 0);
  });
}

void fullDslashQcu(void* fermion_out, void* fermion_in, void* gauge, QcuParam* param, int dagger_flag) {
  guarded([&] {
    check_lattice(param);
    QCU_REQUIRE(fermion_out && fermion_in && gauge, QCU_ERR_INVALID_ARGUMENT, "null pointer");
    int g[4] = {1, 1, 1, 1};
    Session s(param->lattice_size, g, 3);
    apply_settings(s);
    s.load_gauge(gauge, 0);
    for (int p = 0; p < 2; p++)
      caller_dslash(s, qcu::PREC_DOUBLE, &fermion_out, &fermion_in, 1, qcu::SRC_EO_FULL, qcu::SRC_EO_FULL, p,
                    dagger_flag);
  });
}

void cg_inverter(void* x_vector, void* b_vector, void* gauge, QcuParam* param, double p_max_prec, double p_kappa) {
  guarded([&] {
    check_lattice(param);
    QCU_REQUIRE(x_vector && b_vector && gauge, QCU_ERR_INVALID_ARGUMENT, "null pointer");
    const int N = g_session ? g_session->N : 3;
    bool reuse = g_solver_session && g_solver_session->N == N;
    for (int i = 0; reuse && i < 4; i++) reuse = g_solver_session->latt.dim[i] == param->lattice_size[i];
    if (!reuse) {
      int g[4] = {1, 1, 1, 1};
      g_solver_session.reset(new Session(param->lattice_size, g, N));
    }
    Session& s = *g_solver_session;
    apply_settings(s);
    s.load_gauge(gauge, 0);
    qcu::SolveRequest q;
    q.kappa = p_kappa;
    q.tol = p_max_prec;
    q.inner_prec = qcu::PREC_SINGLE;
    q.src_mode = qcu::SRC_EO_FULL;
    qcu::SolveResult r = qcu::solve(s, &x_vector, &b_vector, 1, q);
    QCU_REQUIRE(r.converged[0], QCU_ERR_NOT_CONVERGED,
                "cg_inverter: not converged, true residual " + std::to_string(r.true_residual[0]));
  });
}

// ---- extensions (include/qcu_gb300.h) --------------------------------------
int qcuGetLastError(void) { return g_last_error; }
const char* qcuGetLastErrorString(void) { return g_last_message.c_str(); }
void qcuClearError(void) {
  g_last_error = 0;
  g_last_message.clear();
}
const char* qcuVersion(void) { return "mrhs_qcu_gb300 0.1 (sm_103a)"; }

int qcuSetAntiperiodicT(int flag) {
  return guarded([&] {
    g_antiperiodic = flag ? 1 : 0;
    if (g_session) g_session->antiperiodic_t = g_antiperiodic != 0;
  });
}

int qcuSetStream(void* stream) {
  return guarded([&] {
    g_user_stream = static_cast<cudaStream_t>(stream);
    if (g_session) g_session->set_user_stream(g_user_stream);
  });
}

int qcuSynchronize(void) {
  return guarded([&] { session().sync(); });
}

int qcuFieldBytes(int precision, int nrhs, size_t* data_bytes, size_t* norm_bytes) {
  return guarded([&] {
    Session& s = session();
    QCU_REQUIRE(qcu::prec_valid(precision), QCU_ERR_INVALID_ARGUMENT, "bad precision");
    QCU_REQUIRE(nrhs >= 1, QCU_ERR_INVALID_ARGUMENT, "nrhs must be positive");
    if (data_bytes) *data_bytes = s.field_bytes(precision, nrhs);
    if (norm_bytes) *norm_bytes = s.norm_bytes(precision, nrhs);
  });
}

int qcuPackFermions(void* dst, void* dst_norm, void* const* src, int nrhs, int src_mode, int parity, int precision) {
  return guarded([&] {
    Session& s = session();
    QCU_REQUIRE(nrhs >= 1 && nrhs <= qcu::QCU_MAX_RHS, QCU_ERR_INVALID_ARGUMENT, "nrhs must be in 1..256");
    QCU_REQUIRE(src_mode >= 0 && src_mode <= 2, QCU_ERR_INVALID_ARGUMENT, "bad source mode");
    QCU_REQUIRE(qcu::prec_valid(precision), QCU_ERR_INVALID_ARGUMENT, "bad precision");
    QCU_REQUIRE(!qcu::prec_has_norm(precision) || dst_norm, QCU_ERR_INVALID_ARGUMENT, "FP16 fields need a norm array");
    qcu::PtrArray p{};
    for (int r = 0; r < nrhs; r++) p.p[r] = src[r];
    qcu::pack_fermions(precision, s.N, p, src_mode, parity, dst, static_cast<float*>(dst_norm), s.geo, nrhs,
                       s.stream());
  });
}

int qcuUnpackFermions(void* const* dst, const void* src, const void* src_norm, int nrhs, int dst_mode, int parity,
                      int precision) {
  return guarded([&] {
    Session& s = session();
    QCU_REQUIRE(nrhs >= 1 && nrhs <= qcu::QCU_MAX_RHS, QCU_ERR_INVALID_ARGUMENT, "nrhs must be in 1..256");
    QCU_REQUIRE(dst_mode >= 0 && dst_mode <= 2, QCU_ERR_INVALID_ARGUMENT, "bad destination mode");
    QCU_REQUIRE(qcu::prec_valid(precision), QCU_ERR_INVALID_ARGUMENT, "bad precision");
    qcu::PtrArray p{};
    for (int r = 0; r < nrhs; r++) p.p[r] = dst[r];
    qcu::unpack_fermions(precision, s.N, p, dst_mode, parity, src, static_cast<const float*>(src_norm), s.geo, nrhs,
                         s.stream());
  });
}

int qcuLoadGaugeLex(void* gauge_lex) {
  return guarded([&] {
    Session& s = session();
    s.load_gauge(gauge_lex, 1);
    s.sync();
  });
}

int qcuLexToEo(void* eo_out, const void* lex_in, int ncomp) {
  return guarded([&] {
    Session& s = session();
    QCU_REQUIRE(ncomp == 4 * s.N, QCU_ERR_UNSUPPORTED, "ncomp must be 4*N (a fermion field)");
    qcu::PtrArray src{}, dst{};
    src.p[0] = lex_in;
    dst.p[0] = eo_out;
    qcu::FieldView f = s.alloc_field("lex.tmp", qcu::PREC_DOUBLE, 1);
    for (int p = 0; p < 2; p++) {
      qcu::pack_fermions(qcu::PREC_DOUBLE, s.N, src, qcu::SRC_LEX, p, f.data, nullptr, s.geo, 1, s.stream());
      qcu::unpack_fermions(qcu::PREC_DOUBLE, s.N, dst, qcu::SRC_EO_FULL, p, f.data, nullptr, s.geo, 1, s.stream());
    }
    s.sync();
  });
}

int qcuEoToLex(void* lex_out, const void* eo_in, int ncomp) {
  return guarded([&] {
    Session& s = session();
    QCU_REQUIRE(ncomp == 4 * s.N, QCU_ERR_UNSUPPORTED, "ncomp must be 4*N (a fermion field)");
    qcu::PtrArray src{}, dst{};
    src.p[0] = eo_in;
    dst.p[0] = lex_out;
    qcu::FieldView f = s.alloc_field("lex.tmp", qcu::PREC_DOUBLE, 1);
    for (int p = 0; p < 2; p++) {
      qcu::pack_fermions(qcu::PREC_DOUBLE, s.N, src, qcu::SRC_EO_FULL, p, f.data, nullptr, s.geo, 1, s.stream());
      qcu::unpack_fermions(qcu::PREC_DOUBLE, s.N, dst, qcu::SRC_LEX, p, f.data, nullptr, s.geo, 1, s.stream());
    }
    s.sync();
  });
}

int qcuDslashMRHS(void* out, void* out_norm, const void* in, const void* in_norm, int nrhs, int parity, int dagger,
                  int precision) {
  return qcuDslashXpayMRHS(out, out_norm, in, in_norm, nullptr, nullptr, nrhs, parity, dagger, precision, 1.0, 0.0);
}

int qcuDslashXpayMRHS(void* out, void* out_norm, const void* in, const void* in_norm, const void* x,
                      const void* x_norm, int nrhs, int parity, int dagger, int precision, double a, double b) {
  return guarded([&] {
    Session& s = session();
    QCU_REQUIRE(qcu::prec_valid(precision), QCU_ERR_INVALID_ARGUMENT, "bad precision");
    QCU_REQUIRE(nrhs >= 1, QCU_ERR_INVALID_ARGUMENT, "nrhs must be positive");
    QCU_REQUIRE(out && in, QCU_ERR_INVALID_ARGUMENT, "null field");
    QCU_REQUIRE(out != in, QCU_ERR_INVALID_ARGUMENT, "in-place dslash is not supported");
    QCU_REQUIRE(((uintptr_t)out | (uintptr_t)in | (uintptr_t)x) % 16 == 0, QCU_ERR_INVALID_ARGUMENT,
                "fields must be 16-byte aligned");
    const bool h = qcu::prec_has_norm(precision);
    QCU_REQUIRE(!h || (out_norm && in_norm && (!x || x_norm)), QCU_ERR_INVALID_ARGUMENT,
                "FP16 fields need norm arrays");
    qcu::FieldView fo, fi, fx;
    fo.data = out;
    fo.norm = static_cast<float*>(out_norm);
    fi.data = const_cast<void*>(in);
    fi.norm = static_cast<float*>(const_cast<void*>(in_norm));
    fx.data = const_cast<void*>(x);
    fx.norm = static_cast<float*>(const_cast<void*>(x_norm));
    fo.prec = fi.prec = fx.prec = precision;
    fo.nrhs = fi.nrhs = fx.nrhs = nrhs;
    s.hop(fo, fi, fx, parity, dagger, a, b);
  });
}

int qcuLoadClover(void* clover) {
  return guarded([&] {
    Session& s = session();
    s.load_clover(clover);
    s.sync();
  });
}

int qcuCloverMRHS(void* out, void* out_norm, const void* in, const void* in_norm, int nrhs, int parity, int inverse,
                  int precision) {
  return guarded([&] {
    Session& s = session();
    QCU_REQUIRE(qcu::prec_valid(precision), QCU_ERR_INVALID_ARGUMENT, "bad precision");
    QCU_REQUIRE(nrhs >= 1, QCU_ERR_INVALID_ARGUMENT, "nrhs must be positive");
    QCU_REQUIRE(out && in && out != in, QCU_ERR_INVALID_ARGUMENT, "null or in-place field");
    QCU_REQUIRE(((uintptr_t)out | (uintptr_t)in) % 16 == 0, QCU_ERR_INVALID_ARGUMENT,
                "fields must be 16-byte aligned");
    QCU_REQUIRE(!qcu::prec_has_norm(precision) || (out_norm && in_norm), QCU_ERR_INVALID_ARGUMENT,
                "FP16 fields need norm arrays");
    qcu::FieldView fo, fi;
    fo.data = out;
    fo.norm = static_cast<float*>(out_norm);
    fi.data = const_cast<void*>(in);
    fi.norm = static_cast<float*>(const_cast<void*>(in_norm));
    fo.prec = fi.prec = precision;
    fo.nrhs = fi.nrhs = nrhs;
    s.clover_apply(fo, fi, qcu::FieldView{}, parity, inverse != 0, 1.0, 0.0);
  });
}

int qcuNorm2MRHS(double* out, const void* field, int precision, int nrhs) {
  return guarded([&] {
    Session& s = session();
    QCU_REQUIRE(out && field, QCU_ERR_INVALID_ARGUMENT, "null pointer");
    QCU_REQUIRE(precision == QCU_SINGLE_PRECISION || precision == QCU_DOUBLE_PRECISION, QCU_ERR_UNSUPPORTED,
                "norms are computed for FP32 or FP64 fields");
    QCU_REQUIRE(nrhs >= 1 && nrhs <= qcu::QCU_MAX_RHS, QCU_ERR_INVALID_ARGUMENT, "nrhs must be in 1..256");
    qcu::FieldRef f;
    f.data = const_cast<void*>(field);
    f.prec = precision;
    f.nrhs = nrhs;
    f.n = (int64_t)s.field_elems(nrhs);
    s.blas().norm2(f, out, s.stream());
  });
}

int qcuBlasMRHS(int op, const void* a, const void* b, const void* c, const void* x, int x_precision, void* y,
                int y_precision, void* z, int z_precision, size_t n_elements, int nrhs, void* out) {
  return guarded([&] {
    Session& s = session();
    QCU_REQUIRE(op >= QCU_BLAS_AXPBY && op <= QCU_BLAS_COPY, QCU_ERR_INVALID_ARGUMENT, "qcuBlasMRHS: bad op");
    QCU_REQUIRE(nrhs >= 1 && nrhs <= qcu::QCU_MAX_RHS, QCU_ERR_INVALID_ARGUMENT, "nrhs must be in 1..256");
    QCU_REQUIRE(n_elements > 0 && n_elements % (size_t)nrhs == 0, QCU_ERR_INVALID_ARGUMENT,
                "n_elements must be a positive multiple of nrhs");
    auto field = [&](const void* p, int prec, const char* name) {
      QCU_REQUIRE(p != nullptr, QCU_ERR_INVALID_ARGUMENT, std::string("qcuBlasMRHS: null ") + name);
      QCU_REQUIRE(prec == QCU_SINGLE_PRECISION || prec == QCU_DOUBLE_PRECISION, QCU_ERR_UNSUPPORTED,
                  "BLAS fields are FP32 or FP64");
      qcu::FieldRef f;
      f.data = const_cast<void*>(p);
      f.prec = prec;
      f.n = (int64_t)n_elements;
      f.nrhs = nrhs;
      return f;
    };
    const double2* ca = static_cast<const double2*>(a);
    const double2* cb = static_cast<const double2*>(b);
    const double2* cc = static_cast<const double2*>(c);
    qcu::Blas& blas = s.blas();
    const qcu::FieldRef fx = field(x, x_precision, "x");
    const bool reduces = op == QCU_BLAS_AXPBY_NORM || op == QCU_BLAS_NORM2 || op == QCU_BLAS_NORM2_FP32 ||
                         op == QCU_BLAS_CDOT;
    QCU_REQUIRE(!reduces || out != nullptr, QCU_ERR_INVALID_ARGUMENT, "qcuBlasMRHS: null out");
    switch (op) {
      case QCU_BLAS_NORM2:
      case QCU_BLAS_NORM2_FP32:
        blas.norm2(fx, static_cast<double*>(out), s.stream(), op == QCU_BLAS_NORM2);
        break;
      case QCU_BLAS_AXPBY:
        blas.axpby(ca, fx, cb, field(y, y_precision, "y"), s.stream());
        break;
      case QCU_BLAS_AXPBY_NORM:
        blas.axpby_norm(ca, fx, cb, field(y, y_precision, "y"), static_cast<double*>(out), s.stream());
        break;
      case QCU_BLAS_AXPBYPCZ:
        blas.axpbypcz(ca, fx, cb, field(y, y_precision, "y"), cc, field(z, z_precision, "z"), s.stream());
        break;
      case QCU_BLAS_CDOT:
        blas.cdot(fx, field(y, y_precision, "y"), static_cast<double2*>(out), s.stream());
        break;
      case QCU_BLAS_ADD_TO:
        blas.add_to(fx, field(y, y_precision, "y"), s.stream());
        break;
      default:
        blas.copy(fx, field(y, y_precision, "y"), s.stream());
        break;
    }
  });
}

namespace {
// The fastest work-list shape for these segments: every registered
// work-list form that fits them (nrhs a multiple of R) at block sizes 32, 64,
// 128, timed on the segments themselves (out = a D in + b x does not read
// out, so repeating it is harmless).
qcu::DslashConfig tune_work_list(const std::vector<qcu::DslashArgs>& segs, int prec, int N, cudaStream_t st,
                                 bool* found) {
  int opts[4 * 64];
  const int n = qcu::segments_options(prec, N, opts, 64);
  qcu::DslashConfig best;
  float best_ms = 1e30f;
  *found = false;
  cudaEvent_t e0, e1;
  QCU_CHECK_CUDA(cudaEventCreate(&e0));
  QCU_CHECK_CUDA(cudaEventCreate(&e1));
  for (int i = 0; i < n; i++) {
    bool fits = true;
    for (const qcu::DslashArgs& A : segs) fits &= A.nrhs % opts[4 * i] == 0 && (!opts[4 * i + 3] || A.gauge12);
    if (!fits) continue;
    for (int block : {32, 64, 128}) {
      qcu::DslashConfig c;
      c.R = opts[4 * i];
      c.minb = opts[4 * i + 1];
      c.pk = opts[4 * i + 2];
      c.rc = opts[4 * i + 3];
      c.block = block;
      std::vector<int> misfits;
      qcu::launch_dslash_segments(segs, prec, N, c, st, &misfits);  // warm-up
      QCU_CHECK_CUDA(cudaEventRecord(e0, st));
      for (int k = 0; k < 3; k++) qcu::launch_dslash_segments(segs, prec, N, c, st, &misfits);
      QCU_CHECK_CUDA(cudaEventRecord(e1, st));
      QCU_CHECK_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      QCU_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best_ms) best_ms = ms, best = c, *found = true;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}
}  // namespace

int qcuDslashSegments(const QcuHopSegment* segments, int count, int nColors, int precision, void* stream) {
  return guarded([&] {
    QCU_REQUIRE(count >= 0 && (segments || count == 0), QCU_ERR_INVALID_ARGUMENT, "qcuDslashSegments: bad list");
    QCU_REQUIRE(precision == QCU_SINGLE_PRECISION || precision == QCU_DOUBLE_PRECISION ||
                    precision == QCU_BF16_PRECISION,
                QCU_ERR_UNSUPPORTED, "qcuDslashSegments: FP32, FP64 or BF16 fields");
    QCU_REQUIRE(nColors >= 3 && nColors <= 8, QCU_ERR_UNSUPPORTED, "nColors must be in 3..8");
    if (count == 0) return;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    std::vector<qcu::DslashArgs> segs(count);
    int big = 0;
    int64_t big_units = -1;
    for (int i = 0; i < count; i++) {
      const QcuHopSegment& g = segments[i];
      for (int d = 0; d < 4; d++) QCU_REQUIRE(g.lattice[d] > 0, QCU_ERR_INVALID_ARGUMENT, "lattice sizes must be positive");
      QCU_REQUIRE(g.lattice[0] % 2 == 0, QCU_ERR_INVALID_ARGUMENT, "lattice X extent must be even");
      QCU_REQUIRE(g.gauge && g.in && g.out && g.out != g.in && g.out != g.x, QCU_ERR_INVALID_ARGUMENT,
                  "segment " + std::to_string(i) + ": null field, or out the same memory as in or x");
      QCU_REQUIRE(((uintptr_t)g.in | (uintptr_t)g.out | (uintptr_t)g.x) % 16 == 0, QCU_ERR_INVALID_ARGUMENT,
                  "fields must be 16-byte aligned");
      QCU_REQUIRE(g.nrhs >= 1 && (g.parity == 0 || g.parity == 1) && (g.dagger == 0 || g.dagger == 1),
                  QCU_ERR_INVALID_ARGUMENT, "segment " + std::to_string(i) + ": bad nrhs, parity or dagger");
      QCU_REQUIRE(!g.gauge_two_row || nColors == 3, QCU_ERR_INVALID_ARGUMENT, "two-row links are SU(3) only");
      qcu::DslashArgs& A = segs[i];
      A.gauge = g.gauge;
      A.gauge12 = g.gauge_two_row;
      A.in = g.in;
      A.in_norm = nullptr;
      A.out = g.out;
      A.out_norm = nullptr;
      A.x = g.x;
      A.x_norm = nullptr;
      A.mask = nullptr;
      A.a_rhs_f = nullptr;
      A.a_rhs_d = nullptr;
      A.a = g.a;
      A.b = g.b;
      A.geo = qcu::make_geometry(g.lattice);
      A.nrhs = g.nrhs;
      A.parity = g.parity;
      A.dagger = g.dagger;
      A.antiperiodic_t = g.antiperiodic_t ? 1 : 0;
      const int64_t units = (int64_t)A.geo.vh * A.nrhs;
      if (units > big_units) big_units = units, big = i;
    }
    // The shape: pinned by QCU_DSLASH_CONFIG; else the one tuned for this work
    // list (cached per list); else the largest segment's own shape.
    qcu::Autotuner& tuner = qcu::global_tuner();
    bool found = false;
    const qcu::DslashArgs& B = segs[big];
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    QCU_CHECK_CUDA(cudaStreamIsCapturing(st, &cs));
    const bool may_tune = tuner.enabled() && cs == cudaStreamCaptureStatusNone;
    qcu::DslashConfig c;
    if (getenv("QCU_DSLASH_CONFIG")) c = tuner.lookup(precision, nColors, B.nrhs, B.geo.vh, &found);
    if (!found && count > 1) {  // one segment: the lattice's own tuned shape, as for qcuDslashMRHS
      std::string key = std::to_string(precision) + ":" + std::to_string(nColors);
      for (const qcu::DslashArgs& A : segs)
        key += ":" + std::to_string(A.geo.vh) + "x" + std::to_string(A.nrhs) + (A.gauge12 ? "r" : "f");
      static std::map<std::string, qcu::DslashConfig> tuned_lists;  // under the API lock
      auto it = tuned_lists.find(key);
      if (it != tuned_lists.end()) {
        c = it->second;
        found = true;
      } else if (may_tune) {
        c = tune_work_list(segs, precision, nColors, st, &found);
        if (found) tuned_lists[key] = c;
      }
    }
    if (!found) {
      c = tuner.lookup(precision, nColors, B.nrhs, B.geo.vh, &found);
      if (!found && may_tune) c = tuner.tune(B, precision, nColors, st);
    }
    std::vector<int> misfits;
    qcu::launch_dslash_segments(segs, precision, nColors, c, st, &misfits);
    for (int i : misfits) {  // an RHS count the shared shape cannot take: the segment's own shape
      const qcu::DslashArgs& A = segs[i];
      qcu::DslashConfig own = tuner.lookup(precision, nColors, A.nrhs, A.geo.vh, &found);
      if (!found && may_tune) own = tuner.tune(A, precision, nColors, st);
      qcu::launch_dslash(A, precision, nColors, own, st);
    }
  });
}

int qcuCheckWaitTimeout(double limit_seconds) {
  return guarded([&] {
    QCU_REQUIRE(limit_seconds > 0.0 && limit_seconds <= 1.0, QCU_ERR_INVALID_ARGUMENT,
                "qcuCheckWaitTimeout: limit_seconds must be in (0, 1]");
    const bool timed_out = qcu::wait_timeout_selftest(limit_seconds, 0);
    QCU_REQUIRE(!timed_out, QCU_ERR_DEVICE_TIMEOUT,
                "a device-side wait gave up after its bound (diagnostic kernel; the context stays usable)");
  });
}

int qcuDslashKernels(int precision, int nColors, int* shapes, int max_shapes, int* count) {
  return guarded_unlocked([&] {
    QCU_REQUIRE(qcu::prec_valid(precision), QCU_ERR_INVALID_ARGUMENT, "bad precision");
    QCU_REQUIRE(count != nullptr && (shapes != nullptr || max_shapes == 0) && max_shapes >= 0,
                QCU_ERR_INVALID_ARGUMENT, "qcuDslashKernels: bad output arrays");
    int n = 0;
    auto put = [&](int R, int m, int pk, int st, int rc, int lt) {
      if (n < max_shapes) {
        int* o = shapes + 6 * n;
        o[0] = R, o[1] = m, o[2] = pk, o[3] = st, o[4] = rc, o[5] = lt;
      }
      n++;
    };
    for (int R = 1; R <= 8; R++)
      for (int v = 0; v < 8; v++)  // packed x two-row links x links staged by TMA
        for (int m = 1; m <= 7; m++) {
          const int pk = v & 1, rc = (v >> 1) & 1, lt = v >> 2;
          if (qcu::find_dslash(precision, nColors, R, m, pk, rc, lt)) put(R, m, pk, 0, rc, lt);
        }
    int tr[32], ts[32];
    const int nt = qcu::tma_options(precision, nColors, tr, ts, 32);
    for (int i = 0; i < nt; i++) put(tr[i], 0, 0, ts[i], 0, 0);
    for (int v = 1; v <= qcu::kTcVariants; v++)
      if (qcu::find_tc(precision, nColors, v)) put(1, 0, 0, -v, 0, 0);
    *count = n;
  });
}

int qcuLastDslashShape(int* shape) {
  return guarded_unlocked([&] {
    QCU_REQUIRE(shape != nullptr, QCU_ERR_INVALID_ARGUMENT, "qcuLastDslashShape: null output");
    const qcu::DslashConfig c = qcu::last_launched_dslash();
    shape[0] = c.R, shape[1] = c.minb, shape[2] = c.pk, shape[3] = c.tc ? -c.tc : c.tma, shape[4] = c.rc,
    shape[5] = c.lt;
  });
}

int qcuTuneDslash(int nrhs, int precision, int* rhs_per_thread, int* block, int* min_blocks, int* packed,
                  int* stages, int* recon, int* linktma) {
  return guarded([&] {
    Session& s = session();
    QCU_REQUIRE(qcu::prec_valid(precision), QCU_ERR_INVALID_ARGUMENT, "bad precision");
    qcu::FieldView fi = s.alloc_field("tune.in", precision, nrhs);
    qcu::FieldView fo = s.alloc_field("tune.out", precision, nrhs);
    QCU_CHECK_CUDA(cudaMemsetAsync(fi.data, 0, s.field_bytes(precision, nrhs), s.stream()));
    if (fi.norm) QCU_CHECK_CUDA(cudaMemsetAsync(fi.norm, 0, s.norm_bytes(precision, nrhs), s.stream()));
    qcu::DslashArgs A;
    A.gauge = s.gauge(precision);
    A.gauge12 = s.gauge12(precision);
    if (qcu::prec_bf16(precision) && nrhs % 4 == 0) A.gauge_tc = s.gauge_tc();
    A.in = fi.data;
    A.in_norm = fi.norm;
    A.out = fo.data;
    A.out_norm = fo.norm;
    A.x = nullptr;
    A.x_norm = nullptr;
    A.mask = nullptr;
    A.a_rhs_f = nullptr;
    A.a_rhs_d = nullptr;
    A.a = 1.0;
    A.b = 0.0;
    A.geo = s.geo;
    A.nrhs = nrhs;
    A.parity = 0;
    A.dagger = 0;
    A.antiperiodic_t = 0;
    // the shape the dslash uses: the pinned or cached choice, else tuned now
    bool found = false;
    qcu::DslashConfig c = s.tuner.lookup(precision, s.N, nrhs, s.geo.vh, &found);
    if (!found) c = s.tuner.tune(A, precision, s.N, s.stream());
    if (rhs_per_thread) *rhs_per_thread = c.R;
    if (block) *block = c.block;
    if (min_blocks) *min_blocks = c.minb;
    if (packed) *packed = c.pk;
    if (stages) *stages = c.tc ? -c.tc : c.tma;
    if (recon) *recon = c.rc;
    if (linktma) *linktma = c.lt;
  });
}

// ---- solve server ---------------------------------------------------------
int qcuServerCreate(void** server, size_t hbm_budget_bytes, int max_slots_per_gauge, int inner_precision,
                    int solver) {
  return guarded_unlocked([&] {
    QCU_REQUIRE(server != nullptr, QCU_ERR_INVALID_ARGUMENT, "null server handle");
    QCU_REQUIRE(solver == QCU_SOLVER_CG || solver == QCU_SOLVER_BICGSTAB, QCU_ERR_INVALID_ARGUMENT, "bad solver");
    *server = new qcu::Server(hbm_budget_bytes, max_slots_per_gauge, inner_precision, solver);
  });
}

int qcuServerAddGauge(void* server, int gauge_id, const int lattice[4], int nColors, const void* gauge,
                      int antiperiodic_t) {
  return guarded_unlocked([&] {
    QCU_REQUIRE(server && lattice && gauge, QCU_ERR_INVALID_ARGUMENT, "null argument");
    QcuParam p;
    for (int i = 0; i < 4; i++) p.lattice_size[i] = lattice[i];
    check_lattice(&p);
    QCU_REQUIRE(nColors >= 3 && nColors <= 8, QCU_ERR_UNSUPPORTED, "nColors must be in 3..8");
    static_cast<qcu::Server*>(server)->add_gauge(gauge_id, lattice, nColors, gauge, antiperiodic_t);
  });
}

int qcuServerSubmit(void* server, int gauge_id, double kappa, double tol, int nrhs, void* const* x,
                    void* const* b, long long* request_id) {
  return guarded_unlocked([&] {
    QCU_REQUIRE(server && request_id, QCU_ERR_INVALID_ARGUMENT, "null argument");
    *request_id = static_cast<qcu::Server*>(server)->submit(gauge_id, kappa, tol, nrhs, x, b);
  });
}

int qcuServerWait(void* server, long long request_id, double timeout_s, QcuRequestInfo* info) {
  return guarded_unlocked([&] {
    QCU_REQUIRE(server != nullptr, QCU_ERR_INVALID_ARGUMENT, "null server");
    qcu::RequestInfo ri;
    static_cast<qcu::Server*>(server)->wait(request_id, timeout_s, &ri);
    if (info) {
      info->done = ri.done;
      info->status = ri.status;
      info->nrhs = ri.nrhs;
      info->iterations = ri.iterations;
      info->latency_s = ri.latency_s;
      info->queue_s = ri.queue_s;
      info->max_true_residual = ri.max_true_residual;
      info->all_converged = ri.all_converged;
    }
  });
}

int qcuServerStats(void* server, QcuServerStats* stats) {
  return guarded_unlocked([&] {
    QCU_REQUIRE(server && stats, QCU_ERR_INVALID_ARGUMENT, "null argument");
    qcu::ServerStats s = static_cast<qcu::Server*>(server)->stats();
    stats->submitted = s.submitted;
    stats->completed = s.completed;
    stats->p50_s = s.p50_s;
    stats->p99_s = s.p99_s;
    stats->mean_s = s.mean_s;
    stats->solves_per_s = s.solves_per_s;
    stats->rhs_per_s = s.rhs_per_s;
    stats->hbm_used = s.hbm_used;
  });
}

int qcuServerDestroy(void* server) {
  return guarded_unlocked([&] { delete static_cast<qcu::Server*>(server); });
}

void qcuSolverParamDefaults(QcuSolverParam* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->solver = QCU_SOLVER_CG;
  p->inner_precision = QCU_SINGLE_PRECISION;
  p->kappa = 0.125;
  p->tol = 1e-10;
  p->max_iter = 10000;
  p->delta = 0.1;
  p->use_graph = 1;
  p->src_mode = QCU_SRC_EO_FULL;
}

int qcuInvert(void* const* x, void* const* b, int nrhs, QcuSolverParam* p) {
  return guarded([&] {
    Session& s = session();
    QCU_REQUIRE(p != nullptr, QCU_ERR_INVALID_ARGUMENT, "null solver parameters");
    QCU_REQUIRE(x && b, QCU_ERR_INVALID_ARGUMENT, "null field arrays");
    qcu::SolveRequest q;
    q.solver = p->solver;
    q.inner_prec = p->inner_precision;
    q.kappa = p->kappa;
    q.tol = p->tol;
    q.max_iter = p->max_iter;
    q.delta = p->delta > 0 ? p->delta : 0.1;
    q.use_graph = p->use_graph != 0;
    q.src_mode = p->src_mode;
    q.clover = p->use_clover != 0;
    qcu::SolveResult r = qcu::solve(s, x, b, nrhs, q);
    p->iterations = r.iterations;
    p->reliable_updates = r.reliable_updates;
    p->seconds = r.seconds;
    bool all = true;
    std::string bad;
    for (int i = 0; i < nrhs && i < 256; i++) {
      p->true_residual[i] = r.true_residual[i];
      p->converged[i] = r.converged[i];
      all &= r.converged[i] != 0;
      if (r.bad_source[i]) bad += (bad.empty() ? "" : ", ") + std::to_string(i);
    }
    QCU_REQUIRE(bad.empty(), QCU_ERR_INVALID_ARGUMENT,
                "qcuInvert: source(s) " + bad + " hold NaN or Inf; they were not solved (the others were)");
    QCU_REQUIRE(all, QCU_ERR_NOT_CONVERGED, "qcuInvert: not every RHS converged");
  });
}

}  // extern "C"
