// Session, operator and resource management behind the C ABI.
//
// Mirrors the reference's host layer: qcu::Qcu (src/qcu.cu:17-123 of the
// reference) -> Session; qcu::Dirac / DiracWilson (include/qcu_dirac.h:7-50,
// src/qcu_dirac.cu:7-14) -> HopOperator / WilsonHopOperator on resident
// fields; QcuLattDesc / QcuProcDesc (include/qcuDesc/qcu_desc.h:9-97) ->
// LattDesc / ProcDesc; ExecutionStreams (include/qcu_kernel_param.cuh:9-38)
// -> one library stream created on first use (the reference creates nine
// streams during static initialisation).  The reference's own C++ classes,
// with their signatures, are exported from dirac_api.cu.
//
// Resources are cached: the gauge is converted once per precision, and MRHS
// work buffers are allocated once and reused (the reference allocates and
// frees two buffers per RHS per call, src/qcu.cu:93-94,70-77).
#pragma once

#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "blas.h"
#include "dslash.h"
#include "layout.h"

namespace qcu {

struct LattDesc {
  int dim[4];
};
struct ProcDesc {
  int dim[4];
};

class DeviceBuffer {
 public:
  DeviceBuffer() = default;
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  ~DeviceBuffer() { release(); }
  void* ensure(size_t bytes);
  void release();
  void* get() const { return p_; }
  size_t bytes() const { return bytes_; }

 private:
  void* p_ = nullptr;
  size_t bytes_ = 0;
};

// named, growable device buffers reused across calls
class Workspace {
 public:
  void* get(const std::string& name, size_t bytes) { return bufs_[name].ensure(bytes); }
  void clear() { bufs_.clear(); }
  size_t total_bytes() const;

 private:
  std::map<std::string, DeviceBuffer> bufs_;
};

// dslash kernel-shape cache, keyed by (precision, N, nrhs, volume)
class Autotuner {
 public:
  DslashConfig lookup(int prec, int N, int nrhs, int vh, bool* found);
  void store(int prec, int N, int nrhs, int vh, const DslashConfig& c);
  static DslashConfig heuristic(int prec, int N, int nrhs);
  // time every compiled (R, block) candidate on the given arguments; the
  // output buffers of A are overwritten
  DslashConfig tune(const DslashArgs& A, int prec, int N, cudaStream_t st);
  bool enabled() const;
  // the BF16 field layout chosen for (N, nrhs, vh): *known = false if none yet
  bool layout_site_major(int N, int nrhs, int vh, bool* known);
  void store_layout(int N, int nrhs, int vh, bool site_major);

 private:
  std::mutex m_;
  std::map<std::string, DslashConfig> cache_;
  std::map<std::string, bool> layout_;
  std::string key(int prec, int N, int nrhs, int vh) const;
  void load_file();
  void save_file();
  bool file_loaded_ = false;
};

class Session;

// one MRHS field of one parity in some precision (views into buffers)
struct FieldView {
  void* data = nullptr;
  float* norm = nullptr;
  int prec = PREC_DOUBLE;
  int nrhs = 0;
};

// The operator getDslash selects (the reference's Dirac / DiracWilson of
// include/qcu_dirac.h:7-50, which the public C++ interface of libqcu.so
// mirrors in include/qcu_dirac.h); internally it works on resident MRHS
// fields of a session.
class HopOperator {
 public:
  HopOperator(Session& s, double mass, int nColors, int prec, int type)
      : s_(s), mass_(mass), kappa_(1.0 / (2.0 * (4.0 + mass))), nColors_(nColors), prec_(prec), type_(type) {}
  virtual ~HopOperator() = default;
  // out = D_parity^f in for nInputs RHS of the internal MRHS fields
  virtual void Dslash(FieldView out, FieldView in, int parity, int dagger, int nInputs) = 0;
  // out = a * D in + b * x
  virtual void DslashXpay(FieldView out, FieldView in, FieldView x, int parity, int dagger, int nInputs, double a,
                          double b) = 0;
  double kappa() const { return kappa_; }
  double mass() const { return mass_; }
  int precision() const { return prec_; }
  int type() const { return type_; }

 protected:
  Session& s_;
  double mass_, kappa_;
  int nColors_, prec_, type_;
};

class WilsonHopOperator : public HopOperator {
 public:
  using HopOperator::HopOperator;
  void Dslash(FieldView out, FieldView in, int parity, int dagger, int nInputs) override;
  void DslashXpay(FieldView out, FieldView in, FieldView x, int parity, int dagger, int nInputs, double a,
                  double b) override;
};

class Session {
 public:
  Session(const int L[4], const int grid[4], int nColors);
  ~Session();

  // ---- state -------------------------------------------------------------
  LattDesc latt;
  ProcDesc proc;
  Geometry geo;
  int N;
  bool antiperiodic_t = false;
  std::unique_ptr<HopOperator> dirac;
  std::vector<std::pair<void*, void*>> queue;  // (out, in) caller pointers
  Workspace ws;
  Autotuner& tuner;

  // The library's own stream is a blocking stream (ordered after work on the
  // legacy default stream, as a caller of the drop-in ABI expects) unless
  // nonblocking_stream is set before its first use: the solve server's lanes
  // capture CUDA graphs on worker threads, and a capture on a blocking stream
  // makes every legacy-stream call of other threads fail meanwhile.
  bool nonblocking_stream = false;
  cudaStream_t stream();
  void set_user_stream(cudaStream_t s) { user_stream_ = s; }
  void sync();

  // ---- gauge -------------------------------------------------------------
  void load_gauge(const void* caller_gauge, int lex);
  bool gauge_loaded() const { return gauge_loaded_; }
  const void* gauge(int prec);  // internal gauge in `prec`, converted once
  // SU(3) only: the gauge as the first two rows of every link ([8][6][Vh] in
  // `prec`), or nullptr when the loaded field is not SU(3) to that precision's
  // rounding (then the third rows are not reconstructible)
  const void* gauge12(int prec);
  // the links in BF16 as per-site records split into rows (layout.h
  // gauge_tc_records_bf16), for the spinor-operand tensor-core dslash; built
  // on first use
  const void* gauge_tc();

  // ---- clover term (clover.h) ---------------------------------------------
  // caller field [2][Vh][2][2N][2N] complex double, Hermitian blocks; packed
  // to an FP64 master and inverted per site once
  void load_clover(const void* caller_clover);
  bool has_clover() const { return clover_loaded_; }
  const void* clover(int prec, bool inverse);  // resident [2][2][(2N)^2][Vh] in `prec`
  // out = a * C in + b * x, C = A_parity or A_parity^-1, on the library stream
  void clover_apply(FieldView out, FieldView in, FieldView x, int parity, bool inverse, double a, double b,
                    const int* mask = nullptr, const float* a_rhs_f = nullptr, const double* a_rhs_d = nullptr);

  // ---- fields ------------------------------------------------------------
  size_t field_elems(int nrhs) const { return (size_t)geo.vh * 4 * N * nrhs; }
  size_t field_bytes(int prec, int nrhs) const { return field_elems(nrhs) * prec_complex_bytes(prec); }
  size_t norm_bytes(int prec, int nrhs) const { return prec_has_norm(prec) ? (size_t)geo.vh * nrhs * 4 : 0; }
  FieldView alloc_field(const std::string& name, int prec, int nrhs);

  // out = a * D in + b * x  (x.data may be null), on the library stream.
  // mask: per-RHS activity (masked RHS are left untouched); a_rhs_f / a_rhs_d:
  // per-RHS a (device arrays) for FP32 / FP64 arithmetic, replacing a.
  // Whether BF16 operator fields of a.nrhs RHS are faster in the site-major
  // layout (the tensor-core dslash on contiguous site blocks) than in the
  // component-major one: timed once per (N, nrhs, volume) on a and b (two
  // BF16 fields of this session, overwritten), then cached.  False where the
  // site-major kernel cannot run, and during stream capture.
  bool prefer_site_major(FieldView a, FieldView b);
  void hop(FieldView out, FieldView in, FieldView x, int parity, int dagger, double a, double b,
           const int* mask = nullptr, const float* a_rhs_f = nullptr, const double* a_rhs_d = nullptr);

  Blas& blas();
  double* scalars(size_t count);  // device scratch for per-RHS scalars

 private:
  cudaStream_t own_stream_ = nullptr;
  cudaStream_t user_stream_ = nullptr;
  bool gauge_loaded_ = false;
  DeviceBuffer gauge_[5];
  bool gauge_valid_[5] = {false, false, false, false, false};
  DeviceBuffer gauge12_[5];
  bool gauge12_valid_[5] = {false, false, false, false, false};
  DeviceBuffer gauge_tc_;
  bool gauge_tc_valid_ = false;
  double su3_dev_ = -1.0;  // max |row 2 - conj(row 0 x row 1)|, < 0: not measured
  DeviceBuffer su3_scratch_;
  bool clover_loaded_ = false;
  DeviceBuffer clover_[5], cloverinv_[5], clover_flag_;
  bool clover_valid_[5] = {false, false, false, false, false};
  bool cloverinv_valid_[5] = {false, false, false, false, false};
  std::unique_ptr<Blas> blas_;
  DeviceBuffer partials_;
  DeviceBuffer scalars_;
};

Autotuner& global_tuner();

// solver entry (solver.cu)
struct SolveRequest {
  int solver = 0;
  int inner_prec = PREC_SINGLE;
  double kappa = 0.125;
  double tol = 1e-10;
  int max_iter = 10000;
  double delta = 0.1;
  bool use_graph = true;
  int src_mode = SRC_EO_FULL;
  bool clover = false;  // M = A - kappa D with the session's clover field A
};
struct SolveResult {
  int iterations = 0;
  int reliable_updates = 0;
  double seconds = 0.0;
  std::vector<double> true_residual;
  std::vector<int> converged;
  std::vector<int> bad_source;  // 1: the source held NaN or Inf (not solved)
};
SolveResult solve(Session& s, void* const* x, void* const* b, int nrhs, const SolveRequest& req);

}  // namespace qcu
