// The reference's C++ operator interface, with its signatures and mangled
// names: qcu::instantiateDslash (include/qcd/qcu_dslash.h:62-64 and
// src/qcd/qcu_wilson.cu:159-173 of the reference), qcu::DiracWilson::Dslash
// (include/qcu_dirac.h:40-50, src/qcu_dirac.cu:7-14) and the WilsonDslash
// class template (include/qcd/qcu_dslash.h:52-60), on this library's MRHS
// kernels.
//
// The caller's RHS arrive as separate coalesced arrays ([4N][Vh] complex per
// RHS, the reference's internal layout), so each call gathers them into one
// RHS-innermost MRHS field, applies the autotuned MRHS dslash on the
// caller's coalesced gauge (which is already this library's gauge layout)
// and scatters the results back.  The two MRHS work fields are kept between
// calls (one allocation per device and size, not per call).  Errors print
// the reference's messages and are recorded for qcuGetLastError().
#pragma GCC visibility push(default)
#include "../../include/qcu_dirac.h"
#pragma GCC visibility pop

#include <algorithm>
#include <mutex>
#include <new>

#include "layout.h"
#include "session.h"

extern "C" void qcu_record_error(int code, const char* msg);

namespace qcu {
namespace {

struct MrhsScratch {
  std::mutex m;
  DeviceBuffer in, out;
  int device = -1;
};

MrhsScratch& scratch() {
  static MrhsScratch s;
  return s;
}

void run_hop(const QcuLattDesc<Nd>& latt, const QcuProcDesc<Nd>& proc, int parity, int dagger, void* in_ptrs,
             void* out_ptrs, void* gauge, QCU_PRECISION precision, int N, int nrhs, cudaStream_t st) {
  QCU_REQUIRE(precision == QCU_SINGLE_PRECISION || precision == QCU_DOUBLE_PRECISION, QCU_ERR_UNSUPPORTED,
              "Now we only support single and double precision.\n");
  QCU_REQUIRE(N >= 3 && N <= 8, QCU_ERR_UNSUPPORTED, "Now we only support 3-8 colors.\n");
  QCU_REQUIRE(nrhs >= 1, QCU_ERR_INVALID_ARGUMENT, "nInputs must be positive");
  QCU_REQUIRE(parity == 0 || parity == 1, QCU_ERR_INVALID_ARGUMENT, "parity must be 0 or 1");
  QCU_REQUIRE(dagger == 0 || dagger == 1, QCU_ERR_INVALID_ARGUMENT, "daggerFlag must be 0 or 1");
  QCU_REQUIRE(in_ptrs && out_ptrs && gauge, QCU_ERR_INVALID_ARGUMENT, "null fermion or gauge argument");
  for (int i = 0; i < 4; i++) {
    QCU_REQUIRE(proc.dim[i] == 1, QCU_ERR_UNSUPPORTED,
                "multi-process grids are not supported (one GPU per process): QcuProcDesc must be 1x1x1x1");
    QCU_REQUIRE(latt.dim[i] > 0, QCU_ERR_INVALID_ARGUMENT, "lattice sizes must be positive");
  }
  QCU_REQUIRE(latt.dim[0] % 2 == 0, QCU_ERR_INVALID_ARGUMENT, "lattice X extent must be even");
  const int L[4] = {latt.dim[0], latt.dim[1], latt.dim[2], latt.dim[3]};
  const Geometry geo = make_geometry(L);
  const int prec = precision == QCU_SINGLE_PRECISION ? PREC_SINGLE : PREC_DOUBLE;
  void* const* ins = static_cast<void* const*>(in_ptrs);
  void* const* outs = static_cast<void* const*>(out_ptrs);

  MrhsScratch& sc = scratch();
  std::lock_guard<std::mutex> lk(sc.m);
  int dev = 0;
  QCU_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev != sc.device) {  // buffers of another device: drop them
    sc.in.release();
    sc.out.release();
    sc.device = dev;
  }
  Autotuner& tuner = global_tuner();
  for (int base = 0; base < nrhs; base += QCU_MAX_RHS) {
    const int m = std::min(QCU_MAX_RHS, nrhs - base);
    PtrArray pin{}, pout{};
    for (int r = 0; r < m; r++) {
      QCU_REQUIRE(ins[base + r] && outs[base + r], QCU_ERR_INVALID_ARGUMENT, "null RHS pointer");
      pin.p[r] = ins[base + r];
      pout.p[r] = outs[base + r];
    }
    const size_t bytes = (size_t)geo.vh * 4 * N * m * prec_complex_bytes(prec);
    void* fin = sc.in.ensure(bytes);
    void* fout = sc.out.ensure(bytes);
    gather_rhs_arrays(prec, pin, fin, geo.vh, 4 * N, m, st);
    DslashArgs A;
    A.gauge = gauge;
    A.in = fin;
    A.in_norm = nullptr;
    A.out = fout;
    A.out_norm = nullptr;
    A.x = nullptr;
    A.x_norm = nullptr;
    A.mask = nullptr;
    A.a_rhs_f = nullptr;
    A.a_rhs_d = nullptr;
    A.a = 1.0;
    A.b = 0.0;
    A.geo = geo;
    A.nrhs = m;
    A.parity = parity;
    A.dagger = dagger;
    A.antiperiodic_t = 0;  // the reference's kernel is periodic in every direction
    bool found = false;
    DslashConfig c = tuner.lookup(prec, N, m, geo.vh, &found);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    QCU_CHECK_CUDA(cudaStreamIsCapturing(st, &cs));
    if (!found && tuner.enabled() && cs == cudaStreamCaptureStatusNone) c = tuner.tune(A, prec, N, st);
    launch_dslash(A, prec, N, c, st);
    scatter_rhs_arrays(prec, pout, fout, geo.vh, 4 * N, m, st);
  }
  QCU_CHECK_CUDA(cudaStreamSynchronize(st));
}

}  // namespace

#pragma GCC visibility push(default)

void instantiateDslash(const QcuLattDesc<Nd>& lattDesc, const QcuProcDesc<Nd>& procDesc, int parity, int daggerFlag,
                       double kappa, void* mrhsFermionIn, void* mrhsFermionOut, void* gauge, DSLASH_TYPE dtype,
                       QCU_PRECISION floatPrecision, int nColors, int nInputs, ExecutionStreams& streams) {
  (void)kappa;  // the hop term has no mass term; the reference passes kappa along unused
  try {
    QCU_REQUIRE(dtype == DSLASH_WILSON, QCU_ERR_UNSUPPORTED, "Now we only support Wilson dslash.\n");
    run_hop(lattDesc, procDesc, parity, daggerFlag, mrhsFermionIn, mrhsFermionOut, gauge, floatPrecision, nColors,
            nInputs, streams.stream);
  } catch (const Error& e) {
    qcu_record_error(e.code, e.what());
  } catch (const std::bad_alloc&) {
    qcu_record_error(QCU_ERR_OUT_OF_MEMORY, "host allocation failed");
  } catch (const std::exception& e) {
    qcu_record_error(QCU_ERR_CUDA, e.what());
  }
}

void DiracWilson::Dslash(void* outputMRHS, void* inputMRHS, int parity, int daggerFlag, int nInputs) {
  instantiateDslash(lattDesc_, procDesc_, parity, daggerFlag, kappa_, inputMRHS, outputMRHS, gauge_, DSLASH_WILSON,
                    floatPrecision_, nColors_, nInputs, streams_);
}

template <typename _Float, int _nColor, int _nInput>
void WilsonDslash<_Float, _nColor, _nInput>::apply() {
  const DslashParam& p = this->dslashParam_;
  instantiateDslash(p.lattDesc, p.procDesc, p.parity, p.daggerFlag, p.kappa, p.fermionIn_MRHS, p.fermionOut_MRHS,
                    p.gauge, DSLASH_WILSON, sizeof(_Float) == 4 ? QCU_SINGLE_PRECISION : QCU_DOUBLE_PRECISION,
                    _nColor, _nInput, p.streams);
}

template <typename _Float, int _nColor, int _nInput>
void WilsonDslash<_Float, _nColor, _nInput>::preApply() {}

template <typename _Float, int _nColor, int _nInput>
void WilsonDslash<_Float, _nColor, _nInput>::postApply() {}

// the instances the reference builds (src/qcd/qcu_wilson.cu:61-155)
#define QCU_WILSON_DSLASH_INSTANCES(F, N) \
  template class WilsonDslash<F, N, 1>;   \
  template class WilsonDslash<F, N, 2>;   \
  template class WilsonDslash<F, N, 3>;   \
  template class WilsonDslash<F, N, 4>;   \
  template class WilsonDslash<F, N, 5>;
QCU_WILSON_DSLASH_INSTANCES(float, 3)
QCU_WILSON_DSLASH_INSTANCES(float, 4)
QCU_WILSON_DSLASH_INSTANCES(float, 5)
QCU_WILSON_DSLASH_INSTANCES(double, 3)
QCU_WILSON_DSLASH_INSTANCES(double, 4)
QCU_WILSON_DSLASH_INSTANCES(double, 5)
#undef QCU_WILSON_DSLASH_INSTANCES

#pragma GCC visibility pop

}  // namespace qcu
