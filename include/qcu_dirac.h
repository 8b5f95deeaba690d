/*
 * qcu_dirac.h -- the Dirac-operator classes of the reference's C++
 * interface (include/qcu_dirac.h:7-50 and src/qcu_dirac.cu:7-14 of the
 * reference).  Same members in the same order, same virtual functions in
 * the same order, so objects and calls pass between code built against
 * either header and libqcu.so.
 *
 * DiracWilson::Dslash(out, in, parity, daggerFlag, nInputs) is
 * instantiateDslash (qcd/qcu_dslash.h) on the operator's gauge, precision,
 * colours, descriptors and streams; kappa = 1 / (2 (4 + mass)).
 * DslashXpay() is the reference's empty stub; the library's xpay operation
 * is qcuDslashXpayMRHS (qcu_gb300.h).
 */
#pragma once

#include "qcd/qcu_dslash.h"
#include "qcuDesc/qcu_desc.h"
#include "qcu_kernel_param.cuh"

namespace qcu {

class Dirac {
 protected:
  void *gauge_;
  double kappa_;
  double mass_;
  int nColors_;
  QCU_PRECISION floatPrecision_;
  const QcuLattDesc<Nd> &lattDesc_;
  const QcuProcDesc<Nd> &procDesc_;
  DSLASH_TYPE dslashType_;
  ExecutionStreams &streams_;

 public:
  Dirac(void *gauge, double mass, int nColors, QCU_PRECISION floatPrecision, const QcuLattDesc<Nd> &lattDesc,
        const QcuProcDesc<Nd> &procDesc, DSLASH_TYPE dslashType, ExecutionStreams &streams)
      : gauge_(gauge),
        kappa_(1.0 / (2.0 * (4.0 + mass))),
        mass_(mass),
        nColors_(nColors),
        floatPrecision_(floatPrecision),
        lattDesc_(lattDesc),
        procDesc_(procDesc),
        dslashType_(dslashType),
        streams_(streams) {}

  virtual ~Dirac() {}
  virtual void Dslash(void *outputMRHS, void *inputMRHS, int parity, int daggerFlag, int nInputs) = 0;
  virtual void DslashXpay() = 0;
};

class DiracWilson : public Dirac {
 public:
  DiracWilson(void *gauge, double mass, int nColors, QCU_PRECISION floatPrecision, const QcuLattDesc<Nd> &lattDesc,
              const QcuProcDesc<Nd> &procDesc, DSLASH_TYPE dslashType, ExecutionStreams &streams)
      : Dirac(gauge, mass, nColors, floatPrecision, lattDesc, procDesc, dslashType, streams) {}
  ~DiracWilson() {}
  virtual void Dslash(void *outputMRHS, void *inputMRHS, int parity, int daggerFlag, int nInputs);
  virtual void DslashXpay() {}
};

}  // namespace qcu
