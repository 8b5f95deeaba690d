/*
 * qcd/qcu_dslash.h -- the dslash entry point of the reference's C++
 * interface (include/qcd/qcu_dslash.h:9-64 of the reference), same
 * declarations, implemented by libqcu.so on its MRHS kernels.
 *
 * instantiateDslash applies the even-odd Wilson hopping term
 *   out_r = sum_mu [ (1 - f g_mu) U_mu(x) in_r(x+mu) + (1 + f g_mu) U_mu(x-mu)^dag in_r(x-mu) ]
 * (f = +1, or -1 when daggerFlag = 1; periodic boundaries) for output
 * parity `parity` to nInputs right-hand sides:
 *   mrhsFermionIn / mrhsFermionOut: host pointers to MrhsInput<nInputs>,
 *       i.e. nInputs device pointers, each one parity of one RHS in the
 *       coalesced layout [4 * nColors][Vh] complex (float2 / double2)
 *   gauge: device pointer, coalesced [4][2][nColors * nColors][Vh] complex
 *   floatPrecision: QCU_SINGLE_PRECISION or QCU_DOUBLE_PRECISION (the
 *       arithmetic and storage type of every operand)
 *   nColors: 3..8 (every N has its own kernels; the reference computes
 *       6..8 as 5); nInputs: any positive count (the reference takes 1..5)
 *   kappa: accepted and unused, as in the reference (the hop term has no mass)
 *   procDesc: 1 x 1 x 1 x 1 (grids are rejected, where the reference drops
 *       the boundary hops)
 *   streams.stream: the work runs there; the call returns when it is done.
 * Errors print the reference's message and are recorded for
 * qcuGetLastError() (qcu_gb300.h) instead of terminating the process.
 */
#pragma once

#include "../qcu.h"
#include "../qcuDesc/mrhs_desc.h"
#include "../qcuDesc/qcu_desc.h"
#include "../qcu_enum.h"
#include "../qcu_kernel_param.cuh"

namespace qcu {

static constexpr int Ndim = 4;

struct DslashParam {
  const QcuProcDesc<Ndim> &procDesc;
  const QcuLattDesc<Ndim> &lattDesc;
  int parity;
  int daggerFlag;
  double kappa;
  void *fermionIn_MRHS;
  void *fermionOut_MRHS;
  void *gauge;
  ExecutionStreams &streams;
  DslashParam(const QcuLattDesc<Ndim> &pLattDesc, const QcuProcDesc<Ndim> &pProcDesc, int pParity, int pDaggerFlag,
              double pKappa, void *pFermionIn, void *pFermionOut, void *pGauge, ExecutionStreams &pStreams)
      : procDesc(pProcDesc),
        lattDesc(pLattDesc),
        parity(pParity),
        daggerFlag(pDaggerFlag),
        kappa(pKappa),
        fermionIn_MRHS(pFermionIn),
        fermionOut_MRHS(pFermionOut),
        gauge(pGauge),
        streams(pStreams) {}
};

template <typename _Float, int _nColor, int _nInput>
class Dslash {
 protected:
  const DslashParam &dslashParam_;

 public:
  Dslash(const DslashParam &dslashParam) : dslashParam_(dslashParam) {}
  virtual ~Dslash() {}
  virtual void apply() = 0;
  virtual void preApply() = 0;
  virtual void postApply() = 0;
};

/* apply() is instantiateDslash with the template's precision, colours and
 * RHS count; libqcu.so carries the instances the reference builds (float and
 * double, 3..5 colours, 1..5 RHS). */
template <typename _Float, int _nColor, int _nInput>
class WilsonDslash : public Dslash<_Float, _nColor, _nInput> {
 public:
  WilsonDslash(const DslashParam &dslashParam) : Dslash<_Float, _nColor, _nInput>(dslashParam) {}
  virtual ~WilsonDslash() {}
  virtual void apply();
  virtual void preApply();
  virtual void postApply();
};

void instantiateDslash(const QcuLattDesc<Nd> &lattDesc, const QcuProcDesc<Nd> &procDesc, int parity, int daggerFlag,
                       double kappa, void *mrhsFermionIn, void *mrhsFermionOut, void *gauge, DSLASH_TYPE dtype,
                       QCU_PRECISION floatPrecision, int nColors, int nInputs, ExecutionStreams &streams);

}  // namespace qcu
