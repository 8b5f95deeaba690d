/*
 * qcuDesc/mrhs_desc.h -- the multi-RHS argument of the reference's C++
 * interface (include/qcuDesc/mrhs_desc.h:5-10 of the reference): _Nvec
 * device pointers, one per right-hand side, held in host memory and passed
 * to instantiateDslash / Dirac::Dslash as a void pointer.
 */
#pragma once

#include <cstddef>

#ifdef __CUDACC__
#define QCU_HOST_DEVICE __host__ __device__
#else
#define QCU_HOST_DEVICE
#endif

namespace qcu {

template <size_t _Nvec>
struct MrhsInput {
  void *fermion[_Nvec];
  void *data() { return fermion; }
  QCU_HOST_DEVICE void *operator[](size_t i) { return fermion[i]; }
};

}  // namespace qcu
