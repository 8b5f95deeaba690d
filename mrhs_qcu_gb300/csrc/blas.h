// BLAS-1 over MRHS fields (no counterpart in the reference, which has no
// linear algebra; cg_inverter is an empty stub at src/qcu.cu:173 of the
// reference).
//
// A field is `n` complex elements in RHS-innermost order, so element e
// belongs to RHS e % nrhs.  Coefficients are per-RHS device arrays of
// double2 (complex).  FP32 fields are updated in FP32 arithmetic and FP64
// fields in FP64.  Reductions accumulate in FP64 and return per-RHS results
// into device arrays, in a fixed order (deterministic).
#pragma once

#include "qcu_common.cuh"

namespace qcu {

struct FieldRef {
  void* data = nullptr;
  int prec = PREC_DOUBLE;  // PREC_DOUBLE or PREC_SINGLE for BLAS operands
  int64_t n = 0;           // complex elements = vh * ncomp * nrhs
  int nrhs = 1;
};

class Blas {
 public:
  // scratch for the two-stage reductions is owned by the caller (Workspace)
  Blas(double* partials, int max_blocks) : partials_(partials), max_blocks_(max_blocks) {}

  // y = a_r x + b_r y
  void axpby(const double2* a, const FieldRef& x, const double2* b, const FieldRef& y, cudaStream_t st);
  // z = a_r x + b_r y + c_r z
  void axpbypcz(const double2* a, const FieldRef& x, const double2* b, const FieldRef& y, const double2* c,
                const FieldRef& z, cudaStream_t st);
  // y = a_r x + b_r y, then out[r] = |y_r|^2 (double)
  void axpby_norm(const double2* a, const FieldRef& x, const double2* b, const FieldRef& y, double* out,
                  cudaStream_t st);
  // out[r] = |x_r|^2; exact: every product formed in FP64 (exact for FP32
  // inputs), else FP32 fields form their products in FP32 (summed in FP64)
  void norm2(const FieldRef& x, double* out, cudaStream_t st, bool exact = true);
  // out[r] = <x_r, y_r> = sum conj(x) y  (double2); FP32 fields form the
  // products in FP32, summed in FP64
  void cdot(const FieldRef& x, const FieldRef& y, double2* out, cudaStream_t st);
  // hi += lo (any BLAS precisions), elementwise
  void add_to(const FieldRef& lo, const FieldRef& hi, cudaStream_t st);
  // y = x, with precision conversion
  void copy(const FieldRef& x, const FieldRef& y, cudaStream_t st);
  void zero(const FieldRef& x, cudaStream_t st);

  static int blocks_for(int64_t n);

 private:
  double* partials_;
  int max_blocks_;
};

}  // namespace qcu
