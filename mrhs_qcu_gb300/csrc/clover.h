// Clover term (clover.cu): the local part A of the Wilson-clover operator
// M = A - kappa D.  The reference reserves the enum value DSLASH_CLOVER
// (include/qcu_enum.h:12) and the per-site storage of the field
// (include/basic_data/qcu_point.cuh:98-101: (Nc*Ns)^2/2 complex per site, two
// 2N x 2N blocks) but has no clover code; this is new work on that layout.
//
// Caller layout (complex double): [parity=2][Vh][block=2][2N][2N], block 0
// acting on spins 0, 1 and block 1 on spins 2, 3 (the chirality blocks of the
// DeGrand-Rossi basis), row / column index = local spin * N + colour.  The
// blocks must be Hermitian (M^dag = A - kappa D^dag then holds).
// Resident layout: [parity][block][(2N)^2][Vh] complex (component-major like
// the gauge), an FP64 master, its per-site inverse (FP64, Gauss-Jordan with
// partial pivoting) and copies in the storage precisions.
#pragma once

#include "dslash_kernel.cuh"
#include "layout.h"

namespace qcu {

// caller [2][Vh][2][2N][2N] -> resident FP64 [2][2][(2N)^2][Vh]
void pack_clover(int N, const void* src, void* dst, int64_t vh, cudaStream_t st);
// per-site inverse of every block of a resident FP64 clover field; returns
// false (after a sync) when a block is singular
bool invert_clover(int N, const void* src, void* dst, int64_t vh, int* flag, cudaStream_t st);

// out = a * C_parity in + b * x on resident MRHS fields (x optional), C in the
// storage precision prec ([2][2][(2N)^2][Vh]); mask: per-RHS activity
void clover_apply(int prec, int N, const DslashArgs& A, const void* clover, cudaStream_t st);

}  // namespace qcu
