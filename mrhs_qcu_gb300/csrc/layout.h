// Host launchers of the layout-transform kernels (layout.cu).
#pragma once

#include "qcu_common.cuh"

namespace qcu {

constexpr int QCU_MAX_RHS = 256;

// caller-side fermion address modes
enum SrcMode : int {
  SRC_EO_HALF = 0,  // pointer to one parity, [Vh][4][N]
  SRC_EO_FULL = 1,  // pointer to [2][Vh][4][N]; the parity argument selects the half
  SRC_LEX = 2,      // pointer to a lexicographic full field [V][4][N]
};

// one device pointer per RHS, passed by value as a kernel parameter
struct PtrArray {
  const void* p[QCU_MAX_RHS];
};

// caller FP64 fermions (nrhs pointers) -> internal MRHS field of `prec`
void pack_fermions(int prec, int N, const PtrArray& src, int mode, int parity, void* dst, float* dst_norm,
                   const Geometry& g, int nrhs, cudaStream_t st);
// internal MRHS field -> caller FP64 fermions
void unpack_fermions(int prec, int N, const PtrArray& dst, int mode, int parity, const void* src,
                     const float* src_norm, const Geometry& g, int nrhs, cudaStream_t st);
// caller FP64 gauge (eo [4][2][Vh][N][N], or lexicographic [4][V][N][N] when
// lex != 0) -> internal [4][2][N*N][Vh] of `prec`
void pack_gauge(int prec, int N, const void* src, int lex, void* dst, const Geometry& g, cudaStream_t st);
// internal FP64 gauge -> caller eo layout
void unpack_gauge_fp64(int N, const void* src, void* dst, const Geometry& g, cudaStream_t st);
// MRHS field precision conversion (same [ncomp][vh][nrhs] layout); RHS whose
// mask entry is 0 are left untouched (mask may be null)
void convert_field(int prec_in, const void* src, const float* src_norm, int prec_out, void* dst, float* dst_norm,
                   int64_t vh, int ncomp, int nrhs, cudaStream_t st, const int* mask = nullptr);
// FP64 internal gauge -> the same layout in `prec` (no scales: |U_ab| <= 1)
void convert_gauge(const void* src_fp64, int prec, void* dst, int64_t count, cudaStream_t st);
// SU(3) gauge compression (the reference's loadGauge2 keeps the first N - 1
// rows, include/kernels/storageLoadStore/loadAndStore.cuh:17-27): the first
// two rows of every link, [8][6][Vh] in precision prec
void compress_gauge_su3(const void* src_fp64, int prec, void* dst, int64_t vh, cudaStream_t st);
// max over the links of |row 2 - conj(row 0 x row 1)| (0 for exact SU(3));
// scratch: one device unsigned
double su3_row_deviation(const void* src_fp64, int64_t vh, unsigned* scratch, cudaStream_t st);
// BF16 links for the spinor-operand tensor-core dslash, one record per output
// site and parity holding the eight links its hops multiply by, already split
// into the rows its link operand is built from:
// [parity 2][Vh][hop 8][part 2][row 8][col 8] BF16, 256 bytes per link and
// 2 KB per site (one bulk copy per site), rows and columns >= N zero.  Hop
// d = 2 mu (forward) holds the rows of U_mu(x) (part 0 Re, part 1 Im); hop
// 2 mu + 1 (backward) the rows of U_mu(x - mu)^T (the columns of that link),
// which the hop uses conjugated.  Each link appears twice, as in a copy per
// form.  Built from the FP64 master [8][N*N][Vh].
constexpr int kTcLinkBytes = 256;
constexpr int kTcRecordBytes = 8 * kTcLinkBytes;
inline size_t tc_links_bytes(int64_t vh) { return (size_t)2 * vh * kTcRecordBytes; }
void gauge_tc_records_bf16(int N, const void* src_fp64, void* dst, const Geometry& geo, cudaStream_t st);
// per-RHS coalesced arrays (the reference's internal layout, one [ncomp][vh]
// complex array per RHS, include/basic_data/qcu_point.cuh:80-88 of the
// reference) <-> one MRHS field [ncomp][vh][nrhs], FP32 or FP64 (no
// conversion).  nrhs <= QCU_MAX_RHS.
void gather_rhs_arrays(int prec, const PtrArray& src, void* dst, int64_t vh, int ncomp, int nrhs, cudaStream_t st);
void scatter_rhs_arrays(int prec, const PtrArray& dst, const void* src, int64_t vh, int ncomp, int nrhs,
                        cudaStream_t st);
// plain complex-double transpose [rows][cols] -> [cols][rows]
void transpose_c64(const void* src, void* dst, int rows, int cols, cudaStream_t st);

}  // namespace qcu
