// Layout transforms between the caller formats of qcu.h and the internal
// device layouts.
//
// Caller formats (complex double, the reference's "non-coalesced" layouts,
// include/kernels/storage/storage_kernels.cuh:14-101 of the reference):
//   fermion, one parity      [Vh][4][N]
//   fermion, full, eo split  [2][Vh][4][N]   (even half first)
//   fermion, lexicographic   [V][4][N]       (site ((t*Lz+z)*Ly+y)*Lx+X)
//   gauge, eo split          [4][2][Vh][N][N]
//   gauge, lexicographic     [4][V][N][N]
// Internal formats: see qcu_common.cuh.
//
// The reference converts one RHS per launch, double SU(3) only
// (src/storage/qcu_storage.cu:9-35).  Here one launch packs every queued RHS
// into one RHS-innermost MRHS field in the target precision (computing the
// per-(site, RHS) scale for 16-bit storage), and the source may be
// lexicographic: the lexicographic -> even-odd map is applied on the fly.
#include <algorithm>

#include <cstring>

#include "layout.h"

namespace qcu {
namespace {

// half-site i of parity p -> source site offset (in units of 4N complexes)
__device__ __forceinline__ int64_t src_site(int mode, int64_t i, int p, const Geometry& g) {
  if (mode == SRC_EO_HALF) return i;
  if (mode == SRC_EO_FULL) return (int64_t)p * g.vh + i;
  // lexicographic
  uint32_t rest, xh, y, z, t, rest2;
  g.div_hx.divmod((uint32_t)i, rest, xh);
  g.div_y.divmod(rest, rest2, y);
  g.div_z.divmod(rest2, t, z);
  const int X = 2 * (int)xh + (p ^ (int)((y + z + t) & 1));
  return (((int64_t)t * g.L[2] + z) * g.L[1] + y) * g.L[0] + X;
}

template <int P, int N>
__global__ void pack_fermions_kernel(PtrArray src, int mode, int parity, void* dst, float* dst_norm, Geometry g,
                                     int nrhs, FastDiv div_nrhs) {
  using S = Store<P>;
  using E = typename S::elem;
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t site, r;
  div_nrhs.divmod(gid, site, r);
  if ((int)site >= g.vh || src.p[r] == nullptr) return;  // a null pointer leaves RHS r untouched
  const double2* s = static_cast<const double2*>(src.p[r]) + src_site(mode, site, parity, g) * (4 * N);
  double2 v[4 * N];
#pragma unroll
  for (int c = 0; c < 4 * N; c++) v[c] = __ldg(s + c);
  // component c at site * ss + c * cs + r (component- or site-major, by P)
  const int64_t cs = field_comp_stride(P, g.vh, 4 * N, nrhs), ss = field_site_stride(P, g.vh, 4 * N, nrhs);
  E* d = static_cast<E*>(dst) + (int64_t)site * ss + r;
  if constexpr (S::has_norm) {
    double m = 0.0;
#pragma unroll
    for (int c = 0; c < 4 * N; c++) m = fmax(m, fmax(fabs(v[c].x), fabs(v[c].y)));
    const float mf = (float)m;
    const double inv = m > 0.0 ? 1.0 / (double)mf : 0.0;
    dst_norm[(int64_t)site * nrhs + r] = mf;
#pragma unroll
    for (int c = 0; c < 4 * N; c++) d[c * cs] = S::from_c(make_float2((float)(v[c].x * inv), (float)(v[c].y * inv)));
  } else {
#pragma unroll
    for (int c = 0; c < 4 * N; c++) {
      E e;
      e.x = v[c].x;
      e.y = v[c].y;
      d[c * cs] = e;
    }
  }
}

template <int P, int N>
__global__ void unpack_fermions_kernel(PtrArray dstp, int mode, int parity, const void* src, const float* src_norm,
                                       Geometry g, int nrhs, FastDiv div_nrhs) {
  using S = Store<P>;
  using E = typename S::elem;
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t site, r;
  div_nrhs.divmod(gid, site, r);
  if ((int)site >= g.vh || dstp.p[r] == nullptr) return;  // a null pointer skips RHS r
  const int64_t cs = field_comp_stride(P, g.vh, 4 * N, nrhs), ss = field_site_stride(P, g.vh, 4 * N, nrhs);
  const E* s = static_cast<const E*>(src) + (int64_t)site * ss + r;
  double2* d = static_cast<double2*>(const_cast<void*>(dstp.p[r])) + src_site(mode, site, parity, g) * (4 * N);
  double scale = 1.0;
  if constexpr (S::has_norm) scale = (double)src_norm[(int64_t)site * nrhs + r];
#pragma unroll
  for (int c = 0; c < 4 * N; c++) {
    auto v = S::to_c(s[c * cs]);
    d[c] = make_double2((double)v.x * scale, (double)v.y * scale);
  }
}

// Unpack through a shared-memory tile (caller layouts whose sites are
// contiguous: one parity or both parities in eo order).  A block stages ts
// sites x tr RHS of the MRHS field as FP64 complex: the reads walk the
// field's contiguous (site, RHS) runs of each component, the writes each
// RHS's contiguous run of ts sites x 4N caller components.  (One thread per
// (site, RHS) scatters every warp's writes over up to 32 RHS arrays.)
template <int P, int N>
__global__ void unpack_fermions_tiled_kernel(PtrArray dstp, int mode, int parity, const void* src,
                                             const float* src_norm, Geometry g, int nrhs, int ts, int tr) {
  using S = Store<P>;
  using E = typename S::elem;
  constexpr int NC = 4 * N;
  extern __shared__ double2 tile[];  // [tr][ts][NC]
  const int64_t site0 = (int64_t)blockIdx.x * ts;
  const int r0 = blockIdx.y * tr;
  const int64_t cs = field_comp_stride(P, g.vh, NC, nrhs), ss = field_site_stride(P, g.vh, NC, nrhs);
  const E* in = static_cast<const E*>(src);
  const int n = NC * ts * tr;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int r = i % tr, s = (i / tr) % ts, c = i / (tr * ts);
    const int64_t site = site0 + s;
    const int rhs = r0 + r;
    if (site >= g.vh || rhs >= nrhs) continue;
    const auto v = S::to_c(in[site * ss + c * cs + rhs]);
    double scale = 1.0;
    if constexpr (S::has_norm) scale = (double)src_norm[site * nrhs + rhs];
    tile[((int64_t)r * ts + s) * NC + c] = make_double2((double)v.x * scale, (double)v.y * scale);
  }
  __syncthreads();
  const int64_t base = (mode == SRC_EO_FULL ? (int64_t)parity * g.vh : 0) + site0;  // caller site of site0
  const int nsites = (int)min((int64_t)ts, g.vh - site0);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int r = i / (ts * NC), rem = i - r * ts * NC;
    const int rhs = r0 + r;
    if (rem >= nsites * NC || rhs >= nrhs || dstp.p[rhs] == nullptr) continue;  // a null pointer skips RHS r
    static_cast<double2*>(const_cast<void*>(dstp.p[rhs]))[base * NC + rem] = tile[(int64_t)r * ts * NC + rem];
  }
}

// gauge: caller (eo or lexicographic) complex double -> [4][2][N*N][Vh] P
template <int P>
__global__ void pack_gauge_kernel(const double2* __restrict__ src, int lex, void* dst, Geometry g, int nn) {
  using S = Store<P>;
  using E = typename S::elem;
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // over 4 * 2 * vh
  if (gid >= (int64_t)8 * g.vh) return;
  const int64_t i = gid % g.vh;
  const int mp = (int)(gid / g.vh);  // mu * 2 + parity
  const int mu = mp >> 1, p = mp & 1;
  int64_t s;
  if (lex)
    s = (int64_t)mu * 2 * g.vh + src_site(SRC_LEX, i, p, g);
  else
    s = (int64_t)mp * g.vh + i;
  const double2* a = src + s * nn;
  E* d = static_cast<E*>(dst) + (int64_t)mp * nn * g.vh + i;
  for (int k = 0; k < nn; k++) {
    double2 v = __ldg(a + k);
    E e;
    if constexpr (P == PREC_DOUBLE) {
      e = v;
    } else if constexpr (P == PREC_SINGLE) {
      e = make_float2((float)v.x, (float)v.y);
    } else {
      e = S::from_c(make_float2((float)v.x, (float)v.y));
    }
    d[(int64_t)k * g.vh] = e;
  }
}

// internal FP64 gauge -> caller eo layout (the reference's TO_NON_COALESCE)
__global__ void unpack_gauge_kernel(const double2* __restrict__ src, double2* dst, int vh, int nn) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= (int64_t)8 * vh) return;
  const int64_t i = gid % vh;
  const int mp = (int)(gid / vh);
  const double2* s = src + (int64_t)mp * nn * vh + i;
  double2* d = dst + ((int64_t)mp * vh + i) * nn;
  for (int k = 0; k < nn; k++) d[k] = s[(int64_t)k * vh];
}

// convert an MRHS field between storage precisions (and layouts)
template <int PI, int PO>
__global__ void convert_field_kernel(const void* src, const float* src_norm, void* dst, float* dst_norm,
                                     int64_t vh, int ncomp, int nrhs, FastDiv div_nrhs, const int* mask) {
  using SI = Store<PI>;
  using SO = Store<PO>;
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t site, r;
  div_nrhs.divmod(gid, site, r);
  if ((int64_t)site >= vh || (mask && !mask[r])) return;  // masked RHS keep their values
  // component c at site * ss + c * cs + r, strides by each side's layout
  const int64_t csi = field_comp_stride(PI, vh, ncomp, nrhs), csd = field_comp_stride(PO, vh, ncomp, nrhs);
  const auto* s = static_cast<const typename SI::elem*>(src) + (int64_t)site * field_site_stride(PI, vh, ncomp, nrhs) + r;
  auto* d = static_cast<typename SO::elem*>(dst) + (int64_t)site * field_site_stride(PO, vh, ncomp, nrhs) + r;
  double si = 1.0;
  if constexpr (SI::has_norm) si = (double)src_norm[(int64_t)site * nrhs + r];
  double m = 0.0;
  if constexpr (SO::has_norm) {
    for (int c = 0; c < ncomp; c++) {
      auto v = SI::to_c(s[c * csi]);
      m = fmax(m, fmax(fabs((double)v.x * si), fabs((double)v.y * si)));
    }
    dst_norm[(int64_t)site * nrhs + r] = (float)m;
  }
  const double inv = SO::has_norm ? (m > 0.0 ? 1.0 / (double)(float)m : 0.0) : 1.0;
  for (int c = 0; c < ncomp; c++) {
    auto v = SI::to_c(s[c * csi]);
    const double re = (double)v.x * si * inv, im = (double)v.y * si * inv;
    typename SO::elem e;
    if constexpr (PO == PREC_DOUBLE) {
      e = make_double2(re, im);
    } else if constexpr (PO == PREC_SINGLE) {
      e = make_float2((float)re, (float)im);
    } else {
      e = SO::from_c(make_float2((float)re, (float)im));
    }
    d[c * csd] = e;
  }
}

template <int P>
__global__ void convert_gauge_kernel(const double2* __restrict__ src, void* dst, int64_t count) {
  using S = Store<P>;
  using E = typename S::elem;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const double2 v = src[i];
    E e;
    if constexpr (P == PREC_DOUBLE) {
      e = v;
    } else if constexpr (P == PREC_SINGLE) {
      e = make_float2((float)v.x, (float)v.y);
    } else {
      e = S::from_c(make_float2((float)v.x, (float)v.y));
    }
    static_cast<E*>(dst)[i] = e;
  }
}

// SU(3) links stored as their first two rows ([8][6][Vh] from the FP64 master
// [8][9][Vh]: components 0..5 of every (mu, parity) block), converted to P
template <int P>
__global__ void compress_gauge_kernel(const double2* __restrict__ src, void* dst, int64_t vh) {
  using S = Store<P>;
  using E = typename S::elem;
  const int64_t count = 8 * 6 * vh;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const int64_t blk = i / (6 * vh), rem = i - blk * 6 * vh;  // rem = comp * vh + site, comp < 6
    const int64_t comp = rem / vh, site = rem - comp * vh;
    const double2 v = src[blk * 9 * vh + rem];
    E e;
    if constexpr (P == PREC_DOUBLE) {
      e = v;
    } else if constexpr (P == PREC_SINGLE) {
      e = make_float2((float)v.x, (float)v.y);
    } else {
      e = S::from_c(make_float2((float)v.x, (float)v.y));
    }
    // [8][Vh/32][6][32] (Vh padded to 32): the groups of 32 sites of dslash_kernel.cuh two_row_site
    const int64_t vhp = (vh + 31) / 32 * 32;
    static_cast<E*>(dst)[blk * 6 * vhp + (site >> 5) * 192 + comp * 32 + (site & 31)] = e;
  }
}

// max over links of |row 2 - conj(row 0 x row 1)| (FP64 master [8][9][Vh]);
// the maximum of non-negative floats as their bit patterns
__global__ void su3_row_check_kernel(const double2* __restrict__ g, int64_t vh, unsigned* out) {
  const int64_t n = 8 * vh;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  float mx = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t blk = i / vh, site = i - blk * vh;
    double2 u[9];
#pragma unroll
    for (int k = 0; k < 9; k++) u[k] = g[(blk * 9 + k) * vh + site];
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const int k = (j + 1) % 3, l = (j + 2) % 3;
      // conj(u0k u1l - u0l u1k)
      const double re = (u[k].x * u[3 + l].x - u[k].y * u[3 + l].y) - (u[l].x * u[3 + k].x - u[l].y * u[3 + k].y);
      const double im = (u[k].x * u[3 + l].y + u[k].y * u[3 + l].x) - (u[l].x * u[3 + k].y + u[l].y * u[3 + k].x);
      const double dr = u[6 + j].x - re, di = u[6 + j].y + im;
      mx = fmaxf(mx, (float)sqrt(dr * dr + di * di));
    }
  }
  atomicMax(out, __float_as_uint(mx));
}

// [rows][cols] -> [cols][rows] complex double transpose through shared memory
__global__ void transpose_c64_kernel(const double2* __restrict__ src, double2* __restrict__ dst, int rows, int cols) {
  __shared__ double2 tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = by + j, c = bx + threadIdx.x;
    if (r < rows && c < cols) tile[j][threadIdx.x] = src[(int64_t)r * cols + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int c = bx + j, r = by + threadIdx.x;
    if (r < rows && c < cols) dst[(int64_t)c * rows + r] = tile[threadIdx.x][j];
  }
}

template <int N>
void pack_n(int prec, const PtrArray& src, int mode, int parity, void* dst, float* dst_norm, const Geometry& g,
            int nrhs, cudaStream_t st) {
  const int64_t threads = (int64_t)g.vh * nrhs;
  const int block = 128;
  const int grid = (int)((threads + block - 1) / block);
  FastDiv dn((uint32_t)nrhs);
  switch (prec) {
    case PREC_DOUBLE: pack_fermions_kernel<PREC_DOUBLE, N><<<grid, block, 0, st>>>(src, mode, parity, dst, dst_norm, g, nrhs, dn); break;
    case PREC_SINGLE: pack_fermions_kernel<PREC_SINGLE, N><<<grid, block, 0, st>>>(src, mode, parity, dst, dst_norm, g, nrhs, dn); break;
    case PREC_HALF: pack_fermions_kernel<PREC_HALF, N><<<grid, block, 0, st>>>(src, mode, parity, dst, dst_norm, g, nrhs, dn); break;
    case PREC_BF16: pack_fermions_kernel<PREC_BF16, N><<<grid, block, 0, st>>>(src, mode, parity, dst, dst_norm, g, nrhs, dn); break;
    case PREC_BF16S: pack_fermions_kernel<PREC_BF16S, N><<<grid, block, 0, st>>>(src, mode, parity, dst, dst_norm, g, nrhs, dn); break;
  }
}

template <int N>
void unpack_n(int prec, const PtrArray& dst, int mode, int parity, const void* src, const float* src_norm,
              const Geometry& g, int nrhs, cudaStream_t st) {
  if (mode != SRC_LEX) {
    // tiles of ts sites x tr RHS, 24 KB of FP64 complex in shared memory (32^3x64, FP32,
    // nrhs 12: 0.83 ms, against 1.15 ms with 48 KB tiles and 0.89 ms with 12 KB)
    const int tr = std::min(nrhs, 16);
    const int ts = std::max(1, std::min(32, 1536 / (tr * 4 * N)));
    const dim3 grid((unsigned)((g.vh + ts - 1) / ts), (unsigned)((nrhs + tr - 1) / tr));
    const size_t smem = (size_t)ts * tr * 4 * N * sizeof(double2);
#define QCU_UNPACK_TILED(PR)                                                                                      \
  unpack_fermions_tiled_kernel<PR, N><<<grid, 256, smem, st>>>(dst, mode, parity, src, src_norm, g, nrhs, ts, tr); \
  return;
    switch (prec) {
      case PREC_DOUBLE: QCU_UNPACK_TILED(PREC_DOUBLE)
      case PREC_SINGLE: QCU_UNPACK_TILED(PREC_SINGLE)
      case PREC_HALF: QCU_UNPACK_TILED(PREC_HALF)
      case PREC_BF16: QCU_UNPACK_TILED(PREC_BF16)
      case PREC_BF16S: QCU_UNPACK_TILED(PREC_BF16S)
    }
#undef QCU_UNPACK_TILED
  }
  const int64_t threads = (int64_t)g.vh * nrhs;
  const int block = 128;
  const int grid = (int)((threads + block - 1) / block);
  FastDiv dn((uint32_t)nrhs);
  switch (prec) {
    case PREC_DOUBLE: unpack_fermions_kernel<PREC_DOUBLE, N><<<grid, block, 0, st>>>(dst, mode, parity, src, src_norm, g, nrhs, dn); break;
    case PREC_SINGLE: unpack_fermions_kernel<PREC_SINGLE, N><<<grid, block, 0, st>>>(dst, mode, parity, src, src_norm, g, nrhs, dn); break;
    case PREC_HALF: unpack_fermions_kernel<PREC_HALF, N><<<grid, block, 0, st>>>(dst, mode, parity, src, src_norm, g, nrhs, dn); break;
    case PREC_BF16: unpack_fermions_kernel<PREC_BF16, N><<<grid, block, 0, st>>>(dst, mode, parity, src, src_norm, g, nrhs, dn); break;
    case PREC_BF16S: unpack_fermions_kernel<PREC_BF16S, N><<<grid, block, 0, st>>>(dst, mode, parity, src, src_norm, g, nrhs, dn); break;
  }
}

}  // namespace

void pack_fermions(int prec, int N, const PtrArray& src, int mode, int parity, void* dst, float* dst_norm,
                   const Geometry& g, int nrhs, cudaStream_t st) {
  QCU_REQUIRE(nrhs >= 1 && nrhs <= QCU_MAX_RHS, QCU_ERR_INVALID_ARGUMENT, "nrhs out of range");
  QCU_REQUIRE((int64_t)g.vh * nrhs < (1ll << 31), QCU_ERR_INVALID_ARGUMENT, "lattice x nrhs too large");
  switch (N) {
    case 3: pack_n<3>(prec, src, mode, parity, dst, dst_norm, g, nrhs, st); break;
    case 4: pack_n<4>(prec, src, mode, parity, dst, dst_norm, g, nrhs, st); break;
    case 5: pack_n<5>(prec, src, mode, parity, dst, dst_norm, g, nrhs, st); break;
    case 6: pack_n<6>(prec, src, mode, parity, dst, dst_norm, g, nrhs, st); break;
    case 7: pack_n<7>(prec, src, mode, parity, dst, dst_norm, g, nrhs, st); break;
    case 8: pack_n<8>(prec, src, mode, parity, dst, dst_norm, g, nrhs, st); break;
    default: throw Error(QCU_ERR_UNSUPPORTED, "nColors must be in 3..8");
  }
  QCU_CHECK_CUDA(cudaGetLastError());
}

void unpack_fermions(int prec, int N, const PtrArray& dst, int mode, int parity, const void* src,
                     const float* src_norm, const Geometry& g, int nrhs, cudaStream_t st) {
  QCU_REQUIRE(nrhs >= 1 && nrhs <= QCU_MAX_RHS, QCU_ERR_INVALID_ARGUMENT, "nrhs out of range");
  QCU_REQUIRE((int64_t)g.vh * nrhs < (1ll << 31), QCU_ERR_INVALID_ARGUMENT, "lattice x nrhs too large");
  switch (N) {
    case 3: unpack_n<3>(prec, dst, mode, parity, src, src_norm, g, nrhs, st); break;
    case 4: unpack_n<4>(prec, dst, mode, parity, src, src_norm, g, nrhs, st); break;
    case 5: unpack_n<5>(prec, dst, mode, parity, src, src_norm, g, nrhs, st); break;
    case 6: unpack_n<6>(prec, dst, mode, parity, src, src_norm, g, nrhs, st); break;
    case 7: unpack_n<7>(prec, dst, mode, parity, src, src_norm, g, nrhs, st); break;
    case 8: unpack_n<8>(prec, dst, mode, parity, src, src_norm, g, nrhs, st); break;
    default: throw Error(QCU_ERR_UNSUPPORTED, "nColors must be in 3..8");
  }
  QCU_CHECK_CUDA(cudaGetLastError());
}

void pack_gauge(int prec, int N, const void* src, int lex, void* dst, const Geometry& g, cudaStream_t st) {
  const int64_t threads = (int64_t)8 * g.vh;
  const int block = 256;
  const int grid = (int)((threads + block - 1) / block);
  const double2* s = static_cast<const double2*>(src);
  switch (prec) {
    case PREC_DOUBLE: pack_gauge_kernel<PREC_DOUBLE><<<grid, block, 0, st>>>(s, lex, dst, g, N * N); break;
    case PREC_SINGLE: pack_gauge_kernel<PREC_SINGLE><<<grid, block, 0, st>>>(s, lex, dst, g, N * N); break;
    case PREC_HALF: pack_gauge_kernel<PREC_HALF><<<grid, block, 0, st>>>(s, lex, dst, g, N * N); break;
    case PREC_BF16: pack_gauge_kernel<PREC_BF16><<<grid, block, 0, st>>>(s, lex, dst, g, N * N); break;
    default: throw Error(QCU_ERR_UNSUPPORTED, "bad precision");
  }
  QCU_CHECK_CUDA(cudaGetLastError());
}

void unpack_gauge_fp64(int N, const void* src, void* dst, const Geometry& g, cudaStream_t st) {
  const int64_t threads = (int64_t)8 * g.vh;
  const int block = 256;
  const int grid = (int)((threads + block - 1) / block);
  unpack_gauge_kernel<<<grid, block, 0, st>>>(static_cast<const double2*>(src), static_cast<double2*>(dst), g.vh,
                                              N * N);
  QCU_CHECK_CUDA(cudaGetLastError());
}

void convert_field(int prec_in, const void* src, const float* src_norm, int prec_out, void* dst, float* dst_norm,
                   int64_t vh, int ncomp, int nrhs, cudaStream_t st, const int* mask) {
  const int64_t threads = vh * nrhs;
  QCU_REQUIRE(threads < (1ll << 31), QCU_ERR_INVALID_ARGUMENT, "field too large");
  const int block = 256;
  const int grid = (int)((threads + block - 1) / block);
  FastDiv dn((uint32_t)nrhs);
#define QCU_CONV(PI, PO)                                                                                             \
  if (prec_in == PI && prec_out == PO) {                                                                             \
    convert_field_kernel<PI, PO><<<grid, block, 0, st>>>(src, src_norm, dst, dst_norm, vh, ncomp, nrhs, dn, mask);  \
    QCU_CHECK_CUDA(cudaGetLastError());                                                                              \
    return;                                                                                                          \
  }
  QCU_CONV(PREC_DOUBLE, PREC_SINGLE)
  QCU_CONV(PREC_DOUBLE, PREC_HALF)
  QCU_CONV(PREC_DOUBLE, PREC_BF16)
  QCU_CONV(PREC_SINGLE, PREC_DOUBLE)
  QCU_CONV(PREC_HALF, PREC_DOUBLE)
  QCU_CONV(PREC_BF16, PREC_DOUBLE)
  QCU_CONV(PREC_SINGLE, PREC_HALF)
  QCU_CONV(PREC_SINGLE, PREC_BF16)
  QCU_CONV(PREC_HALF, PREC_SINGLE)
  QCU_CONV(PREC_BF16, PREC_SINGLE)
  QCU_CONV(PREC_DOUBLE, PREC_DOUBLE)
  QCU_CONV(PREC_SINGLE, PREC_SINGLE)
  QCU_CONV(PREC_HALF, PREC_HALF)
  QCU_CONV(PREC_BF16, PREC_BF16)
  QCU_CONV(PREC_DOUBLE, PREC_BF16S)
  QCU_CONV(PREC_BF16S, PREC_DOUBLE)
  QCU_CONV(PREC_SINGLE, PREC_BF16S)
  QCU_CONV(PREC_BF16S, PREC_SINGLE)
  QCU_CONV(PREC_BF16, PREC_BF16S)
  QCU_CONV(PREC_BF16S, PREC_BF16)
  QCU_CONV(PREC_BF16S, PREC_BF16S)
#undef QCU_CONV
  throw Error(QCU_ERR_UNSUPPORTED, "unsupported precision conversion");
}

void convert_gauge(const void* src_fp64, int prec, void* dst, int64_t count, cudaStream_t st) {
  const int block = 256;
  const int grid = (int)std::min<int64_t>((count + block - 1) / block, 152 * 32);
  const double2* s = static_cast<const double2*>(src_fp64);
  switch (prec) {
    case PREC_DOUBLE: convert_gauge_kernel<PREC_DOUBLE><<<grid, block, 0, st>>>(s, dst, count); break;
    case PREC_SINGLE: convert_gauge_kernel<PREC_SINGLE><<<grid, block, 0, st>>>(s, dst, count); break;
    case PREC_HALF: convert_gauge_kernel<PREC_HALF><<<grid, block, 0, st>>>(s, dst, count); break;
    case PREC_BF16: convert_gauge_kernel<PREC_BF16><<<grid, block, 0, st>>>(s, dst, count); break;
    default: throw Error(QCU_ERR_UNSUPPORTED, "bad precision");
  }
  QCU_CHECK_CUDA(cudaGetLastError());
}

void compress_gauge_su3(const void* src_fp64, int prec, void* dst, int64_t vh, cudaStream_t st) {
  const int block = 256;
  const int grid = (int)std::min<int64_t>((48 * vh + block - 1) / block, 152 * 32);
  const double2* s = static_cast<const double2*>(src_fp64);
  switch (prec) {
    case PREC_DOUBLE: compress_gauge_kernel<PREC_DOUBLE><<<grid, block, 0, st>>>(s, dst, vh); break;
    case PREC_SINGLE: compress_gauge_kernel<PREC_SINGLE><<<grid, block, 0, st>>>(s, dst, vh); break;
    case PREC_HALF: compress_gauge_kernel<PREC_HALF><<<grid, block, 0, st>>>(s, dst, vh); break;
    case PREC_BF16: compress_gauge_kernel<PREC_BF16><<<grid, block, 0, st>>>(s, dst, vh); break;
    default: throw Error(QCU_ERR_UNSUPPORTED, "bad precision");
  }
  QCU_CHECK_CUDA(cudaGetLastError());
}

namespace {
// one thread per 4-byte word (two BF16 of adjacent columns) of the destination
__global__ void gauge_tc_records_kernel(const double2* __restrict__ src, uint32_t* __restrict__ dst, Geometry geo,
                                        int N) {
  const int64_t vh = geo.vh;
  const int64_t n = 2 * vh * 8 * 64;  // 64 words per link
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int w = (int)(i & 63);
    const int d = (int)((i >> 6) & 7);
    const int64_t ps = i >> 9;  // p * vh + site
    const uint32_t site = (uint32_t)(ps % vh), p = (uint32_t)(ps / vh);
    // hop d = 2 mu + b: forward hops multiply by U_mu(x) (rows of U, form 0),
    // backward hops by U_mu(x - mu)^dag (rows of U^T, form 1) from the other parity
    const int mu = d >> 1, form = d & 1;
    const uint32_t lpar = form ? 1u - p : p;
    const uint32_t lsite = form ? EoSite(geo, site).nb(geo, p, d) : site;
    const int64_t blk = 2 * mu + lpar;
    const int part = w >> 5, row = (w >> 2) & 7, c0 = 2 * (w & 3);
    float v[2] = {0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const int col = c0 + k;
      if (row < N && col < N) {
        const int comp = form == 0 ? row * N + col : col * N + row;  // U[row][col] or U[col][row]
        const double2 u = src[(blk * N * N + comp) * vh + lsite];
        v[k] = (float)(part ? u.y : u.x);
      }
    }
    const __nv_bfloat162 b = __floats2bfloat162_rn(v[0], v[1]);
    dst[i] = *reinterpret_cast<const uint32_t*>(&b);
  }
}
}  // namespace

void gauge_tc_records_bf16(int N, const void* src_fp64, void* dst, const Geometry& geo, cudaStream_t st) {
  const int block = 256;
  const int grid = (int)std::min<int64_t>((2 * (int64_t)geo.vh * 8 * 64 + block - 1) / block, 152 * 32);
  gauge_tc_records_kernel<<<grid, block, 0, st>>>(static_cast<const double2*>(src_fp64), static_cast<uint32_t*>(dst),
                                                  geo, N);
  QCU_CHECK_CUDA(cudaGetLastError());
}

double su3_row_deviation(const void* src_fp64, int64_t vh, unsigned* scratch, cudaStream_t st) {
  QCU_CHECK_CUDA(cudaMemsetAsync(scratch, 0, sizeof(unsigned), st));
  const int block = 256;
  const int grid = (int)std::min<int64_t>((8 * vh + block - 1) / block, 152 * 8);
  su3_row_check_kernel<<<grid, block, 0, st>>>(static_cast<const double2*>(src_fp64), vh, scratch);
  QCU_CHECK_CUDA(cudaGetLastError());
  unsigned v = 0;
  QCU_CHECK_CUDA(cudaMemcpyAsync(&v, scratch, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  QCU_CHECK_CUDA(cudaStreamSynchronize(st));
  float f;
  memcpy(&f, &v, sizeof(f));
  return (double)f;
}

namespace {
// element e of the MRHS field = (c * vh + site) * nrhs + r; RHS fastest, so a
// warp writes one contiguous span and reads nrhs short runs
template <typename E, bool GATHER>
__global__ void rhs_arrays_kernel(PtrArray arrays, void* field, int64_t n, FastDiv div_nrhs) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t q = (uint64_t)e / div_nrhs.d;
    const uint32_t r = (uint32_t)(e - (int64_t)q * div_nrhs.d);
    if (GATHER)
      static_cast<E*>(field)[e] = static_cast<const E*>(arrays.p[r])[q];
    else
      const_cast<E*>(static_cast<const E*>(arrays.p[r]))[q] = static_cast<const E*>(field)[e];
  }
}

template <bool GATHER>
void rhs_arrays(int prec, const PtrArray& arrays, void* field, int64_t vh, int ncomp, int nrhs, cudaStream_t st) {
  QCU_REQUIRE(prec == PREC_SINGLE || prec == PREC_DOUBLE, QCU_ERR_UNSUPPORTED,
              "per-RHS arrays are FP32 or FP64");
  QCU_REQUIRE(nrhs >= 1 && nrhs <= QCU_MAX_RHS, QCU_ERR_INVALID_ARGUMENT, "nrhs out of range");
  const int64_t n = vh * ncomp * nrhs;
  const int block = 256;
  const int grid = (int)std::min<int64_t>((n + block - 1) / block, 152 * 32);
  const FastDiv d((uint32_t)nrhs);
  if (prec == PREC_SINGLE)
    rhs_arrays_kernel<float2, GATHER><<<grid, block, 0, st>>>(arrays, field, n, d);
  else
    rhs_arrays_kernel<double2, GATHER><<<grid, block, 0, st>>>(arrays, field, n, d);
  QCU_CHECK_CUDA(cudaGetLastError());
}
}  // namespace

void gather_rhs_arrays(int prec, const PtrArray& src, void* dst, int64_t vh, int ncomp, int nrhs, cudaStream_t st) {
  rhs_arrays<true>(prec, src, dst, vh, ncomp, nrhs, st);
}

void scatter_rhs_arrays(int prec, const PtrArray& dst, const void* src, int64_t vh, int ncomp, int nrhs,
                        cudaStream_t st) {
  rhs_arrays<false>(prec, dst, const_cast<void*>(src), vh, ncomp, nrhs, st);
}

void transpose_c64(const void* src, void* dst, int rows, int cols, cudaStream_t st) {
  dim3 block(32, 8);
  dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  transpose_c64_kernel<<<grid, block, 0, st>>>(static_cast<const double2*>(src), static_cast<double2*>(dst), rows,
                                               cols);
  QCU_CHECK_CUDA(cudaGetLastError());
}

}  // namespace qcu
