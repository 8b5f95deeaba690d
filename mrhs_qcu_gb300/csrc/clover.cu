// Clover term: packing, per-site inversion and the MRHS apply (clover.h).
#include <algorithm>

#include "clover.h"

namespace qcu {
namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

template <int N>
__global__ void pack_clover_kernel(const double2* __restrict__ src, double2* __restrict__ dst, int64_t vh) {
  constexpr int B = 4 * N * N;  // (2N)^2 entries per block
  const int64_t n = 4 * vh * B;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t e = i % B, rest = i / B;  // src: ((p * vh + site) * 2 + blk) * B + e
    const int64_t blk = rest % 2, ps = rest / 2, site = ps % vh, p = ps / vh;
    dst[((p * 2 + blk) * B + e) * vh + site] = src[i];
  }
}

// Gauss-Jordan with partial pivoting, one (parity, block, site) per thread
template <int N>
__global__ void invert_clover_kernel(const double2* __restrict__ src, double2* __restrict__ dst, int64_t vh,
                                     int* flag) {
  constexpr int M = 2 * N, B = M * M;
  const int64_t n = 4 * vh;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t pb = i / vh, site = i - pb * vh;
    double2 a[M][M], b[M][M];
    for (int r = 0; r < M; r++)
      for (int c = 0; c < M; c++) {
        a[r][c] = src[(pb * B + r * M + c) * vh + site];
        b[r][c] = make_double2(r == c ? 1.0 : 0.0, 0.0);
      }
    bool singular = false;
    for (int col = 0; col < M && !singular; col++) {
      int piv = col;
      double best = a[col][col].x * a[col][col].x + a[col][col].y * a[col][col].y;
      for (int r = col + 1; r < M; r++) {
        const double m = a[r][col].x * a[r][col].x + a[r][col].y * a[r][col].y;
        if (m > best) {
          best = m;
          piv = r;
        }
      }
      if (!(best > 0.0)) {
        singular = true;
        break;
      }
      if (piv != col)
        for (int c = 0; c < M; c++) {
          const double2 ta = a[col][c], tb = b[col][c];
          a[col][c] = a[piv][c];
          b[col][c] = b[piv][c];
          a[piv][c] = ta;
          b[piv][c] = tb;
        }
      const double2 d = a[col][col];
      const double2 inv = make_double2(d.x / best, -d.y / best);  // 1 / d
      for (int c = 0; c < M; c++) {
        a[col][c] = cmul(a[col][c], inv);
        b[col][c] = cmul(b[col][c], inv);
      }
      for (int r = 0; r < M; r++) {
        if (r == col) continue;
        const double2 fct = a[r][col];
        for (int c = 0; c < M; c++) {
          const double2 pa = cmul(fct, a[col][c]), pb2 = cmul(fct, b[col][c]);
          a[r][c] = make_double2(a[r][c].x - pa.x, a[r][c].y - pa.y);
          b[r][c] = make_double2(b[r][c].x - pb2.x, b[r][c].y - pb2.y);
        }
      }
    }
    if (singular) atomicExch(flag, 1);
    for (int r = 0; r < M; r++)
      for (int c = 0; c < M; c++) dst[(pb * B + r * M + c) * vh + site] = b[r][c];
  }
}

// out = a * C_parity in + b * x: one thread = one site x R RHS
template <int P, int N, int R>
__global__ void __launch_bounds__(128) clover_apply_kernel(const DslashArgs A, const void* clover_v) {
  using namespace detail;
  using S = Store<P>;
  using T = typename S::real;
  using E = typename S::elem;
  constexpr int M = 2 * N, B = M * M;
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t site, grp;
  A.div_groups.divmod(gid, site, grp);
  if (site >= (uint32_t)A.geo.vh) return;
  const uint32_t rhs0 = grp * R;
  if (A.mask) {
    bool any = false;
#pragma unroll
    for (int r = 0; r < R; r++) any |= A.mask[rhs0 + r] != 0;
    if (!any) return;
  }
  const uint32_t vh = A.geo.vh, nrhs = A.nrhs, cs = vh * nrhs, o = site * nrhs + rhs0;
  T scale[R];
  if constexpr (S::has_norm) {
    float nr[R];
    load_norms<P, R>(A.in_norm + o, nr);
#pragma unroll
    for (int r = 0; r < R; r++) scale[r] = nr[r];
  } else {
#pragma unroll
    for (int r = 0; r < R; r++) scale[r] = (T)1;
  }
  const E* __restrict__ in = static_cast<const E*>(A.in);
  C2<T> v[4][N][R], acc[4][N][R];
#pragma unroll
  for (int sp = 0; sp < 4; sp++)
#pragma unroll
    for (int c = 0; c < N; c++) {
      VecBuf<E, R> buf;
      Vec<E, R>::load(in + (o + (uint32_t)(sp * N + c) * cs), buf.v);
#pragma unroll
      for (int r = 0; r < R; r++) {
        const auto x = S::to_c(buf.v[r]);
        v[sp][c][r].x = (T)x.x * scale[r];
        v[sp][c][r].y = (T)x.y * scale[r];
        acc[sp][c][r].x = acc[sp][c][r].y = (T)0;
      }
    }
  const E* __restrict__ cl = static_cast<const E*>(clover_v) + (uint64_t)A.parity * 2 * B * vh + site;
#pragma unroll
  for (int blk = 0; blk < 2; blk++)
#pragma unroll
    for (int row = 0; row < M; row++)
#pragma unroll
      for (int col = 0; col < M; col++) {
        const auto m = S::to_c(__ldg(cl + (uint64_t)(blk * B + row * M + col) * vh));
        const T mr = (T)m.x, mi = (T)m.y;
        const int so = 2 * blk + row / N, co = row % N, si = 2 * blk + col / N, ci = col % N;
#pragma unroll
        for (int r = 0; r < R; r++) {
          acc[so][co][r].x = fma(mr, v[si][ci][r].x, acc[so][co][r].x);
          acc[so][co][r].x = fma(-mi, v[si][ci][r].y, acc[so][co][r].x);
          acc[so][co][r].y = fma(mr, v[si][ci][r].y, acc[so][co][r].y);
          acc[so][co][r].y = fma(mi, v[si][ci][r].x, acc[so][co][r].y);
        }
      }
  store_out<P, N, R>(acc, A, site, rhs0);
}

template <int P, int N>
void launch_clover(const DslashArgs& A0, const void* clover, cudaStream_t st) {
  DslashArgs A = A0;
  const int R = (P != PREC_DOUBLE && A.nrhs % 2 == 0 && N == 3) ? 2 : 1;
  A.div_groups = FastDiv((uint32_t)(A.nrhs / R));
  A.af = (float)A.a;
  A.bf = (float)A.b;
  const int64_t threads = (int64_t)A.geo.vh * (A.nrhs / R);
  const int block = 128, grid = (int)((threads + block - 1) / block);
  if (R == 2) {
    if constexpr (N == 3 && P != PREC_DOUBLE) clover_apply_kernel<P, N, 2><<<grid, block, 0, st>>>(A, clover);
  } else {
    clover_apply_kernel<P, N, 1><<<grid, block, 0, st>>>(A, clover);
  }
  QCU_CHECK_CUDA(cudaGetLastError());
}

template <int P>
void launch_clover_n(int N, const DslashArgs& A, const void* clover, cudaStream_t st) {
  switch (N) {
    case 3: launch_clover<P, 3>(A, clover, st); break;
    case 4: launch_clover<P, 4>(A, clover, st); break;
    case 5: launch_clover<P, 5>(A, clover, st); break;
    case 6: launch_clover<P, 6>(A, clover, st); break;
    case 7: launch_clover<P, 7>(A, clover, st); break;
    case 8: launch_clover<P, 8>(A, clover, st); break;
    default: throw Error(QCU_ERR_UNSUPPORTED, "clover: N must be 3..8");
  }
}

}  // namespace

void pack_clover(int N, const void* src, void* dst, int64_t vh, cudaStream_t st) {
  const int block = 256;
  const int64_t n = 4 * vh * 4 * N * N;
  const int grid = (int)std::min<int64_t>((n + block - 1) / block, 152 * 32);
  const double2* s = static_cast<const double2*>(src);
  double2* d = static_cast<double2*>(dst);
  switch (N) {
    case 3: pack_clover_kernel<3><<<grid, block, 0, st>>>(s, d, vh); break;
    case 4: pack_clover_kernel<4><<<grid, block, 0, st>>>(s, d, vh); break;
    case 5: pack_clover_kernel<5><<<grid, block, 0, st>>>(s, d, vh); break;
    case 6: pack_clover_kernel<6><<<grid, block, 0, st>>>(s, d, vh); break;
    case 7: pack_clover_kernel<7><<<grid, block, 0, st>>>(s, d, vh); break;
    case 8: pack_clover_kernel<8><<<grid, block, 0, st>>>(s, d, vh); break;
    default: throw Error(QCU_ERR_UNSUPPORTED, "clover: N must be 3..8");
  }
  QCU_CHECK_CUDA(cudaGetLastError());
}

bool invert_clover(int N, const void* src, void* dst, int64_t vh, int* flag, cudaStream_t st) {
  QCU_CHECK_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
  const int block = 128;
  const int grid = (int)std::min<int64_t>((4 * vh + block - 1) / block, 152 * 16);
  const double2* s = static_cast<const double2*>(src);
  double2* d = static_cast<double2*>(dst);
  switch (N) {
    case 3: invert_clover_kernel<3><<<grid, block, 0, st>>>(s, d, vh, flag); break;
    case 4: invert_clover_kernel<4><<<grid, block, 0, st>>>(s, d, vh, flag); break;
    case 5: invert_clover_kernel<5><<<grid, block, 0, st>>>(s, d, vh, flag); break;
    case 6: invert_clover_kernel<6><<<grid, block, 0, st>>>(s, d, vh, flag); break;
    case 7: invert_clover_kernel<7><<<grid, block, 0, st>>>(s, d, vh, flag); break;
    case 8: invert_clover_kernel<8><<<grid, block, 0, st>>>(s, d, vh, flag); break;
    default: throw Error(QCU_ERR_UNSUPPORTED, "clover: N must be 3..8");
  }
  QCU_CHECK_CUDA(cudaGetLastError());
  int h = 0;
  QCU_CHECK_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
  QCU_CHECK_CUDA(cudaStreamSynchronize(st));
  return h == 0;
}

void clover_apply(int prec, int N, const DslashArgs& A, const void* clover, cudaStream_t st) {
  switch (prec) {
    case PREC_DOUBLE: launch_clover_n<PREC_DOUBLE>(N, A, clover, st); break;
    case PREC_SINGLE: launch_clover_n<PREC_SINGLE>(N, A, clover, st); break;
    case PREC_HALF: launch_clover_n<PREC_HALF>(N, A, clover, st); break;
    case PREC_BF16: launch_clover_n<PREC_BF16>(N, A, clover, st); break;
    case PREC_BF16S: throw Error(QCU_ERR_UNSUPPORTED, "clover: site-major BF16 fields are not supported");
    default: throw Error(QCU_ERR_UNSUPPORTED, "bad precision");
  }
}

}  // namespace qcu
