// BLAS-1 kernels over MRHS fields (see blas.h).
//
// Thread mapping: thread k handles R consecutive complex elements (one
// 128-bit vector for FP64 R=1 / FP32 R=2) and strides over the field with a
// stride that is a multiple of nrhs, so every thread stays on the same R RHS
// and keeps private FP64 partial sums.  Block reduction: per RHS, one warp
// sums the block's partials with shuffles; a second kernel adds the
// per-block results in block order.  No atomics, so results are bitwise
// reproducible for a given launch shape.
#include <algorithm>

#include "blas.h"

// arithmetic helper for the complex reduction value type
__device__ __forceinline__ double2 operator+(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

namespace qcu {
namespace {

__device__ __forceinline__ double shfl_xor(double v, int off) { return __shfl_xor_sync(0xffffffffu, v, off); }
__device__ __forceinline__ double2 shfl_xor(double2 v, int off) {
  return make_double2(__shfl_xor_sync(0xffffffffu, v.x, off), __shfl_xor_sync(0xffffffffu, v.y, off));
}

constexpr int kMaxBlocks = 1024;

template <typename T> struct V2;
template <> struct V2<double> { using t = double2; };
template <> struct V2<float> { using t = float2; };

template <int P> struct BT;
template <> struct BT<PREC_DOUBLE> { using real = double; };
template <> struct BT<PREC_SINGLE> { using real = float; };

struct Shape {
  int64_t nchunks;  // n / R
  int R;
  int G;            // nrhs / R
  int nrhs;
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 tof(double2 a) { return make_float2((float)a.x, (float)a.y); }

template <typename E>
__device__ __forceinline__ double2 ld(const E* p) {
  E v = *p;
  return make_double2((double)v.x, (double)v.y);
}
template <typename E>
__device__ __forceinline__ void st(E* p, double2 v) {
  E e;
  e.x = v.x;
  e.y = v.y;
  *p = e;
}

// block-level per-RHS reduction of `vals` (R values per thread) into
// out[blockIdx.x * nrhs + r]
template <typename A>
__device__ void block_reduce(A* sm, const A* vals, int R, int G, int nrhs, A* out) {
  const int t = threadIdx.x, B = blockDim.x;
  for (int i = 0; i < R; i++) sm[t * R + i] = vals[i];
  __syncthreads();
  const int lane = t & 31, warp = t >> 5, nw = B >> 5;
  const int per = B / G;
  for (int r = warp; r < nrhs; r += nw) {
    const int g = r / R, i = r % R;
    A s;
    s = A{};
    for (int m = lane; m < per; m += 32) {
      const A v = sm[(g + m * G) * R + i];
      s = s + v;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s = s + shfl_xor(s, off);
    if (lane == 0) out[(int64_t)blockIdx.x * nrhs + r] = s;
  }
}


// ---------------------------------------------------------------------------
template <int PX, int PY, int R, bool NORM>
__global__ void axpby_kernel(const double2* __restrict__ a, const void* __restrict__ xv, const double2* __restrict__ b,
                             void* __restrict__ yv, Shape s, double* partials) {
  using EX = typename V2<typename BT<PX>::real>::t;
  using EY = typename V2<typename BT<PY>::real>::t;
  const EX* x = static_cast<const EX*>(xv);
  EY* y = static_cast<EY*>(yv);
  const int g = threadIdx.x % s.G;
  double2 ca[R], cb[R];
  double acc[R];
#pragma unroll
  for (int i = 0; i < R; i++) {
    ca[i] = a ? a[g * R + i] : make_double2(1.0, 0.0);
    cb[i] = b ? b[g * R + i] : make_double2(1.0, 0.0);
    acc[i] = 0.0;
  }
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  if constexpr (PX == PREC_SINGLE && PY == PREC_SINGLE) {
    // FP32 fields: FP32 arithmetic (the FP64 pipe of this GPU is a small
    // fraction of the FP32 one); the norm's per-thread sum stays FP64
    float2 fa[R], fb[R];
#pragma unroll
    for (int i = 0; i < R; i++) {
      fa[i] = tof(ca[i]);
      fb[i] = tof(cb[i]);
    }
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < s.nchunks; c += stride) {
      float2 xs[R], ys[R];
      if constexpr (R == 2) {  // one 16-byte vector per operand (chunks are 16-byte aligned)
        const float4 xq = reinterpret_cast<const float4*>(x)[c], yq = reinterpret_cast<const float4*>(y)[c];
        xs[0] = make_float2(xq.x, xq.y);
        xs[1] = make_float2(xq.z, xq.w);
        ys[0] = make_float2(yq.x, yq.y);
        ys[1] = make_float2(yq.z, yq.w);
      } else {
#pragma unroll
        for (int i = 0; i < R; i++) {
          xs[i] = x[c * R + i];
          ys[i] = y[c * R + i];
        }
      }
      float2 v[R];
#pragma unroll
      for (int i = 0; i < R; i++) {
        const float2 u = cmulf(fa[i], xs[i]), w = cmulf(fb[i], ys[i]);
        v[i] = make_float2(u.x + w.x, u.y + w.y);
        if (NORM) acc[i] += (double)fmaf(v[i].x, v[i].x, v[i].y * v[i].y);
      }
      if constexpr (R == 2) {
        reinterpret_cast<float4*>(y)[c] = make_float4(v[0].x, v[0].y, v[1].x, v[1].y);
      } else {
#pragma unroll
        for (int i = 0; i < R; i++) y[c * R + i] = v[i];
      }
    }
  } else if (b == nullptr) {
    // b = 1: no multiply of y (FP64 arithmetic is bound by the FP64 pipe here)
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < s.nchunks; c += stride) {
#pragma unroll
      for (int i = 0; i < R; i++) {
        const int64_t e = c * R + i;
        const double2 v = cmul(ca[i], ld(x + e)) + ld(y + e);
        st(y + e, v);
        if (NORM) acc[i] += v.x * v.x + v.y * v.y;
      }
    }
  } else {
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < s.nchunks; c += stride) {
#pragma unroll
      for (int i = 0; i < R; i++) {
        const int64_t e = c * R + i;
        const double2 v = cmul(ca[i], ld(x + e)) + cmul(cb[i], ld(y + e));
        st(y + e, v);
        if (NORM) acc[i] += v.x * v.x + v.y * v.y;
      }
    }
  }
  if (NORM) {
    __shared__ double sm[1024 * 2];
    block_reduce<double>(sm, acc, R, s.G, s.nrhs, partials);
  }
}

template <int P, int R>
__global__ void axpbypcz_kernel(const double2* __restrict__ a, const void* __restrict__ xv,
                                const double2* __restrict__ b, const void* __restrict__ yv,
                                const double2* __restrict__ c, void* __restrict__ zv, Shape s) {
  using E = typename V2<typename BT<P>::real>::t;
  const E* x = static_cast<const E*>(xv);
  const E* y = static_cast<const E*>(yv);
  E* z = static_cast<E*>(zv);
  const int g = threadIdx.x % s.G;
  double2 ca[R], cb[R], cc[R];
#pragma unroll
  for (int i = 0; i < R; i++) {
    ca[i] = a[g * R + i];
    cb[i] = b[g * R + i];
    cc[i] = c ? c[g * R + i] : make_double2(1.0, 0.0);
  }
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  if constexpr (P == PREC_SINGLE) {  // FP32 fields: FP32 arithmetic
    float2 fa[R], fb[R], fc[R];
#pragma unroll
    for (int i = 0; i < R; i++) {
      fa[i] = tof(ca[i]);
      fb[i] = tof(cb[i]);
      fc[i] = tof(cc[i]);
    }
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < s.nchunks; k += stride) {
      float2 xs[R], ys[R], zs[R];
      if constexpr (R == 2) {
        const float4 xq = reinterpret_cast<const float4*>(x)[k], yq = reinterpret_cast<const float4*>(y)[k],
                     zq = reinterpret_cast<const float4*>(z)[k];
        xs[0] = make_float2(xq.x, xq.y);
        xs[1] = make_float2(xq.z, xq.w);
        ys[0] = make_float2(yq.x, yq.y);
        ys[1] = make_float2(yq.z, yq.w);
        zs[0] = make_float2(zq.x, zq.y);
        zs[1] = make_float2(zq.z, zq.w);
      } else {
#pragma unroll
        for (int i = 0; i < R; i++) {
          xs[i] = x[k * R + i];
          ys[i] = y[k * R + i];
          zs[i] = z[k * R + i];
        }
      }
      float2 o[R];
#pragma unroll
      for (int i = 0; i < R; i++) {
        const float2 u = cmulf(fa[i], xs[i]), v = cmulf(fb[i], ys[i]), w = cmulf(fc[i], zs[i]);
        o[i] = make_float2(u.x + v.x + w.x, u.y + v.y + w.y);
      }
      if constexpr (R == 2) {
        reinterpret_cast<float4*>(z)[k] = make_float4(o[0].x, o[0].y, o[1].x, o[1].y);
      } else {
#pragma unroll
        for (int i = 0; i < R; i++) z[k * R + i] = o[i];
      }
    }
  } else {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < s.nchunks; k += stride) {
#pragma unroll
      for (int i = 0; i < R; i++) {
        const int64_t e = k * R + i;
        st(z + e, cmul(ca[i], ld(x + e)) + cmul(cb[i], ld(y + e)) + cmul(cc[i], ld(z + e)));
      }
    }
  }
}

// MODE 0: |x|^2, 1: <x, y>.  FAST (FP32 fields): the products in FP32, summed
// in FP64; otherwise every product is formed in FP64 (exact for FP32 inputs).
template <int PX, int PY, int R, int MODE, bool FAST = false>
__global__ void reduce_kernel(const void* __restrict__ xv, const void* __restrict__ yv, Shape s, void* partials) {
  using EX = typename V2<typename BT<PX>::real>::t;
  using EY = typename V2<typename BT<PY>::real>::t;
  const EX* x = static_cast<const EX*>(xv);
  const EY* y = static_cast<const EY*>(yv);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  if (MODE == 0) {
    double acc[R];
#pragma unroll
    for (int i = 0; i < R; i++) acc[i] = 0.0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < s.nchunks; k += stride) {
#pragma unroll
      for (int i = 0; i < R; i++) {
        if constexpr (FAST) {
          const float2 v = reinterpret_cast<const float2*>(x)[k * R + i];
          acc[i] += (double)fmaf(v.x, v.x, v.y * v.y);
        } else {
          const double2 v = ld(x + k * R + i);
          acc[i] += v.x * v.x + v.y * v.y;
        }
      }
    }
    __shared__ double sm[1024 * 2];
    block_reduce<double>(sm, acc, R, s.G, s.nrhs, static_cast<double*>(partials));
  } else {
    double2 acc[R];
#pragma unroll
    for (int i = 0; i < R; i++) acc[i] = make_double2(0.0, 0.0);
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < s.nchunks; k += stride) {
#pragma unroll
      for (int i = 0; i < R; i++) {
        if constexpr (FAST) {
          const float2 u = reinterpret_cast<const float2*>(x)[k * R + i];
          const float2 v = reinterpret_cast<const float2*>(y)[k * R + i];
          acc[i].x += (double)fmaf(u.x, v.x, u.y * v.y);  // conj(u) v
          acc[i].y += (double)fmaf(u.x, v.y, -u.y * v.x);
        } else {
          const double2 u = ld(x + k * R + i), v = ld(y + k * R + i);
          acc[i].x += u.x * v.x + u.y * v.y;  // conj(u) v
          acc[i].y += u.x * v.y - u.y * v.x;
        }
      }
    }
    __shared__ double2 sm2[1024 * 2];
    block_reduce<double2>(sm2, acc, R, s.G, s.nrhs, static_cast<double2*>(partials));
  }
}

// one warp per RHS: lane l sums the block partials l, l + 32, ... in order,
// then a fixed shuffle tree adds the lanes (deterministic)
template <typename A>
__global__ void finalize_kernel(const A* __restrict__ partials, int nblocks, int nrhs, A* out) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (r >= nrhs) return;  // whole warps leave together
  A s = A{};
  for (int b = lane; b < nblocks; b += 32) s = s + partials[(int64_t)b * nrhs + r];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s = s + shfl_xor(s, off);
  if (lane == 0) out[r] = s;
}

// launch of finalize_kernel: 4 RHS (warps) per block
template <typename A>
void finalize(const A* partials, int nblocks, int nrhs, A* out, cudaStream_t st) {
  finalize_kernel<A><<<(nrhs + 3) / 4, 128, 0, st>>>(partials, nblocks, nrhs, out);
}

template <int PX, int PY>
__global__ void add_copy_kernel(const void* __restrict__ xv, void* __restrict__ yv, int64_t n, int add) {
  using EX = typename V2<typename BT<PX>::real>::t;
  using EY = typename V2<typename BT<PY>::real>::t;
  const EX* x = static_cast<const EX*>(xv);
  EY* y = static_cast<EY*>(yv);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
    double2 v = ld(x + e);
    if (add) v = v + ld(y + e);
    st(y + e, v);
  }
}

Shape make_shape(const FieldRef& f, int R) {
  Shape s;
  s.R = R;
  s.nrhs = f.nrhs;
  s.G = f.nrhs / R;
  s.nchunks = f.n / R;
  return s;
}

// two complex FP32 elements (one 16-byte vector) per thread when nrhs is even
// and every operand is 16-byte aligned
int pick_r(const FieldRef& f, const void* other = nullptr, const void* third = nullptr) {
  const uintptr_t al = (uintptr_t)f.data | (uintptr_t)other | (uintptr_t)third;
  return (f.prec == PREC_SINGLE && f.nrhs % 2 == 0 && al % 16 == 0) ? 2 : 1;
}

// block size: a multiple of both G (so the RHS of a thread is fixed) and 32
int block_size(int G) {
  int b = G;
  while (b % 32) b += G;
  while (b < 128 && b * 2 <= 1024) b *= 2;
  return b;
}

int grid_for(int64_t nchunks, int block) {
  int64_t g = (nchunks + block - 1) / block;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, kMaxBlocks));
}

void check_field(const FieldRef& f) {
  QCU_REQUIRE(f.prec == PREC_DOUBLE || f.prec == PREC_SINGLE, QCU_ERR_UNSUPPORTED,
              "BLAS operands must be FP64 or FP32 fields");
  QCU_REQUIRE(f.nrhs >= 1 && f.n % f.nrhs == 0, QCU_ERR_INVALID_ARGUMENT, "bad field shape");
}

}  // namespace

int Blas::blocks_for(int64_t n) { return kMaxBlocks; }

void Blas::axpby(const double2* a, const FieldRef& x, const double2* b, const FieldRef& y, cudaStream_t st) {
  check_field(x);
  check_field(y);
  QCU_REQUIRE(x.n == y.n && x.nrhs == y.nrhs, QCU_ERR_INVALID_ARGUMENT, "axpby: shape mismatch");
  const int R = (x.prec == y.prec) ? pick_r(x, y.data) : 1;
  Shape s = make_shape(x, R);
  const int B = block_size(s.G);
  QCU_REQUIRE(B <= 1024, QCU_ERR_UNSUPPORTED, "nrhs too large for BLAS block");
  const int grid = grid_for(s.nchunks, B);
  if (x.prec == PREC_DOUBLE && y.prec == PREC_DOUBLE)
    axpby_kernel<PREC_DOUBLE, PREC_DOUBLE, 1, false><<<grid, B, 0, st>>>(a, x.data, b, y.data, s, nullptr);
  else if (x.prec == PREC_SINGLE && y.prec == PREC_SINGLE && R == 2)
    axpby_kernel<PREC_SINGLE, PREC_SINGLE, 2, false><<<grid, B, 0, st>>>(a, x.data, b, y.data, s, nullptr);
  else if (x.prec == PREC_SINGLE && y.prec == PREC_SINGLE)
    axpby_kernel<PREC_SINGLE, PREC_SINGLE, 1, false><<<grid, B, 0, st>>>(a, x.data, b, y.data, s, nullptr);
  else if (x.prec == PREC_SINGLE && y.prec == PREC_DOUBLE)
    axpby_kernel<PREC_SINGLE, PREC_DOUBLE, 1, false><<<grid, B, 0, st>>>(a, x.data, b, y.data, s, nullptr);
  else
    axpby_kernel<PREC_DOUBLE, PREC_SINGLE, 1, false><<<grid, B, 0, st>>>(a, x.data, b, y.data, s, nullptr);
  QCU_CHECK_CUDA(cudaGetLastError());
}

void Blas::axpby_norm(const double2* a, const FieldRef& x, const double2* b, const FieldRef& y, double* out,
                      cudaStream_t st) {
  check_field(x);
  check_field(y);
  QCU_REQUIRE(x.n == y.n && x.nrhs == y.nrhs && x.prec == y.prec, QCU_ERR_INVALID_ARGUMENT,
              "axpby_norm: shape/precision mismatch");
  const int R = pick_r(x, y.data);
  Shape s = make_shape(x, R);
  const int B = block_size(s.G);
  QCU_REQUIRE(B <= 1024, QCU_ERR_UNSUPPORTED, "nrhs too large for BLAS block");
  const int grid = grid_for(s.nchunks, B);
  QCU_REQUIRE(grid <= max_blocks_, QCU_ERR_INVALID_ARGUMENT, "partials too small");
  if (x.prec == PREC_DOUBLE)
    axpby_kernel<PREC_DOUBLE, PREC_DOUBLE, 1, true><<<grid, B, 0, st>>>(a, x.data, b, y.data, s, partials_);
  else if (R == 2)
    axpby_kernel<PREC_SINGLE, PREC_SINGLE, 2, true><<<grid, B, 0, st>>>(a, x.data, b, y.data, s, partials_);
  else
    axpby_kernel<PREC_SINGLE, PREC_SINGLE, 1, true><<<grid, B, 0, st>>>(a, x.data, b, y.data, s, partials_);
  QCU_CHECK_CUDA(cudaGetLastError());
  finalize<double>(partials_, grid, x.nrhs, out, st);
  QCU_CHECK_CUDA(cudaGetLastError());
}

void Blas::axpbypcz(const double2* a, const FieldRef& x, const double2* b, const FieldRef& y, const double2* c,
                    const FieldRef& z, cudaStream_t st) {
  check_field(x);
  QCU_REQUIRE(x.prec == y.prec && y.prec == z.prec && x.n == y.n && y.n == z.n, QCU_ERR_INVALID_ARGUMENT,
              "axpbypcz: shape/precision mismatch");
  const int R = pick_r(x, y.data, z.data);
  Shape s = make_shape(x, R);
  const int B = block_size(s.G);
  QCU_REQUIRE(B <= 1024, QCU_ERR_UNSUPPORTED, "nrhs too large for BLAS block");
  const int grid = grid_for(s.nchunks, B);
  if (x.prec == PREC_DOUBLE)
    axpbypcz_kernel<PREC_DOUBLE, 1><<<grid, B, 0, st>>>(a, x.data, b, y.data, c, z.data, s);
  else if (R == 2)
    axpbypcz_kernel<PREC_SINGLE, 2><<<grid, B, 0, st>>>(a, x.data, b, y.data, c, z.data, s);
  else
    axpbypcz_kernel<PREC_SINGLE, 1><<<grid, B, 0, st>>>(a, x.data, b, y.data, c, z.data, s);
  QCU_CHECK_CUDA(cudaGetLastError());
}

void Blas::norm2(const FieldRef& x, double* out, cudaStream_t st, bool exact) {
  check_field(x);
  const int R = pick_r(x);
  Shape s = make_shape(x, R);
  const int B = block_size(s.G);
  QCU_REQUIRE(B <= 1024, QCU_ERR_UNSUPPORTED, "nrhs too large for BLAS block");
  const int grid = grid_for(s.nchunks, B);
  if (x.prec == PREC_DOUBLE)
    reduce_kernel<PREC_DOUBLE, PREC_DOUBLE, 1, 0><<<grid, B, 0, st>>>(x.data, x.data, s, partials_);
  else if (R == 2 && exact)
    reduce_kernel<PREC_SINGLE, PREC_SINGLE, 2, 0><<<grid, B, 0, st>>>(x.data, x.data, s, partials_);
  else if (R == 2)
    reduce_kernel<PREC_SINGLE, PREC_SINGLE, 2, 0, true><<<grid, B, 0, st>>>(x.data, x.data, s, partials_);
  else if (exact)
    reduce_kernel<PREC_SINGLE, PREC_SINGLE, 1, 0><<<grid, B, 0, st>>>(x.data, x.data, s, partials_);
  else
    reduce_kernel<PREC_SINGLE, PREC_SINGLE, 1, 0, true><<<grid, B, 0, st>>>(x.data, x.data, s, partials_);
  QCU_CHECK_CUDA(cudaGetLastError());
  finalize<double>(partials_, grid, x.nrhs, out, st);
  QCU_CHECK_CUDA(cudaGetLastError());
}

void Blas::cdot(const FieldRef& x, const FieldRef& y, double2* out, cudaStream_t st) {
  check_field(x);
  check_field(y);
  QCU_REQUIRE(x.n == y.n && x.nrhs == y.nrhs && x.prec == y.prec, QCU_ERR_INVALID_ARGUMENT,
              "cdot: shape/precision mismatch");
  const int R = pick_r(x);
  Shape s = make_shape(x, R);
  const int B = block_size(s.G);
  QCU_REQUIRE(B <= 1024, QCU_ERR_UNSUPPORTED, "nrhs too large for BLAS block");
  const int grid = grid_for(s.nchunks, B);
  QCU_REQUIRE(2 * grid <= max_blocks_ * 2, QCU_ERR_INVALID_ARGUMENT, "partials too small");
  double2* p2 = reinterpret_cast<double2*>(partials_);
  if (x.prec == PREC_DOUBLE)
    reduce_kernel<PREC_DOUBLE, PREC_DOUBLE, 1, 1><<<grid, B, 0, st>>>(x.data, y.data, s, p2);
  else if (R == 2)
    reduce_kernel<PREC_SINGLE, PREC_SINGLE, 2, 1, true><<<grid, B, 0, st>>>(x.data, y.data, s, p2);
  else
    reduce_kernel<PREC_SINGLE, PREC_SINGLE, 1, 1, true><<<grid, B, 0, st>>>(x.data, y.data, s, p2);
  QCU_CHECK_CUDA(cudaGetLastError());
  finalize<double2>(p2, grid, x.nrhs, out, st);
  QCU_CHECK_CUDA(cudaGetLastError());
}

void Blas::add_to(const FieldRef& lo, const FieldRef& hi, cudaStream_t st) {
  check_field(lo);
  check_field(hi);
  QCU_REQUIRE(lo.n == hi.n, QCU_ERR_INVALID_ARGUMENT, "add_to: shape mismatch");
  const int grid = grid_for(lo.n, 256);
  if (lo.prec == PREC_SINGLE && hi.prec == PREC_DOUBLE)
    add_copy_kernel<PREC_SINGLE, PREC_DOUBLE><<<grid, 256, 0, st>>>(lo.data, hi.data, lo.n, 1);
  else if (lo.prec == PREC_DOUBLE && hi.prec == PREC_DOUBLE)
    add_copy_kernel<PREC_DOUBLE, PREC_DOUBLE><<<grid, 256, 0, st>>>(lo.data, hi.data, lo.n, 1);
  else if (lo.prec == PREC_SINGLE && hi.prec == PREC_SINGLE)
    add_copy_kernel<PREC_SINGLE, PREC_SINGLE><<<grid, 256, 0, st>>>(lo.data, hi.data, lo.n, 1);
  else
    add_copy_kernel<PREC_DOUBLE, PREC_SINGLE><<<grid, 256, 0, st>>>(lo.data, hi.data, lo.n, 1);
  QCU_CHECK_CUDA(cudaGetLastError());
}

void Blas::copy(const FieldRef& x, const FieldRef& y, cudaStream_t st) {
  check_field(x);
  check_field(y);
  QCU_REQUIRE(x.n == y.n, QCU_ERR_INVALID_ARGUMENT, "copy: shape mismatch");
  const int grid = grid_for(x.n, 256);
  if (x.prec == PREC_SINGLE && y.prec == PREC_DOUBLE)
    add_copy_kernel<PREC_SINGLE, PREC_DOUBLE><<<grid, 256, 0, st>>>(x.data, y.data, x.n, 0);
  else if (x.prec == PREC_DOUBLE && y.prec == PREC_DOUBLE)
    add_copy_kernel<PREC_DOUBLE, PREC_DOUBLE><<<grid, 256, 0, st>>>(x.data, y.data, x.n, 0);
  else if (x.prec == PREC_SINGLE && y.prec == PREC_SINGLE)
    add_copy_kernel<PREC_SINGLE, PREC_SINGLE><<<grid, 256, 0, st>>>(x.data, y.data, x.n, 0);
  else
    add_copy_kernel<PREC_DOUBLE, PREC_SINGLE><<<grid, 256, 0, st>>>(x.data, y.data, x.n, 0);
  QCU_CHECK_CUDA(cudaGetLastError());
}

void Blas::zero(const FieldRef& x, cudaStream_t st) {
  QCU_CHECK_CUDA(cudaMemsetAsync(x.data, 0, (size_t)x.n * prec_complex_bytes(x.prec), st));
}

}  // namespace qcu
