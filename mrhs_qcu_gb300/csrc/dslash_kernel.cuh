// Multi-right-hand-side even-odd Wilson hopping term on CUDA cores.
//
//   out(x) = a * sum_mu [ (1 - f g_mu) U_mu(x) in(x+mu)
//                        + (1 + f g_mu) U_mu(x-mu)^dag in(x-mu) ] * bc + b * xin(x)
//
// for x on the output parity and every RHS of an MRHS field.  This is the
// operator of the reference's dslashKernel/applyWilson
// (include/kernels/wilson_dslash_4d.cuh:25-322): same gamma basis, same
// f = +1 / -1 dagger flag (src/qcd/qcu_wilson.cu:41), same even-odd
// neighbour rule (include/basic_data/qcu_point.cuh:33-78).  Added here:
// antiperiodic time boundaries (bc = -1 on hops across t = Lt-1 <-> 0), the
// optional a/b "xpay" epilogue (the reference's DslashXpay stub,
// include/qcu_dirac.h:49), 16-bit storage with per-(site, RHS) scales, and
// a per-RHS activity mask.
//
// Work decomposition: one thread = one output site x R right-hand sides.  The
// G = nrhs / R threads of a site read the same link words (one coalesced
// transaction serves the warp); each link is used for all R RHS of the thread,
// and the neighbour spinors are read as 128-bit vectors (R RHS contiguous).
// Spin projection to two half-spinor rows happens before the SU(N)
// multiply; reconstruction folds the projector and boundary signs into FMA
// coefficients.
#pragma once

#include "qcu_common.cuh"

namespace qcu {

struct DslashArgs {
  const void* gauge;     // [4][2][N*N][Vh] complex<P>
  const void* in;        // MRHS field, parity 1 - parity
  const float* in_norm;  // [Vh][nrhs] (16-bit storage only)
  void* out;             // MRHS field, output parity
  float* out_norm;
  const void* x;         // xpay input (output parity) or nullptr
  const float* x_norm;
  const int* mask;       // [nrhs] 0 = skip RHS, nullptr = all active
  double a, b;           // out = a * D in + b * x
  Geometry geo;
  int nrhs;
  int parity;            // output parity
  int dagger;            // 0: f = +1, 1: f = -1
  int antiperiodic_t;
  FastDiv div_groups;    // G = nrhs / R
};

namespace detail {

// gamma_mu row r: single non-zero in column perm, value sign * (imag ? i : 1)
// (DeGrand-Rossi basis of the reference, wilson_dslash_4d.cuh:74-81,
// 134-141, 193-200, 253-260)
__host__ __device__ constexpr int gperm(int mu, int r) { return mu < 2 ? 3 - r : (r ^ 2); }
__host__ __device__ constexpr bool gimag(int mu) { return mu == 0 || mu == 2; }
__host__ __device__ constexpr int gsign(int mu, int r) {
  return mu == 0 ? (r < 2 ? 1 : -1)
                 : mu == 1 ? ((r == 0 || r == 3) ? -1 : 1)
                           : mu == 2 ? ((r == 0 || r == 3) ? 1 : -1) : 1;
}

template <typename T>
struct C2 {
  T x, y;
};

// Vector load/store of R consecutive storage elements (R RHS of one
// component).  The offset is a multiple of R, so the widest vector whose size
// divides R * sizeof(E) is aligned.
template <typename E, int R>
struct Vec {
  static constexpr int bytes = R * (int)sizeof(E);
  static constexpr int vbytes = (bytes % 16 == 0) ? 16 : (bytes % 8 == 0) ? 8 : 4;
  static constexpr int nv = bytes / vbytes;
  __device__ __forceinline__ static void load(const E* p, E (&v)[R]) {
    if constexpr (vbytes == 16) {
      const uint4* q = reinterpret_cast<const uint4*>(p);
      uint4* d = reinterpret_cast<uint4*>(v);
#pragma unroll
      for (int i = 0; i < nv; i++) d[i] = __ldg(q + i);
    } else if constexpr (vbytes == 8) {
      const uint2* q = reinterpret_cast<const uint2*>(p);
      uint2* d = reinterpret_cast<uint2*>(v);
#pragma unroll
      for (int i = 0; i < nv; i++) d[i] = __ldg(q + i);
    } else {
      const unsigned* q = reinterpret_cast<const unsigned*>(p);
      unsigned* d = reinterpret_cast<unsigned*>(v);
#pragma unroll
      for (int i = 0; i < nv; i++) d[i] = __ldg(q + i);
    }
  }
  __device__ __forceinline__ static void store(E* p, const E (&v)[R]) {
    if constexpr (vbytes == 16) {
      uint4* q = reinterpret_cast<uint4*>(p);
      const uint4* s = reinterpret_cast<const uint4*>(v);
#pragma unroll
      for (int i = 0; i < nv; i++) q[i] = s[i];
    } else if constexpr (vbytes == 8) {
      uint2* q = reinterpret_cast<uint2*>(p);
      const uint2* s = reinterpret_cast<const uint2*>(v);
#pragma unroll
      for (int i = 0; i < nv; i++) q[i] = s[i];
    } else {
      unsigned* q = reinterpret_cast<unsigned*>(p);
      const unsigned* s = reinterpret_cast<const unsigned*>(v);
#pragma unroll
      for (int i = 0; i < nv; i++) q[i] = s[i];
    }
  }
};

template <typename E, int R>
struct alignas(Vec<E, R>::vbytes) VecBuf {
  E v[R];
};

template <int P, int R>
__device__ __forceinline__ void load_norms(const float* p, float (&nrm)[R]) {
  if constexpr (R % 4 == 0) {
#pragma unroll
    for (int i = 0; i < R / 4; i++) {
      float4 q = __ldg(reinterpret_cast<const float4*>(p) + i);
      nrm[4 * i] = q.x;
      nrm[4 * i + 1] = q.y;
      nrm[4 * i + 2] = q.z;
      nrm[4 * i + 3] = q.w;
    }
  } else if constexpr (R % 2 == 0) {
#pragma unroll
    for (int i = 0; i < R / 2; i++) {
      float2 q = __ldg(reinterpret_cast<const float2*>(p) + i);
      nrm[2 * i] = q.x;
      nrm[2 * i + 1] = q.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < R; i++) nrm[i] = __ldg(p + i);
  }
}

// One hop (direction MU, forward or backward) accumulated into acc.
//   s = -f (forward, projector 1 - f g) or +f (backward, 1 + f g)
//   kup  = bc * scale_r        multiplies the two upper rows
//   klo  = s * sign(lo) * bc * scale_r   the reconstructed lower rows
template <int P, int N, int R, int MU, bool FWD>
__device__ __forceinline__ void hop(C2<typename Store<P>::real> (&acc)[4][N][R], const DslashArgs& A,
                                   const typename Store<P>::elem* __restrict__ in,
                                   const typename Store<P>::elem* __restrict__ gauge, int64_t link_base,
                                   int64_t nb, int rhs0, typename Store<P>::real bc,
                                   typename Store<P>::real f) {
  using S = Store<P>;
  using T = typename S::real;
  using E = typename S::elem;
  constexpr int u0p = gperm(MU, 0), u1p = gperm(MU, 1);
  constexpr bool im = gimag(MU);
  const T s = FWD ? -f : f;
  const int64_t vh = A.geo.vh;
  const int nrhs = A.nrhs;

  T scale[R];
  if constexpr (S::has_norm) {
    float nr[R];
    load_norms<P, R>(A.in_norm + nb * nrhs + rhs0, nr);
#pragma unroll
    for (int r = 0; r < R; r++) scale[r] = bc * nr[r];
  } else {
#pragma unroll
    for (int r = 0; r < R; r++) scale[r] = bc;
  }

  // project: h_u = psi_u + s g(u) psi_perm(u), u = 0, 1
  C2<T> h[2][N][R];
  // component-major field: component c of site nb at (c * Vh + nb) * nrhs
  const int64_t cs = vh * nrhs;
  const E* base = in + nb * nrhs + rhs0;
#pragma unroll
  for (int a = 0; a < N; a++) {
    VecBuf<E, R> p0, p1, q0, q1;
    Vec<E, R>::load(base + (0 * N + a) * cs, p0.v);
    Vec<E, R>::load(base + (1 * N + a) * cs, p1.v);
    Vec<E, R>::load(base + (u0p * N + a) * cs, q0.v);
    Vec<E, R>::load(base + (u1p * N + a) * cs, q1.v);
    const T k0 = s * (T)gsign(MU, 0), k1 = s * (T)gsign(MU, 1);
#pragma unroll
    for (int r = 0; r < R; r++) {
      auto x0 = S::to_c(p0.v[r]);
      auto x1 = S::to_c(p1.v[r]);
      auto y0 = S::to_c(q0.v[r]);
      auto y1 = S::to_c(q1.v[r]);
      if constexpr (im) {
        h[0][a][r].x = fma(-k0, (T)y0.y, (T)x0.x);
        h[0][a][r].y = fma(k0, (T)y0.x, (T)x0.y);
        h[1][a][r].x = fma(-k1, (T)y1.y, (T)x1.x);
        h[1][a][r].y = fma(k1, (T)y1.x, (T)x1.y);
      } else {
        h[0][a][r].x = fma(k0, (T)y0.x, (T)x0.x);
        h[0][a][r].y = fma(k0, (T)y0.y, (T)x0.y);
        h[1][a][r].x = fma(k1, (T)y1.x, (T)x1.x);
        h[1][a][r].y = fma(k1, (T)y1.y, (T)x1.y);
      }
    }
  }

  // colour multiply row by row, then reconstruct
  const T klo0 = s * (T)gsign(MU, u0p), klo1 = s * (T)gsign(MU, u1p);
#pragma unroll
  for (int a = 0; a < N; a++) {
    C2<T> t[2][R];
#pragma unroll
    for (int u = 0; u < 2; u++)
#pragma unroll
      for (int r = 0; r < R; r++) t[u][r].x = t[u][r].y = (T)0;
#pragma unroll
    for (int b = 0; b < N; b++) {
      // forward uses U[a][b]; backward uses conj(U[b][a])
      const int comp = FWD ? (a * N + b) : (b * N + a);
      auto uc = S::to_c(__ldg(gauge + link_base + (int64_t)comp * vh));
      const T ur = (T)uc.x;
      const T ui = FWD ? (T)uc.y : -(T)uc.y;
#pragma unroll
      for (int u = 0; u < 2; u++)
#pragma unroll
        for (int r = 0; r < R; r++) {
          t[u][r].x = fma(ur, h[u][b][r].x, t[u][r].x);
          t[u][r].x = fma(-ui, h[u][b][r].y, t[u][r].x);
          t[u][r].y = fma(ur, h[u][b][r].y, t[u][r].y);
          t[u][r].y = fma(ui, h[u][b][r].x, t[u][r].y);
        }
    }
#pragma unroll
    for (int r = 0; r < R; r++) {
      const T ku = scale[r];
      const T kl0 = klo0 * scale[r], kl1 = klo1 * scale[r];
      acc[0][a][r].x = fma(ku, t[0][r].x, acc[0][a][r].x);
      acc[0][a][r].y = fma(ku, t[0][r].y, acc[0][a][r].y);
      acc[1][a][r].x = fma(ku, t[1][r].x, acc[1][a][r].x);
      acc[1][a][r].y = fma(ku, t[1][r].y, acc[1][a][r].y);
      if constexpr (im) {
        acc[u0p][a][r].x = fma(-kl0, t[0][r].y, acc[u0p][a][r].x);
        acc[u0p][a][r].y = fma(kl0, t[0][r].x, acc[u0p][a][r].y);
        acc[u1p][a][r].x = fma(-kl1, t[1][r].y, acc[u1p][a][r].x);
        acc[u1p][a][r].y = fma(kl1, t[1][r].x, acc[u1p][a][r].y);
      } else {
        acc[u0p][a][r].x = fma(kl0, t[0][r].x, acc[u0p][a][r].x);
        acc[u0p][a][r].y = fma(kl0, t[0][r].y, acc[u0p][a][r].y);
        acc[u1p][a][r].x = fma(kl1, t[1][r].x, acc[u1p][a][r].x);
        acc[u1p][a][r].y = fma(kl1, t[1][r].y, acc[u1p][a][r].y);
      }
    }
  }
}

}  // namespace detail

// MINB: minimum resident blocks of 256 threads per SM requested from the
// compiler, i.e. a register cap of 65536 / (256 * MINB) per thread (1: 255).
template <int P, int N, int R, int MINB>
__global__ void __launch_bounds__(256, MINB) wilson_mrhs_kernel(const DslashArgs A) {
  using S = Store<P>;
  using T = typename S::real;
  using E = typename S::elem;
  using namespace detail;

  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t site_u, grp;
  A.div_groups.divmod(gid, site_u, grp);
  if ((int)site_u >= A.geo.vh) return;
  const int rhs0 = (int)grp * R;
  if (A.mask) {
    bool any = false;
#pragma unroll
    for (int r = 0; r < R; r++) any |= A.mask[rhs0 + r] != 0;
    if (!any) return;
  }

  const int64_t site = site_u;
  uint32_t rest, xh, y, z, t;
  A.geo.div_hx.divmod(site_u, rest, xh);
  uint32_t rest2;
  A.geo.div_y.divmod(rest, rest2, y);
  A.geo.div_z.divmod(rest2, t, z);
  const int hx = A.geo.hx, Ly = A.geo.L[1], Lz = A.geo.L[2], Lt = A.geo.L[3];
  const int p = A.parity;
  const int eo = (int)((y + z + t) & 1);
  const T f = A.dagger ? (T)-1 : (T)1;
  const int64_t vh = A.geo.vh;
  const E* __restrict__ in = static_cast<const E*>(A.in);
  const E* __restrict__ gauge = static_cast<const E*>(A.gauge);
  constexpr int64_t NN = N * N;

  C2<T> acc[4][N][R];
#pragma unroll
  for (int sp = 0; sp < 4; sp++)
#pragma unroll
    for (int a = 0; a < N; a++)
#pragma unroll
      for (int r = 0; r < R; r++) acc[sp][a][r].x = acc[sp][a][r].y = (T)0;

  // link bases: forward links at (mu, p, site), backward at (mu, 1-p, nb)
  const int64_t lf = (int64_t)p * NN * vh + site;
  const int64_t lb = (int64_t)(1 - p) * NN * vh;
  {  // X
    const int64_t nf = (eo != p) ? ((int)xh == hx - 1 ? site - (hx - 1) : site + 1) : site;
    const int64_t nbk = (eo == p) ? (xh == 0 ? site + (hx - 1) : site - 1) : site;
    hop<P, N, R, 0, true>(acc, A, in, gauge, 0 * 2 * NN * vh + lf, nf, rhs0, (T)1, f);
    hop<P, N, R, 0, false>(acc, A, in, gauge, 0 * 2 * NN * vh + lb + nbk, nbk, rhs0, (T)1, f);
  }
  {  // Y
    const int64_t nf = ((int)y == Ly - 1) ? site - (int64_t)(Ly - 1) * hx : site + hx;
    const int64_t nbk = (y == 0) ? site + (int64_t)(Ly - 1) * hx : site - hx;
    hop<P, N, R, 1, true>(acc, A, in, gauge, 1 * 2 * NN * vh + lf, nf, rhs0, (T)1, f);
    hop<P, N, R, 1, false>(acc, A, in, gauge, 1 * 2 * NN * vh + lb + nbk, nbk, rhs0, (T)1, f);
  }
  {  // Z
    const int64_t pl = A.geo.plane;
    const int64_t nf = ((int)z == Lz - 1) ? site - (int64_t)(Lz - 1) * pl : site + pl;
    const int64_t nbk = (z == 0) ? site + (int64_t)(Lz - 1) * pl : site - pl;
    hop<P, N, R, 2, true>(acc, A, in, gauge, 2 * 2 * NN * vh + lf, nf, rhs0, (T)1, f);
    hop<P, N, R, 2, false>(acc, A, in, gauge, 2 * 2 * NN * vh + lb + nbk, nbk, rhs0, (T)1, f);
  }
  {  // T, with the optional antiperiodic sign
    const int64_t cb = A.geo.cube;
    const bool top = (int)t == Lt - 1, bot = t == 0;
    const int64_t nf = top ? site - (int64_t)(Lt - 1) * cb : site + cb;
    const int64_t nbk = bot ? site + (int64_t)(Lt - 1) * cb : site - cb;
    const T bcf = (A.antiperiodic_t && top) ? (T)-1 : (T)1;
    const T bcb = (A.antiperiodic_t && bot) ? (T)-1 : (T)1;
    hop<P, N, R, 3, true>(acc, A, in, gauge, 3 * 2 * NN * vh + lf, nf, rhs0, bcf, f);
    hop<P, N, R, 3, false>(acc, A, in, gauge, 3 * 2 * NN * vh + lb + nbk, nbk, rhs0, bcb, f);
  }

  // epilogue: out = a * acc + b * x
  const int nrhs = A.nrhs;
  const T ca = (T)A.a;
  const T cbx = (T)A.b;
  const E* __restrict__ xin = static_cast<const E*>(A.x);
  float xs[R];
  if constexpr (S::has_norm) {
    if (xin) load_norms<P, R>(A.x_norm + site * nrhs + rhs0, xs);
  }
#pragma unroll
  for (int sp = 0; sp < 4; sp++)
#pragma unroll
    for (int a = 0; a < N; a++) {
      const int64_t off = ((int64_t)(sp * N + a) * vh + site) * nrhs + rhs0;
      if (xin) {
        VecBuf<E, R> xv;
        Vec<E, R>::load(xin + off, xv.v);
#pragma unroll
        for (int r = 0; r < R; r++) {
          auto xc = S::to_c(xv.v[r]);
          T sx = cbx;
          if constexpr (S::has_norm) sx *= (T)xs[r];
          acc[sp][a][r].x = fma(sx, (T)xc.x, ca * acc[sp][a][r].x);
          acc[sp][a][r].y = fma(sx, (T)xc.y, ca * acc[sp][a][r].y);
        }
      } else {
#pragma unroll
        for (int r = 0; r < R; r++) {
          acc[sp][a][r].x *= ca;
          acc[sp][a][r].y *= ca;
        }
      }
    }

  E* __restrict__ out = static_cast<E*>(A.out);
  if constexpr (S::has_norm) {
    float inv[R];
    float mx[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      float m = 0.f;
#pragma unroll
      for (int sp = 0; sp < 4; sp++)
#pragma unroll
        for (int a = 0; a < N; a++) m = fmaxf(m, fmaxf(fabsf(acc[sp][a][r].x), fabsf(acc[sp][a][r].y)));
      mx[r] = m;
      inv[r] = m > 0.f ? 1.0f / m : 0.f;
    }
#pragma unroll
    for (int r = 0; r < R; r++) A.out_norm[site * nrhs + rhs0 + r] = mx[r];
#pragma unroll
    for (int sp = 0; sp < 4; sp++)
#pragma unroll
      for (int a = 0; a < N; a++) {
        VecBuf<E, R> ov;
#pragma unroll
        for (int r = 0; r < R; r++) {
          float2 v = make_float2(acc[sp][a][r].x * inv[r], acc[sp][a][r].y * inv[r]);
          ov.v[r] = S::from_c(v);
        }
        Vec<E, R>::store(out + ((int64_t)(sp * N + a) * vh + site) * nrhs + rhs0, ov.v);
      }
  } else {
#pragma unroll
    for (int sp = 0; sp < 4; sp++)
#pragma unroll
      for (int a = 0; a < N; a++) {
        VecBuf<E, R> ov;
#pragma unroll
        for (int r = 0; r < R; r++) {
          E e;
          e.x = acc[sp][a][r].x;
          e.y = acc[sp][a][r].y;
          ov.v[r] = e;
        }
        Vec<E, R>::store(out + ((int64_t)(sp * N + a) * vh + site) * nrhs + rhs0, ov.v);
      }
  }
}

// host-side launcher of one instantiation
template <int P, int N, int R, int MINB>
void launch_wilson_mrhs(const DslashArgs& A, int block, cudaStream_t stream) {
  const int groups = A.nrhs / R;
  const int64_t threads = (int64_t)A.geo.vh * groups;
  const int grid = (int)((threads + block - 1) / block);
  wilson_mrhs_kernel<P, N, R, MINB><<<grid, block, 0, stream>>>(A);
}

}  // namespace qcu
