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
  const void* gauge12 = nullptr;  // SU(3): [4][2][6][Vh], the first two rows (or nullptr)
  const void* gauge_tc = nullptr; // BF16 per-site link records (layout.h gauge_tc_records_bf16) for the tensor-core dslash, or nullptr
  const void* in;        // MRHS field, parity 1 - parity
  const float* in_norm;  // [Vh][nrhs] (16-bit storage only)
  void* out;             // MRHS field, output parity
  float* out_norm;
  const void* x;         // xpay input (output parity) or nullptr
  const float* x_norm;
  const int* mask;       // [nrhs] 0 = skip RHS, nullptr = all active
  double a, b;           // out = a * D in + b * x
  float af, bf;          // a, b rounded once on the host for the FP32 kernels
  const float* a_rhs_f;  // optional per-RHS a (replaces a) for FP32 arithmetic
  const double* a_rhs_d; // optional per-RHS a for FP64 arithmetic
  Geometry geo;
  int nrhs;
  int parity;            // output parity
  int dagger;            // 0: f = +1, 1: f = -1
  int antiperiodic_t;
  FastDiv div_groups;    // G = nrhs / R
  int site_major = 0;    // spinor fields in the site-major layout (PREC_BF16S; set by launch_dslash)
  // Site order of the register kernel (set by launch_dslash): slabs of zb
  // z-planes, t slowest within a slab, so that the reads of an input site
  // (as the x, y, z neighbour of its own slice and the t neighbour of the
  // slices on either side) fall within about three slab-slices instead of
  // three whole t-slices, and stay in L2.  zb = 0: the field's own order.
  uint32_t zb = 0;
  FastDiv div_plane, div_zb, div_lt;
  int stream_out = 0;  // output stores marked evict-first (the output is not re-read by the launch)
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

// complex register type of the compute precision: float2 or double2
template <typename T>
using C2 = typename cplx<T>::t;

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
  // the same from shared memory (plain loads)
  __device__ __forceinline__ static void load_shared(const E* p, E (&v)[R]) {
    if constexpr (vbytes == 16) {
      const uint4* q = reinterpret_cast<const uint4*>(p);
      uint4* d = reinterpret_cast<uint4*>(v);
#pragma unroll
      for (int i = 0; i < nv; i++) d[i] = q[i];
    } else if constexpr (vbytes == 8) {
      const uint2* q = reinterpret_cast<const uint2*>(p);
      uint2* d = reinterpret_cast<uint2*>(v);
#pragma unroll
      for (int i = 0; i < nv; i++) d[i] = q[i];
    } else {
      const unsigned* q = reinterpret_cast<const unsigned*>(p);
      unsigned* d = reinterpret_cast<unsigned*>(v);
#pragma unroll
      for (int i = 0; i < nv; i++) d[i] = q[i];
    }
  }
  __device__ __forceinline__ static void store(E* p, const E (&v)[R], bool cs = false) {
    if constexpr (vbytes == 16) {
      uint4* q = reinterpret_cast<uint4*>(p);
      const uint4* s = reinterpret_cast<const uint4*>(v);
#pragma unroll
      for (int i = 0; i < nv; i++) {
        if (cs)
          __stcs(q + i, s[i]);
        else
          q[i] = s[i];
      }
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

// One link component: a read-only global load, or a shared-memory load where
// the links were staged there (SMEM).
template <typename E, bool SMEM>
__device__ __forceinline__ E ld_link(const char* p) {
  if constexpr (SMEM)
    return *reinterpret_cast<const E*>(p);
  else
    return __ldg(reinterpret_cast<const E*>(p));
}

// Two-row SU(3) gauge layout: per (mu, parity) block, sites in groups of
// 32, the six components of a group one after another: component k of site s
// at (s / 32) * 192 + k * 32 + s % 32 (the half volume padded to a multiple of
// 32).  A warp's read of one component over 32 consecutive sites is one
// contiguous run (as in a component-major copy), and a site's eight links lie
// in eight 1.5 KB blocks (instead of 48 arrays).
__host__ __device__ constexpr uint32_t two_row_site(uint32_t s) { return (s >> 5) * 192u + (s & 31u); }
__host__ __device__ constexpr uint32_t two_row_vh(uint32_t vh) { return (vh + 31u) & ~31u; }

// SU(3) link from its first two rows: row 2 = conj(row 0 x row 1), each real
// part one multiply and three FMAs (the reference's two-row gauge read,
// include/kernels/storageLoadStore/loadAndStore.cuh:17-27, completed in
// registers).  Loads the six stored components at lbase + k * ls_bytes.
template <typename S, typename T, bool SMEM = false>
__device__ __forceinline__ void load_su3_two_row(const char* lbase, uint32_t ls_bytes, C2<T> (&u)[3][3]) {
  using E = typename S::elem;
#pragma unroll
  for (int k = 0; k < 6; k++) {
    const auto v = S::to_c(ld_link<E, SMEM>(lbase));
    u[k / 3][k % 3].x = (T)v.x;
    u[k / 3][k % 3].y = (T)v.y;
    lbase += ls_bytes;
  }
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const int k = (j + 1) % 3, l = (j + 2) % 3;
    T re = u[0][k].x * u[1][l].x;
    re = fma(-u[0][k].y, u[1][l].y, re);
    re = fma(-u[0][l].x, u[1][k].x, re);
    re = fma(u[0][l].y, u[1][k].y, re);
    T im = -(u[0][k].x * u[1][l].y);
    im = fma(-u[0][k].y, u[1][l].x, im);
    im = fma(u[0][l].x, u[1][k].y, im);
    im = fma(u[0][l].y, u[1][k].x, im);
    u[2][j].x = re;
    u[2][j].y = im;
  }
}

// One hop (direction MU, forward or backward) accumulated into acc.
//   s = -f (forward, projector 1 - f g) or +f (backward, 1 + f g)
//   kup  = bc * scale_r        multiplies the two upper rows
//   klo  = s * sign(lo) * bc * scale_r   the reconstructed lower rows
// Offsets are 32-bit element indices into the field / gauge arrays (the host
// checks that every array has fewer than 2^32 elements).
template <int P, int N, int R, int MU, bool FWD, bool RC = false>
__device__ __forceinline__ void hop(C2<typename Store<P>::real> (&acc)[4][N][R], const DslashArgs& A,
                                   const typename Store<P>::elem* __restrict__ in,
                                   const typename Store<P>::elem* __restrict__ gauge, uint32_t link_off,
                                   uint32_t nb, uint32_t rhs0, typename Store<P>::real bc,
                                   typename Store<P>::real f) {
  using S = Store<P>;
  using T = typename S::real;
  using E = typename S::elem;
  constexpr int u0p = gperm(MU, 0), u1p = gperm(MU, 1);
  constexpr bool im = gimag(MU);
  const T s = FWD ? -f : f;
  const uint32_t vh = (uint32_t)A.geo.vh;
  const uint32_t nrhs = (uint32_t)A.nrhs;

  T scale[R];
  if constexpr (S::has_norm) {
    float nr[R];
    load_norms<P, R>(A.in_norm + (nb * nrhs + rhs0), nr);
#pragma unroll
    for (int r = 0; r < R; r++) scale[r] = bc * nr[r];
  } else {
#pragma unroll
    for (int r = 0; r < R; r++) scale[r] = bc;
  }

  // project: h_u = psi_u + s g(u) psi_perm(u), u = 0, 1
  C2<T> h[2][N][R];
  // component-major field: component c of site nb at (c * Vh + nb) * nrhs.
  // One 64-bit base per hop; each component is then base + c * stride with a
  // compile-time c (a single wide multiply-add per address).
  const uint32_t cs_bytes = vh * nrhs * (uint32_t)sizeof(E);
  const char* base = reinterpret_cast<const char*>(in + (nb * nrhs + rhs0));
#pragma unroll
  for (int a = 0; a < N; a++) {
    VecBuf<E, R> p0, p1, q0, q1;
    Vec<E, R>::load(reinterpret_cast<const E*>(base + (uint64_t)(0 * N + a) * cs_bytes), p0.v);
    Vec<E, R>::load(reinterpret_cast<const E*>(base + (uint64_t)(1 * N + a) * cs_bytes), p1.v);
    Vec<E, R>::load(reinterpret_cast<const E*>(base + (uint64_t)(u0p * N + a) * cs_bytes), q0.v);
    Vec<E, R>::load(reinterpret_cast<const E*>(base + (uint64_t)(u1p * N + a) * cs_bytes), q1.v);
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

  // colour multiply row by row, then reconstruct; link component k at
  // lbase + k * ls_bytes
  const char* lbase = reinterpret_cast<const char*>(gauge + link_off);
  const uint32_t ls_bytes = (RC ? 32u : vh) * (uint32_t)sizeof(E);  // component stride (two-row: groups of 32)
  const T klo0 = s * (T)gsign(MU, u0p), klo1 = s * (T)gsign(MU, u1p);
  // SU(3) two-row links: row 2 = conj(row 0 x row 1), reconstructed in the arithmetic precision
  C2<T> ul[RC ? 3 : 1][RC ? 3 : 1];
  if constexpr (RC) {
    static_assert(N == 3, "link reconstruction is SU(3) only");
    load_su3_two_row<S, T>(lbase, ls_bytes, ul);
  }
#pragma unroll
  for (int a = 0; a < N; a++) {
    C2<T> t[2][R];
#pragma unroll
    for (int b = 0; b < N; b++) {
      // forward uses U[a][b]; backward uses conj(U[b][a])
      T ur, ui;
      if constexpr (RC) {
        const C2<T> uc = FWD ? ul[a][b] : ul[b][a];
        ur = uc.x;
        ui = FWD ? uc.y : -uc.y;
      } else {
        const uint32_t comp = FWD ? (a * N + b) : (b * N + a);
        auto uc = S::to_c(__ldg(reinterpret_cast<const E*>(lbase + (uint64_t)comp * ls_bytes)));
        ur = (T)uc.x;
        ui = FWD ? (T)uc.y : -(T)uc.y;
      }
#pragma unroll
      for (int u = 0; u < 2; u++)
#pragma unroll
        for (int r = 0; r < R; r++) {
          if (b == 0) {
            t[u][r].x = ur * h[u][b][r].x;
            t[u][r].y = ur * h[u][b][r].y;
          } else {
            t[u][r].x = fma(ur, h[u][b][r].x, t[u][r].x);
            t[u][r].y = fma(ur, h[u][b][r].y, t[u][r].y);
          }
          t[u][r].x = fma(-ui, h[u][b][r].y, t[u][r].x);
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

// The same hop with FP32 arithmetic on the packed FP32x2 pipe (sm_100+
// fma.rn.f32x2), for storage that computes in FP32 (FP32, FP16, BF16).  The
// two lanes of a packed register hold two right-hand sides, RHS 2q and
// 2q + 1 of the thread: every quantity of the hop (projected half-spinor,
// link product, accumulator) is the same for both, and the link element is
// the same, so the two lanes take one pair of broadcast link values.
//   tr(q) += (ur, ur) * hr(q) + (-ui, -ui) * hi(q)
//   ti(q) += (ur, ur) * hi(q) + ( ui,  ui) * hr(q)
// The spin rows never change lanes, so every reconstruction is packed too.
// Each lane performs exactly the FMA sequence of hop() for its RHS, so the
// results are bit-identical to it.  The 4N spinor components are loaded in
// order with a running pointer (64-bit adds instead of wide multiply-adds).
// The link's components lie at lbase + k * ls_bytes (global memory, or shared
// memory when SMEM).
template <int P, int N, int R, int MU, bool FWD, bool RC, bool SMEM = false>
__device__ __forceinline__ void hop_pk(float2 (&re)[4][N][R / 2], float2 (&im)[4][N][R / 2], const DslashArgs& A,
                                       const typename Store<P>::elem* __restrict__ in, const char* lbase,
                                       uint32_t ls_bytes, uint32_t nb, uint32_t rhs0, float bc, float f) {
  using S = Store<P>;
  using E = typename S::elem;
  static_assert(R % 2 == 0, "packed arithmetic pairs the RHS of a thread");
  constexpr int Q = R / 2;
  constexpr int u0p = gperm(MU, 0), u1p = gperm(MU, 1);
  constexpr bool imag = gimag(MU);
  const float s = FWD ? -f : f;
  const uint32_t vh = (uint32_t)A.geo.vh;
  const uint32_t nrhs = (uint32_t)A.nrhs;

  float2 ku[Q];
  if constexpr (S::has_norm) {
    float nr[R];
    load_norms<P, R>(A.in_norm + (nb * nrhs + rhs0), nr);
#pragma unroll
    for (int q = 0; q < Q; q++) ku[q] = make_float2(bc * nr[2 * q], bc * nr[2 * q + 1]);
  } else {
#pragma unroll
    for (int q = 0; q < Q; q++) ku[q] = make_float2(bc, bc);
  }

  VecBuf<E, R> comp[4 * N];
  {
    const uint32_t cs_bytes = vh * nrhs * (uint32_t)sizeof(E);
    const char* pc = reinterpret_cast<const char*>(in + (nb * nrhs + rhs0));
#pragma unroll
    for (int c = 0; c < 4 * N; c++) {
      Vec<E, R>::load(reinterpret_cast<const E*>(pc), comp[c].v);
      pc += cs_bytes;
    }
  }
  // projection h_u = psi_u + s g(u) psi_perm(u), scalar FMAs into the lanes
  float2 hr[2][N][Q], hi[2][N][Q];
  const float k0 = s * (float)gsign(MU, 0), k1 = s * (float)gsign(MU, 1);
#pragma unroll
  for (int a = 0; a < N; a++)
#pragma unroll
    for (int r = 0; r < R; r++) {
      const float2 x0 = S::to_c(comp[0 * N + a].v[r]), x1 = S::to_c(comp[1 * N + a].v[r]);
      const float2 y0 = S::to_c(comp[u0p * N + a].v[r]), y1 = S::to_c(comp[u1p * N + a].v[r]);
      float h0r, h0i, h1r, h1i;
      if constexpr (imag) {
        h0r = fmaf(-k0, y0.y, x0.x);
        h0i = fmaf(k0, y0.x, x0.y);
        h1r = fmaf(-k1, y1.y, x1.x);
        h1i = fmaf(k1, y1.x, x1.y);
      } else {
        h0r = fmaf(k0, y0.x, x0.x);
        h0i = fmaf(k0, y0.y, x0.y);
        h1r = fmaf(k1, y1.x, x1.x);
        h1i = fmaf(k1, y1.y, x1.y);
      }
      const int q = r >> 1;
      if (r & 1) {
        hr[0][a][q].y = h0r;
        hi[0][a][q].y = h0i;
        hr[1][a][q].y = h1r;
        hi[1][a][q].y = h1i;
      } else {
        hr[0][a][q].x = h0r;
        hi[0][a][q].x = h0i;
        hr[1][a][q].x = h1r;
        hi[1][a][q].x = h1i;
      }
    }

  C2<float> ul[RC ? 3 : 1][RC ? 3 : 1];
  if constexpr (RC) {
    static_assert(N == 3, "link reconstruction is SU(3) only");
    load_su3_two_row<S, float, SMEM>(lbase, ls_bytes, ul);
  }
  const float klo0 = s * (float)gsign(MU, u0p), klo1 = s * (float)gsign(MU, u1p);
#pragma unroll
  for (int a = 0; a < N; a++) {
    float2 tr[2][Q], ti[2][Q];
#pragma unroll
    for (int b = 0; b < N; b++) {
      float ur, uim;  // the stored link element; the backward hop conjugates it
      if constexpr (RC) {
        const C2<float> uc = FWD ? ul[a][b] : ul[b][a];
        ur = uc.x;
        uim = uc.y;
      } else {
        const uint32_t comp_l = FWD ? (a * N + b) : (b * N + a);
        const float2 uc = S::to_c(ld_link<E, SMEM>(lbase + (uint64_t)comp_l * ls_bytes));
        ur = uc.x;
        uim = uc.y;
      }
      // forward: ui = uim, tr -= ui hi, ti += ui hr; backward: ui = -uim
      const float2 ur2 = make_float2(ur, ur);
      const float2 up2 = make_float2(uim, uim), un2 = make_float2(-uim, -uim);
#pragma unroll
      for (int v = 0; v < 2; v++)
#pragma unroll
        for (int q = 0; q < Q; q++) {
          if (b == 0) {
            tr[v][q] = __fmul2_rn(ur2, hr[v][b][q]);
            ti[v][q] = __fmul2_rn(ur2, hi[v][b][q]);
          } else {
            tr[v][q] = __ffma2_rn(ur2, hr[v][b][q], tr[v][q]);
            ti[v][q] = __ffma2_rn(ur2, hi[v][b][q], ti[v][q]);
          }
          tr[v][q] = __ffma2_rn(FWD ? un2 : up2, hi[v][b][q], tr[v][q]);
          ti[v][q] = __ffma2_rn(FWD ? up2 : un2, hr[v][b][q], ti[v][q]);
        }
    }
#pragma unroll
    for (int q = 0; q < Q; q++) {
      const float2 kl0 = make_float2(klo0 * ku[q].x, klo0 * ku[q].y);
      const float2 kl1 = make_float2(klo1 * ku[q].x, klo1 * ku[q].y);
      re[0][a][q] = __ffma2_rn(ku[q], tr[0][q], re[0][a][q]);
      im[0][a][q] = __ffma2_rn(ku[q], ti[0][q], im[0][a][q]);
      re[1][a][q] = __ffma2_rn(ku[q], tr[1][q], re[1][a][q]);
      im[1][a][q] = __ffma2_rn(ku[q], ti[1][q], im[1][a][q]);
      if constexpr (imag) {
        re[u0p][a][q] = __ffma2_rn(make_float2(-kl0.x, -kl0.y), ti[0][q], re[u0p][a][q]);
        im[u0p][a][q] = __ffma2_rn(kl0, tr[0][q], im[u0p][a][q]);
        re[u1p][a][q] = __ffma2_rn(make_float2(-kl1.x, -kl1.y), ti[1][q], re[u1p][a][q]);
        im[u1p][a][q] = __ffma2_rn(kl1, tr[1][q], im[u1p][a][q]);
      } else {
        re[u0p][a][q] = __ffma2_rn(kl0, tr[0][q], re[u0p][a][q]);
        im[u0p][a][q] = __ffma2_rn(kl0, ti[0][q], im[u0p][a][q]);
        re[u1p][a][q] = __ffma2_rn(kl1, tr[1][q], re[u1p][a][q]);
        im[u1p][a][q] = __ffma2_rn(kl1, ti[1][q], im[u1p][a][q]);
      }
    }
  }
}

// accumulator of one thread: complex rows, or the packed lane pairs of hop_pk
template <typename T, int N, int R, bool PK>
struct HopAcc {
  C2<T> c[4][N][R];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int sp = 0; sp < 4; sp++)
#pragma unroll
      for (int a = 0; a < N; a++)
#pragma unroll
        for (int r = 0; r < R; r++) c[sp][a][r].x = c[sp][a][r].y = (T)0;
  }
  __device__ __forceinline__ void to_rows(C2<T> (&acc)[4][N][R]) const {
#pragma unroll
    for (int sp = 0; sp < 4; sp++)
#pragma unroll
      for (int a = 0; a < N; a++)
#pragma unroll
        for (int r = 0; r < R; r++) acc[sp][a][r] = c[sp][a][r];
  }
};

template <typename T, int N, int R>
struct HopAcc<T, N, R, true> {
  float2 re[4][N][R / 2], im[4][N][R / 2];  // lanes: RHS 2q, 2q + 1
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int s = 0; s < 4; s++)
#pragma unroll
      for (int a = 0; a < N; a++)
#pragma unroll
        for (int q = 0; q < R / 2; q++) re[s][a][q] = im[s][a][q] = make_float2(0.f, 0.f);
  }
  __device__ __forceinline__ void to_rows(C2<T> (&acc)[4][N][R]) const {
#pragma unroll
    for (int s = 0; s < 4; s++)
#pragma unroll
      for (int a = 0; a < N; a++)
#pragma unroll
        for (int r = 0; r < R; r++) {
          const int q = r >> 1;
          acc[s][a][r].x = (r & 1) ? re[s][a][q].y : re[s][a][q].x;
          acc[s][a][r].y = (r & 1) ? im[s][a][q].y : im[s][a][q].x;
        }
  }
};

// prefetch of the line holding p into L1: no register is held while it is in flight
__device__ __forceinline__ void prefetch_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

template <int P, int N, int R, bool PK, int MU, bool FWD, bool RC>
__device__ __forceinline__ void hop_any(HopAcc<typename Store<P>::real, N, R, PK>& acc, const DslashArgs& A,
                                       const typename Store<P>::elem* __restrict__ in,
                                       const typename Store<P>::elem* __restrict__ gauge, uint32_t link_off,
                                       uint32_t nb, uint32_t rhs0, typename Store<P>::real bc,
                                       typename Store<P>::real f) {
  if constexpr (PK)
    hop_pk<P, N, R, MU, FWD, RC>(acc.re, acc.im, A, in, reinterpret_cast<const char*>(gauge + link_off),
                                 (RC ? 32u : (uint32_t)A.geo.vh) * (uint32_t)sizeof(typename Store<P>::elem), nb,
                                 rhs0, bc, f);
  else
    hop<P, N, R, MU, FWD, RC>(acc.c, A, in, gauge, link_off, nb, rhs0, bc, f);
}

}  // namespace detail

namespace detail {

// Epilogue of both hop kernels: out = a_r * acc + b * x for one site and R
// RHS (a_r per RHS when a_rhs_f / a_rhs_d is given), written in the storage
// precision; 16-bit storage also writes the per-(site, RHS) scale.
template <int P, int N, int R>
__device__ __forceinline__ void store_out(C2<typename Store<P>::real> (&acc)[4][N][R], const DslashArgs& A,
                                          uint32_t site, uint32_t rhs0) {
  using S = Store<P>;
  using T = typename S::real;
  using E = typename S::elem;
  const uint32_t vh = A.geo.vh;
  const uint32_t nrhs = A.nrhs;
  T ca[R], cbx;
  if constexpr (sizeof(T) == 4) {
    cbx = A.bf;
#pragma unroll
    for (int r = 0; r < R; r++) ca[r] = A.a_rhs_f ? A.a_rhs_f[rhs0 + r] : A.af;
  } else {
    cbx = (T)A.b;
#pragma unroll
    for (int r = 0; r < R; r++) ca[r] = A.a_rhs_d ? (T)A.a_rhs_d[rhs0 + r] : (T)A.a;
  }
  const E* __restrict__ xin = static_cast<const E*>(A.x);
  float xs[R];
  if constexpr (S::has_norm) {
    if (xin) load_norms<P, R>(A.x_norm + (site * nrhs + rhs0), xs);
  }
  const uint32_t cs = vh * nrhs;
  const uint32_t o = site * nrhs + rhs0;
  // a plain D application (a = 1, no x): the accumulator is the result
  const bool plain = !xin && (sizeof(T) == 4 ? (!A.a_rhs_f && A.af == 1.f) : (!A.a_rhs_d && A.a == 1.0));
#pragma unroll
  for (int sp = 0; sp < 4; sp++)
#pragma unroll
    for (int a = 0; a < N; a++) {
      const uint32_t off = o + (uint32_t)(sp * N + a) * cs;
      if (plain) continue;
      if (xin) {
        VecBuf<E, R> xv;
        Vec<E, R>::load(xin + off, xv.v);
#pragma unroll
        for (int r = 0; r < R; r++) {
          auto xc = S::to_c(xv.v[r]);
          T sx = cbx;
          if constexpr (S::has_norm) sx *= (T)xs[r];
          acc[sp][a][r].x = fma(sx, (T)xc.x, ca[r] * acc[sp][a][r].x);
          acc[sp][a][r].y = fma(sx, (T)xc.y, ca[r] * acc[sp][a][r].y);
        }
      } else {
#pragma unroll
        for (int r = 0; r < R; r++) {
          acc[sp][a][r].x *= ca[r];
          acc[sp][a][r].y *= ca[r];
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
    for (int r = 0; r < R; r++) A.out_norm[o + r] = mx[r];
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
        Vec<E, R>::store(out + (o + (uint32_t)(sp * N + a) * cs), ov.v, A.stream_out != 0);
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
        Vec<E, R>::store(out + (o + (uint32_t)(sp * N + a) * cs), ov.v, A.stream_out != 0);
      }
  }
}

}  // namespace detail

// MINB: register-cap variant of the kernel (registers per thread, and with
// them the resident warps per SM, against spills):
//   1: no cap (255), 2: 128, 3: 85, 4: 112, 5: 96, 6: 104.
// 2 and 3 are the caps of 2 and 3 resident 256-thread blocks per SM.
template <int MINB>
struct RegCap {
  static constexpr int regs =
      MINB == 2 ? 128 : MINB == 3 ? 85 : MINB == 4 ? 112 : MINB == 5 ? 96 : MINB == 6 ? 104 : 255;
};

namespace detail {

// The work of one thread of the register kernel: output site x R RHS number
// gid of the launch (gid = site * G + RHS group).
// PK: FP32 arithmetic on the packed FP32x2 pipe, two RHS per packed register
// (FP32 / 16-bit storage, even R).
// RC: SU(3) links read as their first two rows (gauge12), the third reconstructed.
template <int P, int N, int R, bool PK, bool RC>
__device__ __forceinline__ void wilson_site(const DslashArgs& A, uint32_t gid) {
  using S = Store<P>;
  using T = typename S::real;
  using E = typename S::elem;
  static_assert(!PK || sizeof(T) == 4, "packed arithmetic is FP32 only");
  static_assert(!PK || R % 2 == 0, "packed arithmetic pairs the RHS of a thread");

  uint32_t site, grp;
  A.div_groups.divmod(gid, site, grp);
  if (site >= (uint32_t)A.geo.vh) return;
  uint32_t xh, y, z, t;
  const uint32_t rhs0 = grp * R;
  if (A.mask) {
    bool any = false;
#pragma unroll
    for (int r = 0; r < R; r++) any |= A.mask[rhs0 + r] != 0;
    if (!any) return;
  }

  if (A.zb) {  // the site-th site of the slab order: (slab, t, z in slab, y, x)
    uint32_t q, r, q2, zz, slab;
    A.div_plane.divmod(site, q, r);
    A.div_zb.divmod(q, q2, zz);
    A.div_lt.divmod(q2, slab, t);
    z = slab * A.zb + zz;
    A.geo.div_hx.divmod(r, y, xh);
    site = (t * (uint32_t)A.geo.L[2] + z) * (uint32_t)A.geo.plane + r;
  } else {
    uint32_t rest, rest2;
    A.geo.div_hx.divmod(site, rest, xh);
    A.geo.div_y.divmod(rest, rest2, y);
    A.geo.div_z.divmod(rest2, t, z);
  }
  const uint32_t hx = A.geo.hx, Ly = A.geo.L[1], Lz = A.geo.L[2], Lt = A.geo.L[3];
  const uint32_t p = A.parity;
  const uint32_t eo = (y + z + t) & 1u;
  const T f = A.dagger ? (T)-1 : (T)1;
  const uint32_t vh = A.geo.vh;
  const E* __restrict__ in = static_cast<const E*>(A.in);
  const E* __restrict__ gauge = static_cast<const E*>(RC ? A.gauge12 : A.gauge);
  constexpr uint32_t NN = RC ? (N - 1) * N : N * N;  // stored components per link

  HopAcc<T, N, R, PK> hacc;
  hacc.zero();

  // link offsets: forward links at (mu, p, site), backward at (mu, 1-p, nb);
  // full links [8][NN][Vh] (component stride Vh), two-row links in groups of
  // 32 sites (two_row_site, component stride 32)
  const uint32_t lvh = RC ? two_row_vh(vh) : vh;
  const uint32_t lcs = RC ? 32u : vh;
  auto lsite = [](uint32_t s) { return RC ? two_row_site(s) : s; };
  const uint32_t lf = p * NN * lvh + lsite(site);
  const uint32_t lb = (1u - p) * NN * lvh;
  const uint32_t dmu = 2 * NN * lvh;  // one direction's links
  // FP32 and BF16 storage prefetch every hop's links (below; measured 4-19%
  // faster).  FP64 is bound by its FMA pipe and FP16 (with its norm loads)
  // measured 2-6% slower with the prefetch, so they run the hops without it,
  // in the form that compiles best for them.
  if constexpr (P == PREC_SINGLE || P == PREC_BF16) {
    const uint32_t pl = A.geo.plane, cb = A.geo.cube;
    const bool top = t == Lt - 1, bot = t == 0;
    // neighbour of hop h: X+, X-, Y+, Y-, Z+, Z-, T+, T-
    auto nbr = [&](int h) -> uint32_t {
      switch (h) {
        case 0: return (eo != p) ? (xh == hx - 1 ? site - (hx - 1) : site + 1) : site;
        case 1: return (eo == p) ? (xh == 0 ? site + (hx - 1) : site - 1) : site;
        case 2: return (y == Ly - 1) ? site - (Ly - 1) * hx : site + hx;
        case 3: return (y == 0) ? site + (Ly - 1) * hx : site - hx;
        case 4: return (z == Lz - 1) ? site - (Lz - 1) * pl : site + pl;
        case 5: return (z == 0) ? site + (Lz - 1) * pl : site - pl;
        case 6: return top ? site - (Lt - 1) * cb : site + cb;
        default: return bot ? site + (Lt - 1) * cb : site - cb;
      }
    };
    // Each link is read once per launch, so every hop's link comes from DRAM.
    // Prefetching all eight into L1 here, with no registers held, leaves the
    // hops waiting only on their neighbour spinors (mostly L2 hits); the
    // R-groups of a site split the link components between them.
    for (uint32_t k = grp; k < NN; k += A.div_groups.d) {
#pragma unroll
      for (int h = 0; h < 8; h++)
        prefetch_l1(gauge + ((h >> 1) * dmu + ((h & 1) ? lb + lsite(nbr(h)) : lf) + k * lcs));
    }
    hop_any<P, N, R, PK, 0, true, RC>(hacc, A, in, gauge, lf, nbr(0), rhs0, (T)1, f);
    hop_any<P, N, R, PK, 0, false, RC>(hacc, A, in, gauge, lb + lsite(nbr(1)), nbr(1), rhs0, (T)1, f);
    hop_any<P, N, R, PK, 1, true, RC>(hacc, A, in, gauge, dmu + lf, nbr(2), rhs0, (T)1, f);
    hop_any<P, N, R, PK, 1, false, RC>(hacc, A, in, gauge, dmu + lb + lsite(nbr(3)), nbr(3), rhs0, (T)1, f);
    hop_any<P, N, R, PK, 2, true, RC>(hacc, A, in, gauge, 2 * dmu + lf, nbr(4), rhs0, (T)1, f);
    hop_any<P, N, R, PK, 2, false, RC>(hacc, A, in, gauge, 2 * dmu + lb + lsite(nbr(5)), nbr(5), rhs0, (T)1, f);
    {  // T, with the optional antiperiodic sign
      const T bcf = (A.antiperiodic_t && top) ? (T)-1 : (T)1;
      const T bcb = (A.antiperiodic_t && bot) ? (T)-1 : (T)1;
      hop_any<P, N, R, PK, 3, true, RC>(hacc, A, in, gauge, 3 * dmu + lf, nbr(6), rhs0, bcf, f);
      hop_any<P, N, R, PK, 3, false, RC>(hacc, A, in, gauge, 3 * dmu + lb + lsite(nbr(7)), nbr(7), rhs0, bcb, f);
    }
  } else {
    {  // X
      const uint32_t nf = (eo != p) ? (xh == hx - 1 ? site - (hx - 1) : site + 1) : site;
      const uint32_t nbk = (eo == p) ? (xh == 0 ? site + (hx - 1) : site - 1) : site;
      hop_any<P, N, R, PK, 0, true, RC>(hacc, A, in, gauge, lf, nf, rhs0, (T)1, f);
      hop_any<P, N, R, PK, 0, false, RC>(hacc, A, in, gauge, lb + lsite(nbk), nbk, rhs0, (T)1, f);
    }
    {  // Y
      const uint32_t nf = (y == Ly - 1) ? site - (Ly - 1) * hx : site + hx;
      const uint32_t nbk = (y == 0) ? site + (Ly - 1) * hx : site - hx;
      hop_any<P, N, R, PK, 1, true, RC>(hacc, A, in, gauge, dmu + lf, nf, rhs0, (T)1, f);
      hop_any<P, N, R, PK, 1, false, RC>(hacc, A, in, gauge, dmu + lb + lsite(nbk), nbk, rhs0, (T)1, f);
    }
    {  // Z
      const uint32_t pl = A.geo.plane;
      const uint32_t nf = (z == Lz - 1) ? site - (Lz - 1) * pl : site + pl;
      const uint32_t nbk = (z == 0) ? site + (Lz - 1) * pl : site - pl;
      hop_any<P, N, R, PK, 2, true, RC>(hacc, A, in, gauge, 2 * dmu + lf, nf, rhs0, (T)1, f);
      hop_any<P, N, R, PK, 2, false, RC>(hacc, A, in, gauge, 2 * dmu + lb + lsite(nbk), nbk, rhs0, (T)1, f);
    }
    {  // T, with the optional antiperiodic sign
      const uint32_t cb = A.geo.cube;
      const bool top = t == Lt - 1, bot = t == 0;
      const uint32_t nf = top ? site - (Lt - 1) * cb : site + cb;
      const uint32_t nbk = bot ? site + (Lt - 1) * cb : site - cb;
      const T bcf = (A.antiperiodic_t && top) ? (T)-1 : (T)1;
      const T bcb = (A.antiperiodic_t && bot) ? (T)-1 : (T)1;
      hop_any<P, N, R, PK, 3, true, RC>(hacc, A, in, gauge, 3 * dmu + lf, nf, rhs0, bcf, f);
      hop_any<P, N, R, PK, 3, false, RC>(hacc, A, in, gauge, 3 * dmu + lb + lsite(nbk), nbk, rhs0, bcb, f);
    }
  }

  C2<T> acc[4][N][R];
  hacc.to_rows(acc);

  store_out<P, N, R>(acc, A, site, rhs0);
}

}  // namespace detail

template <int P, int N, int R, int MINB, bool PK, bool RC = false>
__global__ void __maxnreg__(RegCap<MINB>::regs) wilson_mrhs_kernel(const DslashArgs A) {
  detail::wilson_site<P, N, R, PK, RC>(A, blockIdx.x * blockDim.x + threadIdx.x);
}

// host-side launcher of one instantiation
template <int P, int N, int R, int MINB, bool PK = false, bool RC = false>
void launch_wilson_mrhs(const DslashArgs& A, int block, cudaStream_t stream) {
  const int groups = A.nrhs / R;
  const int64_t threads = (int64_t)A.geo.vh * groups;
  const int grid = (int)((threads + block - 1) / block);
  wilson_mrhs_kernel<P, N, R, MINB, PK, RC><<<grid, block, 0, stream>>>(A);
}

// One launch over a work list of up to kMaxHopSegments segments: each
// segment is a whole register-kernel launch of its own (lattice, gauge,
// fields, nrhs, parity, coefficients), and block b of the launch is block
// b - block_begin[s] of segment s.  Every thread does exactly what it does in
// the segment's own launch with the same block size, so the results are
// bit-identical to one launch per segment; small lattices share the GPU
// instead of each paying a launch and a tail.
constexpr int kMaxHopSegments = 16;
struct HopSegments {
  int count = 0;
  uint32_t block_begin[kMaxHopSegments + 1];
  DslashArgs A[kMaxHopSegments];
};

template <int P, int N, int R, int MINB, bool PK, bool RC = false>
__global__ void __maxnreg__(RegCap<MINB>::regs) wilson_segments_kernel(const __grid_constant__ HopSegments S) {
  int s = 0;
#pragma unroll 1
  while (s + 1 < S.count && blockIdx.x >= S.block_begin[s + 1]) s++;
  detail::wilson_site<P, N, R, PK, RC>(S.A[s], (blockIdx.x - S.block_begin[s]) * blockDim.x + threadIdx.x);
}

// the segments' div_groups must be set (nrhs / R); fills block_begin
template <int P, int N, int R, int MINB, bool PK = false, bool RC = false>
void launch_wilson_segments(HopSegments& S, int block, cudaStream_t stream) {
  uint32_t total = 0;
  for (int s = 0; s < S.count; s++) {
    S.block_begin[s] = total;
    const int64_t threads = (int64_t)S.A[s].geo.vh * (S.A[s].nrhs / R);
    total += (uint32_t)((threads + block - 1) / block);
  }
  S.block_begin[S.count] = total;
  wilson_segments_kernel<P, N, R, MINB, PK, RC><<<total, block, 0, stream>>>(S);
}

}  // namespace qcu
