// TMA-staged persistent MRHS Wilson hop (the same operator as
// wilson_mrhs_kernel in dslash_kernel.cuh, bit-identical results).
//
// Tile = one x-row of output sites (hx = X/2 consecutive even-odd sites at
// fixed y, z, t) x one chunk of rcta right-hand sides.  Every neighbour of a
// tile lies in one x-row of the input field: the tile's own row for both x
// hops, and the rows at y+-1, z+-1, t+-1 (wrapped) for the others.  So a tile
// is seven stages; stage k brings, with one TMA box each,
//   * the neighbour row of the MRHS field: [4N][hx][rcta] complex, and
//   * the link row(s) of that hop: [N*N][hx] complex (forward links at the
//     tile's own sites, backward links at the neighbour sites),
// into a ring of NST shared-memory buffers.  The links are staged once per
// tile and reused by all rcta RHS of the tile.
//
// Warp roles: one producer warp (lane 0 issues the copies; the others idle)
// and hx * rcta / R consumer threads (one site x R RHS each, like the
// register kernel).  Full / empty mbarriers per buffer; consumers release a
// buffer per warp.  The kernel is persistent: each CTA walks tiles
// blockIdx.x, blockIdx.x + gridDim.x, ..., with the ring running across
// tiles, so the next tile's rows load while the current one finishes.
//
// Every mbarrier wait is bounded (about one second of %globaltimer); on
// timeout the thread sets *err and returns, and the host reports
// QCU_ERR_DEVICE_TIMEOUT.
#pragma once

#include <cuda.h>

#include "dslash_kernel.cuh"

namespace qcu {

struct TmaDslashArgs {
  DslashArgs A;  // operator arguments, as for the register kernel
  int rcta;      // RHS per tile (box inner extent)
  int chunks;    // nrhs / rcta
  int ntiles;    // rows * chunks
  int rows;      // Vh / hx
  uint32_t spin_bytes, norm_bytes, link_bytes;     // exact box sizes (the transaction counts)
  uint32_t spin_stride, norm_stride, link_stride;  // their 128-byte aligned places in a buffer;
                                                   // norm: 16-bit storage only, else 0
  uint32_t stage_bytes;               // one ring buffer
  int* err;      // set to 1 when a wait times out
};

namespace tma {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ uint64_t now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait until the phase with the given parity has completed; false after
// about limit_ns nanoseconds (default one second; then *err is set).  After
// the first poll the warp is suspended in try_wait (suspend-time hint) until
// the phase completes or the hint runs out, so waiting warps take no issue
// slots from working ones; the clock is read every 16 polls.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err,
                                          uint64_t limit_ns = 1000000000ull) {
  uint32_t ok = 0;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  if (ok) return true;
  const uint64_t t0 = now_ns();
  for (uint32_t i = 1;; i++) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(1000000u)
        : "memory");
    if (ok) return true;
    if ((i & 15u) == 0 && now_ns() - t0 > limit_ns) {
      atomicExch(err, 1);
      return false;
    }
  }
}

// The same bounded wait, polling with the non-blocking test_wait (no warp
// suspension): for barriers that tcgen05.commit arrives on, where a short
// wait is expected.
__device__ __forceinline__ bool mbar_poll(uint32_t bar, uint32_t parity, int* err) {
  uint64_t t0 = 0;
  for (uint32_t i = 0;; i++) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (i == 0) t0 = now_ns();
    if ((i & 63u) == 63u && now_ns() - t0 > 1000000000ull) {
      atomicExch(err, 1);
      return false;
    }
  }
}

// 2-D tiled TMA load into shared memory, completion counted on bar
__device__ __forceinline__ void load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
      : "memory");
}

// 3-D tiled TMA load into shared memory, completion counted on bar
__device__ __forceinline__ void load_3d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
      : "memory");
}

// One hop from staged data.  spin: the neighbour site's component 0 for this
// thread's R RHS, components cs elements apart; nrm: the neighbour site's
// scales of those RHS (16-bit storage); link: component 0 of the link,
// components ls elements apart.  The arithmetic is detail::hop's, operation
// for operation.
template <int P, int N, int R, int MU, bool FWD>
__device__ __forceinline__ void hop_staged(detail::C2<typename Store<P>::real> (&acc)[4][N][R],
                                           const typename Store<P>::elem* spin, uint32_t cs, const float* nrm,
                                           const typename Store<P>::elem* link, uint32_t ls,
                                           typename Store<P>::real bc, typename Store<P>::real f) {
  using namespace detail;
  using S = Store<P>;
  using T = typename S::real;
  using E = typename S::elem;
  constexpr int u0p = gperm(MU, 0), u1p = gperm(MU, 1);
  constexpr bool im = gimag(MU);
  const T s = FWD ? -f : f;
  T scale[R];
#pragma unroll
  for (int r = 0; r < R; r++) {
    if constexpr (S::has_norm)
      scale[r] = bc * nrm[r];
    else
      scale[r] = bc;
  }
  C2<T> h[2][N][R];
  const T k0 = s * (T)gsign(MU, 0), k1 = s * (T)gsign(MU, 1);
#pragma unroll
  for (int a = 0; a < N; a++) {
    VecBuf<E, R> p0, p1, q0, q1;
    Vec<E, R>::load_shared(spin + (0 * N + a) * cs, p0.v);
    Vec<E, R>::load_shared(spin + (1 * N + a) * cs, p1.v);
    Vec<E, R>::load_shared(spin + (u0p * N + a) * cs, q0.v);
    Vec<E, R>::load_shared(spin + (u1p * N + a) * cs, q1.v);
#pragma unroll
    for (int r = 0; r < R; r++) {
      const auto x0 = S::to_c(p0.v[r]), x1 = S::to_c(p1.v[r]);
      const auto y0 = S::to_c(q0.v[r]), y1 = S::to_c(q1.v[r]);
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
      const uint32_t comp = FWD ? (a * N + b) : (b * N + a);
      const auto uc = S::to_c(link[comp * ls]);
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

}  // namespace tma

// The seven stages of a tile: 0 = x (own row: both x hops), then +y, -y,
// +z, -z, +t, -t.  Forward hops use the forward link at the tile's own sites
// (parity p); backward hops the link at the neighbour site (parity 1 - p),
// which lies in the neighbour row.
template <int P, int N, int R, int NST>
__global__ void __launch_bounds__(512, 1)
    wilson_tma_kernel(const __grid_constant__ TmaDslashArgs T, const __grid_constant__ CUtensorMap map_in,
                      const __grid_constant__ CUtensorMap map_gauge, const __grid_constant__ CUtensorMap map_norm) {
  using S = Store<P>;
  using Tr = typename S::real;
  using E = typename S::elem;
  using namespace detail;
  constexpr int KST = 7;
  const DslashArgs& A = T.A;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)NST * T.stage_bytes);
  const uint32_t full0 = tma::smem_u32(bars), empty0 = tma::smem_u32(bars + NST);

  const int hx = A.geo.hx;
  const int G = T.rcta / R;                       // consumer threads per site
  const int n_cons = (int)blockDim.x - 32;        // consumer threads (whole warps)
  const int n_cons_warps = n_cons / 32;
  const bool producer = (int)threadIdx.x >= n_cons;

  if (threadIdx.x == 0) {
    for (int b = 0; b < NST; b++) {
      tma::mbar_init(full0 + 8 * b, 1);
      tma::mbar_init(empty0 + 8 * b, n_cons_warps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  const int Ly = A.geo.L[1], Lz = A.geo.L[2], Lt = A.geo.L[3];
  const int p = A.parity;

  if (producer) {
    if (threadIdx.x != (unsigned)n_cons) return;
    uint32_t q = 0;
    for (int tile = blockIdx.x; tile < T.ntiles; tile += gridDim.x) {
      const int row = tile / T.chunks, chunk = tile - row * T.chunks;
      const int y = row % Ly, zt = row / Ly, z = zt % Lz, t = zt / Lz;
      const int yp = y + 1 == Ly ? 0 : y + 1, ym = y == 0 ? Ly - 1 : y - 1;
      const int zp = z + 1 == Lz ? 0 : z + 1, zm = z == 0 ? Lz - 1 : z - 1;
      const int tp = t + 1 == Lt ? 0 : t + 1, tm = t == 0 ? Lt - 1 : t - 1;
      const int rows_in[KST] = {row, (t * Lz + z) * Ly + yp, (t * Lz + z) * Ly + ym, (t * Lz + zp) * Ly + y,
                                (t * Lz + zm) * Ly + y, (tp * Lz + z) * Ly + y, (tm * Lz + z) * Ly + y};
      for (int k = 0; k < KST; k++, q++) {
        const int b = q % NST;
        if (q >= (uint32_t)NST && !tma::mbar_wait(empty0 + 8 * b, ((q / NST) - 1) & 1, T.err)) return;
        const uint32_t full = full0 + 8 * b;
        unsigned char* buf = smem + (size_t)b * T.stage_bytes;
        const int nlinks = k == 0 ? 2 : 1;
        tma::mbar_expect_tx(full, T.spin_bytes + T.norm_bytes + nlinks * T.link_bytes);
        // field box {rcta, hx, 4N} at (chunk * rcta, row start, 0); coordinates in 4-byte units
        tma::load_3d(tma::smem_u32(buf), &map_in, chunk * T.rcta * (int)(sizeof(E) / 4), rows_in[k] * hx, 0, full);
        // 16-bit storage: the row's scales, box {rcta, hx} of the [Vh][nrhs] float array
        if constexpr (S::has_norm)
          tma::load_2d(tma::smem_u32(buf + T.spin_stride), &map_norm, chunk * T.rcta, rows_in[k] * hx, full);
        // links: box {hx, N*N, 1} at (row start, 0, 2 mu + parity)
        const int mu = (k + 1) / 2;
        const bool fwd = k == 0 || (k & 1);
        const int lrow = fwd ? row : rows_in[k];
        const int lpar = fwd ? p : 1 - p;
        const uint32_t l0 = tma::smem_u32(buf + T.spin_stride + T.norm_stride);
        tma::load_3d(l0, &map_gauge, lrow * hx * (int)(sizeof(E) / 4), 0, 2 * mu + lpar, full);
        if (k == 0)  // backward x links: own row, parity 1 - p
          tma::load_3d(l0 + T.link_stride, &map_gauge, row * hx * (int)(sizeof(E) / 4), 0, 1 - p, full);
      }
    }
    return;
  }

  // ---- consumers ------------------------------------------------------------
  const int lane = threadIdx.x & 31;
  const int s = (int)threadIdx.x / G, g = (int)threadIdx.x - s * G;
  const bool worker = s < hx;
  const Tr f = A.dagger ? (Tr)-1 : (Tr)1;
  const uint32_t cs = (uint32_t)(hx * T.rcta);  // field component stride in the buffer (elements)
  const uint32_t ls = (uint32_t)hx;             // link component stride
  const uint32_t nrhs = (uint32_t)A.nrhs;
  uint32_t q = 0;
  for (int tile = blockIdx.x; tile < T.ntiles; tile += gridDim.x) {
    const int row = tile / T.chunks, chunk = tile - row * T.chunks;
    const int y = row % Ly, zt = row / Ly, z = zt % Lz, t = zt / Lz;
    const uint32_t eo = (uint32_t)(y + z + t) & 1u;
    const int rhs0 = chunk * T.rcta + g * R;
    bool active = worker;
    if (active && A.mask) {
      bool any = false;
#pragma unroll
      for (int r = 0; r < R; r++) any |= A.mask[rhs0 + r] != 0;
      active = any;
    }
    C2<Tr> acc[4][N][R];
#pragma unroll
    for (int sp = 0; sp < 4; sp++)
#pragma unroll
      for (int a = 0; a < N; a++)
#pragma unroll
        for (int r = 0; r < R; r++) acc[sp][a][r].x = acc[sp][a][r].y = (Tr)0;

    for (int k = 0; k < KST; k++, q++) {
      const int b = q % NST;
      if (!tma::mbar_wait(full0 + 8 * b, (q / NST) & 1, T.err)) return;
      if (active) {
        const unsigned char* buf = smem + (size_t)b * T.stage_bytes;
        const E* spin = reinterpret_cast<const E*>(buf) + g * R;
        const float* nrm = reinterpret_cast<const float*>(buf + T.spin_stride) + g * R;
        const E* link = reinterpret_cast<const E*>(buf + T.spin_stride + T.norm_stride);
        switch (k) {
          case 0: {
            const uint32_t xh = (uint32_t)s;
            const uint32_t nf = (eo != (uint32_t)p) ? (xh == (uint32_t)hx - 1 ? 0 : xh + 1) : xh;
            const uint32_t nbk = (eo == (uint32_t)p) ? (xh == 0 ? (uint32_t)hx - 1 : xh - 1) : xh;
            tma::hop_staged<P, N, R, 0, true>(acc, spin + nf * T.rcta, cs, nrm + nf * T.rcta, link + xh, ls, (Tr)1, f);
            tma::hop_staged<P, N, R, 0, false>(acc, spin + nbk * T.rcta, cs, nrm + nbk * T.rcta,
                                                link + T.link_stride / sizeof(E) + nbk, ls, (Tr)1, f);
            break;
          }
          case 1:
            tma::hop_staged<P, N, R, 1, true>(acc, spin + s * T.rcta, cs, nrm + s * T.rcta, link + s, ls, (Tr)1, f);
            break;
          case 2:
            tma::hop_staged<P, N, R, 1, false>(acc, spin + s * T.rcta, cs, nrm + s * T.rcta, link + s, ls, (Tr)1, f);
            break;
          case 3:
            tma::hop_staged<P, N, R, 2, true>(acc, spin + s * T.rcta, cs, nrm + s * T.rcta, link + s, ls, (Tr)1, f);
            break;
          case 4:
            tma::hop_staged<P, N, R, 2, false>(acc, spin + s * T.rcta, cs, nrm + s * T.rcta, link + s, ls, (Tr)1, f);
            break;
          case 5: {
            const Tr bcf = (A.antiperiodic_t && t == Lt - 1) ? (Tr)-1 : (Tr)1;
            tma::hop_staged<P, N, R, 3, true>(acc, spin + s * T.rcta, cs, nrm + s * T.rcta, link + s, ls, bcf, f);
            break;
          }
          default: {
            const Tr bcb = (A.antiperiodic_t && t == 0) ? (Tr)-1 : (Tr)1;
            tma::hop_staged<P, N, R, 3, false>(acc, spin + s * T.rcta, cs, nrm + s * T.rcta, link + s, ls, bcb, f);
            break;
          }
        }
      }
      __syncwarp();
      if (lane == 0) tma::mbar_arrive(empty0 + 8 * b);
    }
    if (!active) continue;

    detail::store_out<P, N, R>(acc, A, (uint32_t)(row * hx + s), (uint32_t)rhs0);
  }
}

}  // namespace qcu
