// Tensor-core MRHS Wilson hop for SU(N), N = 4..8, BF16 storage (tcgen05).
//
// For one output site x and one hop (mu, +-), every RHS r and projected spin
// row u in {0, 1} needs t_u(r) = W h_u(r), W = U_mu(x) or U_mu(x - mu)^dag, an
// N x N complex link shared by all RHS.  Written as real matrices,
//   D[m][n] += sum_k A[m][k] B[k][n],   m = 2 r + u,
//   A[m][2b + c] = (Re, Im)_c of h_u(r)_b            (one packed BF16 pair per colour; K padded to 16)
//   B[2b + c][2a + c'] = the 2x2 real block of W_ab: [[Re W_ab, Im W_ab], [-Im W_ab, Re W_ab]]
// is one tcgen05.mma of M = 128 (64 RHS x 2 rows), N = 16, K = 16 per hop
// for the upper spin rows, and a second one for the lower rows: the rows of
// A' hold klo_u h_u at the lower row they feed (rows swapped for mu = x, y),
// and B' = B times the +-i of the imaginary gamma rows (mu = x, z).  Both
// accumulate over the eight hops in tensor memory (FP32, 2 x 16 columns of
// 128 lanes), so the CUDA cores only project (h = psi_u + k psi_perm(u),
// times the boundary sign), convert to
// BF16 and write the operands; the N x N complex multiply runs on the tensor
// pipe, with the link operand built once per hop and used by all RHS of the
// tile.  The epilogue reads the accumulators back (tcgen05.ld), applies the
// xpay / per-RHS a, and writes BF16 (BF16 fields are stored unscaled).
//
// CTA = 128 threads, thread m = 2 r + u owns row m (TMEM lane m).  Operands
// are double buffered in shared memory; an mbarrier per buffer signals
// (tcgen05.commit) when the MMAs reading it have finished.  Every wait is
// bounded; a timeout sets *err, the CTA agrees to stop (__syncthreads_or),
// waits once more (bounded) for its MMAs in flight, frees its tensor memory
// and returns.  Tensor memory: 32 columns per CTA; the shared memory of a CTA
// keeps at most 12 CTAs on an SM (384 of its 512 columns), so the allocation
// never waits.
#pragma once

#include <type_traits>

#include "dslash_kernel.cuh"
#include "dslash_tma.cuh"

namespace qcu {

struct TcDslashArgs {
  DslashArgs A;
  int rt;      // RHS per tile (<= 64)
  int chunks;  // nrhs / rt
  int ntiles;  // vh * chunks
  int* err;    // set to 1 when a wait times out
  // TMA-fed variant: ring stage = the neighbour site's [4N][rt] spinor block
  uint32_t spin_bytes = 0, stage_bytes = 0;
};

namespace tc {

constexpr int kSetBytes = 9216;  // A 4096, A' 4096, B 512, B' 512
constexpr int kSmemBytes = 2 * kSetBytes + 64;
// TMA-fed variant: the stage ring starts 128-byte aligned after the operands
// and the barriers (operand barriers at +0, +8; tensor-memory slot at +16;
// ring barriers at +24 + 8 s)
constexpr int kRingOffset = 2 * kSetBytes + 128;

// shared-memory matrix descriptor: K-major, no swizzle; lbo = byte stride of
// core matrices along K, sbo = along M (N for B); bits 46-48 = 0b001
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
         ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}

// instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// byte offset of element (row, k) in a K-major, no-swizzle operand with
// K = 16: core matrices of 8 rows x 16 bytes, lbo = 128, sbo = 256
__device__ __forceinline__ uint32_t kmaj_off(uint32_t row, uint32_t k) {
  return (row >> 3) * 256u + (k >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's lane
__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc

// neighbour (half-lattice index) of `site` for hop d (mu = d / 2, forward for even d)
__device__ __forceinline__ uint32_t tc_neighbour(const DslashArgs& A, uint32_t site, int d) {
  uint32_t rest, xh, y, z, t, rest2;
  A.geo.div_hx.divmod(site, rest, xh);
  A.geo.div_y.divmod(rest, rest2, y);
  A.geo.div_z.divmod(rest2, t, z);
  const uint32_t hx = A.geo.hx, Ly = A.geo.L[1], Lz = A.geo.L[2], Lt = A.geo.L[3], p = A.parity;
  const uint32_t eo = (y + z + t) & 1u;
  const bool fwd = (d & 1) == 0;
  switch (d >> 1) {
    case 0:
      return fwd ? ((eo != p) ? (xh == hx - 1 ? site - (hx - 1) : site + 1) : site)
                 : ((eo == p) ? (xh == 0 ? site + (hx - 1) : site - 1) : site);
    case 1:
      return fwd ? ((y == Ly - 1) ? site - (Ly - 1) * hx : site + hx) : ((y == 0) ? site + (Ly - 1) * hx : site - hx);
    case 2: {
      const uint32_t pl = A.geo.plane;
      return fwd ? ((z == Lz - 1) ? site - (Lz - 1) * pl : site + pl) : ((z == 0) ? site + (Lz - 1) * pl : site - pl);
    }
    default: {
      const uint32_t cb = A.geo.cube;
      return fwd ? ((t == Lt - 1) ? site - (Lt - 1) * cb : site + cb) : ((t == 0) ? site + (Lt - 1) * cb : site - cb);
    }
  }
}

// NST = 0: the projection reads the neighbour spinors straight from global
// memory; NST > 0: thread 0 streams them with one TMA box
// per hop into a ring of NST shared-memory stages, NST - 1 hops ahead.  The
// CTA barrier of every hop orders the reads of a stage before its refill.
template <int N, int NST>
__global__ void __launch_bounds__(128)
    wilson_tc_kernel(const __grid_constant__ TcDslashArgs T, const __grid_constant__ CUtensorMap map_in) {
  static_assert(N >= 2 && N <= 8, "K = 2N must fit one K = 16 MMA step");
  static_assert(NST >= 0 && NST <= 4, "ring stages");
  using namespace detail;
  using S = Store<PREC_BF16>;
  using E = typename S::elem;
  const DslashArgs& A = T.A;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + 2 * tc::kSetBytes);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 2 * tc::kSetBytes + 16);
  const uint32_t bar0 = tma::smem_u32(bars);
  const uint32_t smem0 = tma::smem_u32(smem);
  const int tid = threadIdx.x, warp = tid >> 5;

  const uint32_t ring_bar0 = bar0 + 24;  // NST ring barriers
  if (tid == 0) {
    tma::mbar_init(bar0, 1);
    tma::mbar_init(bar0 + 8, 1);
    for (int st = 0; st < NST; st++) tma::mbar_init(ring_bar0 + 8 * st, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tma::smem_u32(tmem_slot)),
                 "r"(32u)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tmem_slot;
  constexpr uint32_t idesc = tc::idesc_bf16(128, 16);

  const int r = tid >> 1, u = tid & 1;
  const bool row_live = r < T.rt;
  const uint32_t vh = A.geo.vh, nrhs = A.nrhs, hx = A.geo.hx;
  const uint32_t Ly = A.geo.L[1], Lz = A.geo.L[2], Lt = A.geo.L[3];
  const uint32_t p = A.parity;
  const float f = A.dagger ? -1.f : 1.f;
  const E* __restrict__ in = static_cast<const E*>(A.in);
  const E* __restrict__ gauge = static_cast<const E*>(A.gauge);
  constexpr uint32_t NN = N * N;
  const uint32_t cs = vh * nrhs;  // field component stride (elements)

  // link operand: this thread writes elements (n, 2b) and (n, 2b + 1) of the
  // 16 x 16 (n, k) B and B' (one packed BF16 pair each), n = 2a + c (colour a
  // of t, c = Re / Im), k = 2b + c' (colour b of h): both come from W_ab
  const uint32_t bn = (uint32_t)tid >> 3, bb = (uint32_t)tid & 7u, ba = bn >> 1;
  const bool bim = (bn & 1u) != 0, bval = ba < (uint32_t)N && bb < (uint32_t)N;
  const uint32_t boff_f = (ba * N + bb) * vh, boff_b = (bb * N + ba) * vh;  // W = U_ab, or conj(U_ba)
  const uint32_t boffs = tc::kmaj_off(bn, 2 * bb);

  uint32_t q = 0;  // hops issued so far (operand buffer = q & 1)
  bool failed = false;
  // TMA ring (thread 0): hop qq of this CTA -> its stage, issued NST - 1 hops ahead
  uint32_t issued = 0;
  auto issue = [&](uint32_t qq) {
    if constexpr (NST > 0) {
      const int tile = (int)blockIdx.x + (int)(qq >> 3) * (int)gridDim.x;
      if (tile >= T.ntiles) return;
      const uint32_t st_site = (uint32_t)(tile / T.chunks), st_chunk = (uint32_t)(tile % T.chunks);
      const uint32_t nbq = tc_neighbour(A, st_site, (int)(qq & 7u));
      const uint32_t stage = qq % NST, bar = ring_bar0 + 8 * stage;
      const uint32_t dst = smem0 + tc::kRingOffset + stage * T.stage_bytes;
      tma::mbar_expect_tx(bar, T.spin_bytes);
      tma::load_3d(dst, &map_in, (int)(st_chunk * T.rt), (int)nbq, 0, bar);
      issued = qq + 1;
    }
  };
  if constexpr (NST > 0) {
    if (tid == 0)
      for (uint32_t qq = 0; qq + 1 < (uint32_t)NST; qq++) issue(qq);
  }
  for (int tile = blockIdx.x; tile < T.ntiles && !failed; tile += gridDim.x) {
    const uint32_t site = (uint32_t)(tile / T.chunks), chunk = (uint32_t)(tile % T.chunks);
    const uint32_t rhs = chunk * (uint32_t)T.rt + (uint32_t)r;
    uint32_t rest, xh, y, z, t, rest2;
    A.geo.div_hx.divmod(site, rest, xh);
    A.geo.div_y.divmod(rest, rest2, y);
    A.geo.div_z.divmod(rest2, t, z);
    const uint32_t eo = (y + z + t) & 1u;

    // hop D (mu = D / 2, forward for even D), all choices of the hop known at
    // compile time; returns false when the CTA stops after a timeout
    auto hop = [&](auto dc) -> bool {
      constexpr int D = decltype(dc)::value;
      constexpr int mu = D >> 1;
      constexpr bool fwd = (D & 1) == 0;
      constexpr bool imag = mu == 0 || mu == 2;
      const uint32_t b = q & 1u;
      // operand buffer b is free once the MMAs of hop q - 2 have completed
      bool ok = true;
      if (q >= 2) ok = tma::mbar_poll(bar0 + 8 * b, ((q >> 1) - 1) & 1u, T.err);
      [[maybe_unused]] const unsigned char* stage_p = nullptr;
      if constexpr (NST > 0) {
        // refill the stage hop q - 1 read (all threads have passed its barrier), then wait for hop q's
        if (tid == 0) {
          tc::fence_async_smem();  // the stage's generic reads (ordered by the last barrier) before the refill
          issue(q + NST - 1);
        }
        ok = ok && tma::mbar_poll(ring_bar0 + 8 * (q % NST), (q / NST) & 1u, T.err);
        stage_p = smem + tc::kRingOffset + (q % NST) * T.stage_bytes;
      }
      uint32_t nb;
      float bc = 1.f;
      if constexpr (mu == 0) {
        nb = fwd ? ((eo != p) ? (xh == hx - 1 ? site - (hx - 1) : site + 1) : site)
                 : ((eo == p) ? (xh == 0 ? site + (hx - 1) : site - 1) : site);
      } else if constexpr (mu == 1) {
        nb = fwd ? ((y == Ly - 1) ? site - (Ly - 1) * hx : site + hx) : ((y == 0) ? site + (Ly - 1) * hx : site - hx);
      } else if constexpr (mu == 2) {
        const uint32_t pl = A.geo.plane;
        nb = fwd ? ((z == Lz - 1) ? site - (Lz - 1) * pl : site + pl) : ((z == 0) ? site + (Lz - 1) * pl : site - pl);
      } else {
        const uint32_t cb = A.geo.cube;
        nb = fwd ? ((t == Lt - 1) ? site - (Lt - 1) * cb : site + cb) : ((t == 0) ? site + (Lt - 1) * cb : site - cb);
        if (A.antiperiodic_t && (fwd ? t == Lt - 1 : t == 0)) bc = -1.f;
      }
      const float s = fwd ? -f : f;
      unsigned char* set = smem + b * tc::kSetBytes;

      if (ok && row_live) {
        // projected row u of RHS rhs, times the boundary sign bc; A row word c = (Re h_c, Im h_c)
        const int up = (mu < 2) ? 3 - u : (u ^ 2);
        const E *xp, *yp;
        uint32_t astride;  // element stride between colours
        if constexpr (NST > 0) {
          // stage: [4N][rt] spinor components
          xp = reinterpret_cast<const E*>(stage_p) + (uint32_t)(u * N) * T.rt + r;
          yp = reinterpret_cast<const E*>(stage_p) + (uint32_t)(up * N) * T.rt + r;
          astride = (uint32_t)T.rt;
        } else {
          xp = in + ((uint32_t)(u * N) * cs + nb * nrhs + rhs);
          yp = in + ((uint32_t)(up * N) * cs + nb * nrhs + rhs);
          astride = cs;
        }
        const float scale = bc;
        const float ks = s * (float)gsign(mu, u) * scale;
        uint32_t va[8];
#pragma unroll
        for (int a = 0; a < 8; a++) {
          if (a < N) {
            const float2 x = S::to_c(NST > 0 ? xp[(uint32_t)a * astride] : __ldg(xp + (uint32_t)a * astride));
            const float2 yv = S::to_c(NST > 0 ? yp[(uint32_t)a * astride] : __ldg(yp + (uint32_t)a * astride));
            float hr, hi;
            if constexpr (imag) {
              hr = fmaf(-ks, yv.y, scale * x.x);
              hi = fmaf(ks, yv.x, scale * x.y);
            } else {
              hr = fmaf(ks, yv.x, scale * x.x);
              hi = fmaf(ks, yv.y, scale * x.y);
            }
            const __nv_bfloat162 v = __floats2bfloat162_rn(hr, hi);
            va[a] = *reinterpret_cast<const uint32_t*>(&v);
          } else {
            va[a] = 0u;
          }
        }
        // A' row (lower spin perm(u) - 2) = klo * h, klo = s * sign(mu, perm(u)) = +-1: sign bits flipped
        const uint32_t flip = (s * (float)gsign(mu, up) < 0.f) ? 0x80008000u : 0u;
        const uint32_t row2 = (uint32_t)(2 * r + (up - 2));
        *reinterpret_cast<uint4*>(set + tc::kmaj_off((uint32_t)tid, 0)) = make_uint4(va[0], va[1], va[2], va[3]);
        *reinterpret_cast<uint4*>(set + tc::kmaj_off((uint32_t)tid, 8)) = make_uint4(va[4], va[5], va[6], va[7]);
        *reinterpret_cast<uint4*>(set + 4096 + tc::kmaj_off(row2, 0)) =
            make_uint4(va[0] ^ flip, va[1] ^ flip, va[2] ^ flip, va[3] ^ flip);
        *reinterpret_cast<uint4*>(set + 4096 + tc::kmaj_off(row2, 8)) =
            make_uint4(va[4] ^ flip, va[5] ^ flip, va[6] ^ flip, va[7] ^ flip);
      }
      if (ok) {
        // B: re t_a = sum_b wr re h_b - wi im h_b, im t_a = sum_b wi re h_b + wr im h_b;
        // B' = B for real gamma rows, (re, im) of i t = (-im t, re t) for imaginary ones
        float2 bv = make_float2(0.f, 0.f), bv2 = make_float2(0.f, 0.f);
        if (bval) {
          const uint32_t link_off = ((uint32_t)(2 * mu) + (fwd ? p : 1u - p)) * NN * vh + (fwd ? site : nb);
          const float2 w = S::to_c(__ldg(gauge + (link_off + (fwd ? boff_f : boff_b))));
          const float wr = w.x, wi = fwd ? w.y : -w.y;
          bv = bim ? make_float2(wi, wr) : make_float2(wr, -wi);
          if constexpr (imag)
            bv2 = bim ? make_float2(wr, -wi) : make_float2(-wi, -wr);
          else
            bv2 = bv;
        }
        *reinterpret_cast<__nv_bfloat162*>(set + 8192 + boffs) = __floats2bfloat162_rn(bv.x, bv.y);
        *reinterpret_cast<__nv_bfloat162*>(set + 8704 + boffs) = __floats2bfloat162_rn(bv2.x, bv2.y);
      }
      tc::fence_async_smem();
      if (__syncthreads_or(!ok)) return false;
      if (tid == 0) {
        tc::fence_after();
        const uint32_t base = smem0 + b * tc::kSetBytes;
        const uint64_t da = tc::smem_desc(base, 128, 256), da2 = tc::smem_desc(base + 4096, 128, 256);
        const uint64_t db = tc::smem_desc(base + 8192, 128, 256), db2 = tc::smem_desc(base + 8704, 128, 256);
        tc::mma_bf16(tmem, da, db, idesc, D > 0);
        tc::mma_bf16(tmem + 16, da2, db2, idesc, D > 0);
        tc::commit(bar0 + 8 * b);
      }
      q++;
      return true;
    };
    failed = !(hop(std::integral_constant<int, 0>{}) && hop(std::integral_constant<int, 1>{}) &&
               hop(std::integral_constant<int, 2>{}) && hop(std::integral_constant<int, 3>{}) &&
               hop(std::integral_constant<int, 4>{}) && hop(std::integral_constant<int, 5>{}) &&
               hop(std::integral_constant<int, 6>{}) && hop(std::integral_constant<int, 7>{}));
    if (failed) break;

    // all MMAs of this tile done (the commit of its last hop covers them)
    const uint32_t ql = q - 1;
    const bool ok = tma::mbar_poll(bar0 + 8 * (ql & 1u), (ql >> 1) & 1u, T.err);
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    tc::fence_after();
    float up_v[16], lo_v[16];
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
    tc::ld16(lane_addr, up_v);
    tc::ld16(lane_addr + 16, lo_v);
    tc::fence_before();

    // epilogue: out spins u and 2 + u of RHS rhs at this site
    float o[2][2 * N];  // D column 2a + c = (Re, Im) of colour a
#pragma unroll
    for (int a = 0; a < 2 * N; a++) {
      o[0][a] = up_v[a];
      o[1][a] = lo_v[a];
    }
    if (row_live) {
      const float ca = A.a_rhs_f ? A.a_rhs_f[rhs] : A.af;
      const E* __restrict__ xin = static_cast<const E*>(A.x);
      const float xs = A.bf;
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const uint32_t sp = (uint32_t)(u + 2 * h);
#pragma unroll
        for (int a = 0; a < N; a++) {
          float re = ca * o[h][2 * a], im = ca * o[h][2 * a + 1];
          if (xin) {
            const float2 xv = S::to_c(xin[(sp * N + a) * cs + site * nrhs + rhs]);
            re = fmaf(xs, xv.x, re);
            im = fmaf(xs, xv.y, im);
          }
          o[h][2 * a] = re;
          o[h][2 * a + 1] = im;
        }
      }
    }
    if (row_live && (!A.mask || A.mask[rhs] != 0)) {
      E* __restrict__ out = static_cast<E*>(A.out);
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const uint32_t sp = (uint32_t)(u + 2 * h);
#pragma unroll
        for (int a = 0; a < N; a++)
          out[(sp * N + a) * cs + site * nrhs + rhs] = S::from_c(make_float2(o[h][2 * a], o[h][2 * a + 1]));
      }
    }
  }

  if (failed && tid == 0 && q > 0) {
    // let the MMAs in flight finish before the tensor memory is released (bounded)
    const uint32_t ql = q - 1;
    tma::mbar_poll(bar0 + 8 * (ql & 1u), (ql >> 1) & 1u, T.err);
  }
  if constexpr (NST > 0) {
    // copies still in flight land before the CTA's shared memory is released (bounded)
    if (failed && tid == 0)
      for (uint32_t qq = q; qq < issued; qq++) tma::mbar_poll(ring_bar0 + 8 * (qq % NST), (qq / NST) & 1u, T.err);
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(32u) : "memory");
}

}  // namespace qcu
