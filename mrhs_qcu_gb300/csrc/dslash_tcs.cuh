// Tensor-core MRHS Wilson hop with the neighbour spinor block as the MMA's A
// operand (tcgen05, BF16 storage, SU(N) for N = 2..8).
//
// For one output site and one hop, the contribution to every RHS r is
// out(r) += K_hop psi_nb(r), K_hop = bc (1 -+ f gamma_mu) (x) W, a 4N x 4N
// complex matrix shared by all RHS (W = U_mu(x) or U_mu(x - mu)^dag).  As one
// real tcgen05.mma of M = 128, N = 64, K = 32 (two K = 16 steps):
//   A[m][k] = part ri of psi_nb(r) component (s', b),   m = 2 r + ri, k = 8 s' + b
//   B[k][n] = part of K_hop[(s, a)][(s', b)],           n = 32 part + 8 s + a
// (colours padded to 8).  A is the neighbour's block exactly as it lies in
// the MRHS field ([4N][Vh][nrhs], Re/Im of one RHS adjacent): one TMA box per
// 32 RHS, rows (s', b) of 128 bytes, lands it in shared memory in the
// MN-major 128-byte-swizzled operand layout, and colour rows b >= N are
// filled with zeros by the TMA bounds.  The CUDA cores touch no spinor data
// before the MMA: per hop they build B, once for all RHS of the tile, as
// signed copies of the rows Re W[a][.] and Im W[a][.] (the spin projector
// has one +-1 or +-i off-diagonal entry per row).  D accumulates the eight
// hops in tensor memory (FP32, 128 lanes x 64 columns); the epilogue forms
//   Re out = D[(r, Re)][Re K] - D[(r, Im)][Im K],
//   Im out = D[(r, Im)][Re K] + D[(r, Re)][Im K]
// with one shuffle between the two lanes of an RHS, applies xpay and the
// per-RHS a, and writes BF16 (BF16 fields are stored unscaled).
//
// Compared with the projected form (M = 2 nrhs rows of half-spinors) this
// spends twice the MMA work (K_hop has rank 2N) and saves the CUDA-core
// projection, conversion and operand stores of every spinor element; the
// tensor pipe has that work to spare.
//
// CTA = 128 threads; thread m owns TMEM lane m (= A row m) in the epilogue.
// Ring of NST stages, each the A block of one hop (two 4 KB halves of 32 RHS)
// and the hop's link box ([N*N][4 sites], 16-byte aligned site start);
// thread 0 issues the TMA NST - 1 hops ahead and refills a stage once the MMA
// that read it has committed.  B is double buffered.  Every wait is bounded;
// a timeout sets *err, the CTA agrees to stop (__syncthreads_or), drains its
// MMAs and copies in flight (bounded), frees its tensor memory and returns.
#pragma once

#include <type_traits>

#include "dslash_tc.cuh"

namespace qcu {

struct TcsDslashArgs {
  DslashArgs A;
  int rt;      // RHS per tile (<= 64)
  int chunks;  // nrhs / rt
  int ntiles;  // vh * chunks
  int halves;  // A boxes of 32 RHS per tile: 1 (rt <= 32) or 2
  int* err;    // set to 1 when a wait times out
};

namespace tcs {

constexpr uint32_t kHalfBytes = 4096;               // 4 spins x 8 colours x 128 B
constexpr uint32_t kABytes = 2 * kHalfBytes;        // M = 128 rows
constexpr uint32_t kLinkBytes = 1024;               // [N*N <= 64][4 sites] x 4 B
constexpr uint32_t kStageBytes = kABytes + kLinkBytes;  // 9 KB, keeps every A block 1024-byte aligned
constexpr uint32_t kBBytes = 4096;                  // 64 (n) x 32 (k) BF16, K-major
constexpr uint32_t kTmemCols = 64;

// offsets from the 1024-byte aligned base of dynamic shared memory
__host__ __device__ constexpr uint32_t b_off(int nst) { return (uint32_t)nst * kStageBytes; }
__host__ __device__ constexpr uint32_t w_off(int nst) { return b_off(nst) + 2 * kBBytes; }
__host__ __device__ constexpr uint32_t bar_off(int nst) { return w_off(nst) + 256; }
// + 1024 bytes to align the base
__host__ __device__ constexpr uint32_t smem_bytes(int nst) { return bar_off(nst) + 128 + 1024; }

// instruction descriptor, kind::f16: D = F32, A = B = BF16, A MN-major (bit
// 15), B K-major, N = 64, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

// A: MN-major, 128-byte swizzle (layout type 2): lbo = byte stride between the
// two 64-element MN halves, sbo = between 8-row K groups (one input spin)
__device__ __forceinline__ uint64_t a_desc(uint32_t addr) {
  return tc::smem_desc(addr, kHalfBytes, 1024) | (2ull << 61);
}
// B: K-major, no swizzle: core matrices of 8 rows x 16 B, lbo = 128 along K, sbo = 512 along N
__device__ __forceinline__ uint64_t b_desc(uint32_t addr) { return tc::smem_desc(addr, 128, 512); }

// 8 consecutive FP32 columns of this thread's lane (completion: tcgen05.wait::ld)
__device__ __forceinline__ void ld8(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
}

// 4-D tiled TMA load into shared memory, completion counted on bar
__device__ __forceinline__ void load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                        uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
      "%5}], [%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}

}  // namespace tcs

// map_in: the input field as [site][spin 4][colour N][RHS] of 4-byte complex
// BF16, box (32 RHS, 8 colours, 4 spins, 1 site), 128-byte swizzle.
// map_gauge: the gauge as [(mu, parity) 8][N*N][Vh] of 4-byte elements, box (4 sites, N*N, 1).
template <int N, int NST>
__global__ void __launch_bounds__(128)
    wilson_tcs_kernel(const __grid_constant__ TcsDslashArgs T, const __grid_constant__ CUtensorMap map_in,
                      const __grid_constant__ CUtensorMap map_gauge) {
  static_assert(N >= 2 && N <= 8, "colours are padded to 8");
  static_assert(NST >= 2 && NST <= 4, "ring stages");
  using namespace detail;
  const DslashArgs& A = T.A;
  extern __shared__ unsigned char smem_raw[];
  // 1024-byte alignment for the swizzled A blocks
  const uint32_t raw0 = tma::smem_u32(smem_raw);
  const uint32_t smem0 = (raw0 + 1023u) & ~1023u;
  unsigned char* smem = smem_raw + (smem0 - raw0);
  const uint32_t bar_mma = smem0 + tcs::bar_off(NST);  // [2]: the MMAs of hops using B buffer 0 / 1
  const uint32_t bar_ring = bar_mma + 16;               // [NST]: a stage's TMA landed
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + tcs::bar_off(NST) + 64);
  const int tid = threadIdx.x, warp = tid >> 5;

  if (tid == 0) {
    tma::mbar_init(bar_mma, 1);
    tma::mbar_init(bar_mma + 8, 1);
    for (int st = 0; st < NST; st++) tma::mbar_init(bar_ring + 8 * st, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tma::smem_u32(tmem_slot)),
                 "r"(tcs::kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tmem_slot;

  const uint32_t vh = A.geo.vh, nrhs = A.nrhs;
  const uint32_t p = A.parity;
  const bool dag = A.dagger != 0;

  // TMA producer (thread 0): global hop qq of this CTA -> stage qq % NST
  uint32_t issued = 0;
  auto issue = [&](uint32_t qq) {
    const int tile = (int)blockIdx.x + (int)(qq >> 3) * (int)gridDim.x;
    if (tile >= T.ntiles) return;
    const uint32_t st_site = (uint32_t)(tile / T.chunks), st_chunk = (uint32_t)(tile % T.chunks);
    const int d = (int)(qq & 7u);
    const uint32_t nbq = tc_neighbour(A, st_site, d);
    const bool fwd = (d & 1) == 0;
    const uint32_t lsite = fwd ? st_site : nbq, lpar = fwd ? p : 1u - p;
    const uint32_t stage = qq % NST, bar = bar_ring + 8 * stage;
    const uint32_t dst = smem0 + stage * tcs::kStageBytes;
    tma::mbar_expect_tx(bar, (uint32_t)T.halves * tcs::kHalfBytes + (uint32_t)(N * N * 16));
    for (int h = 0; h < T.halves; h++)
      tcs::load_4d(dst + (uint32_t)h * tcs::kHalfBytes, &map_in, (int)(st_chunk * T.rt) + 32 * h, 0, 0, (int)nbq,
                   bar);
    tma::load_3d(dst + tcs::kABytes, &map_gauge, (int)(lsite & ~3u), 0, (int)(2 * (d >> 1) + lpar), bar);
    issued = qq + 1;
  };
  if (tid == 0)
    for (uint32_t qq = 0; qq + 1 < (uint32_t)NST; qq++) issue(qq);

  // stage 2: this thread's two B chunks c = tid + 128 i: colour a = c & 7,
  // input spin g = (c >> 3) & 3, output spin s = (c >> 5) & 3, part = c >> 7 = i
  const uint32_t ca_ = (uint32_t)tid & 7u, cg = ((uint32_t)tid >> 3) & 3u, cs_ = ((uint32_t)tid >> 5) & 3u;
  const uint32_t boff0 = cs_ * 512u + cg * 128u + ca_ * 16u;  // (n >> 3) * 512 + g * 128 + (n & 7) * 16, part 0
  const uint32_t boff1 = boff0 + 4u * 512u;                   // part 1: n + 32

  uint32_t q = 0;  // hops done by this CTA
  bool failed = false, prod_failed = false;
  for (int tile = blockIdx.x; tile < T.ntiles && !failed; tile += gridDim.x) {
    const uint32_t site = (uint32_t)(tile / T.chunks), chunk = (uint32_t)(tile % T.chunks);

    auto hop = [&](auto dc) -> bool {
      constexpr int D = decltype(dc)::value;
      constexpr int mu = D >> 1;
      constexpr bool fwd = (D & 1) == 0;
      constexpr bool imag = gimag(mu);
      const uint32_t stage = q % NST, b = q & 1u;
      const uint32_t stage_addr = smem0 + stage * tcs::kStageBytes;
      // the hop's A block and link have landed
      bool ok = !prod_failed && tma::mbar_wait(bar_ring + 8 * stage, (q / NST) & 1u, T.err);
      uint32_t nb = 0;
      float bc = 1.f;
      if (!fwd && warp == 1) nb = tc_neighbour(A, site, D);
      if constexpr (mu == 3) {
        uint32_t rest, xh, y, z, t, rest2;
        A.geo.div_hx.divmod(site, rest, xh);
        A.geo.div_y.divmod(rest, rest2, y);
        A.geo.div_z.divmod(rest2, t, z);
        const uint32_t Lt = A.geo.L[3];
        if (A.antiperiodic_t && (fwd ? t == Lt - 1 : t == 0)) bc = -1.f;
      }
      // stage 1 (threads 32..47): rows Re W[a][.] (j < 8) and Im W[a][.] (j >= 8),
      // W[a][b] = U[a][b] (forward) or conj(U[b][a]) (backward), colours padded to 8
      if (ok && warp == 1 && tid < 48) {
        const uint32_t j = (uint32_t)tid - 32u, part = j >> 3, a = j & 7u;
        const uint32_t sidx = (fwd ? site : nb) & 3u;
        const uint32_t* lk = reinterpret_cast<const uint32_t*>(smem + stage * tcs::kStageBytes + tcs::kABytes);
        uint32_t w[8];
#pragma unroll
        for (int bb = 0; bb < 8; bb++) {
          uint32_t v = 0u;
          if (bb < N && a < (uint32_t)N) v = lk[(fwd ? a * N + bb : bb * N + a) * 4u + sidx];
          w[bb] = v;
        }
        uint32_t o[4];
        const uint32_t sel = part ? 0x7632u : 0x5410u;                  // high (Im) or low (Re) halves
        const uint32_t conj = (!fwd && part) ? 0x80008000u : 0u;        // Im of conj(U)
#pragma unroll
        for (int i = 0; i < 4; i++) o[i] = __byte_perm(w[2 * i], w[2 * i + 1], sel) ^ conj;
        *reinterpret_cast<uint4*>(smem + tcs::w_off(NST) + j * 16u) = make_uint4(o[0], o[1], o[2], o[3]);
      }
      __syncthreads();
      // B buffer b is free once the MMAs of hop q - 2 have completed
      if (ok && q >= 2) ok = tma::mbar_poll(bar_mma + 8 * b, ((q >> 1) - 1) & 1u, T.err);
      if (ok) {
        // stage 2: K_hop chunk for output spin s = cs_, input spin g = cg, colour a = ca_:
        // z = P[s][g] = bc (g = s) or bc * sg * (i if imag) (g = perm(s)) or 0
        const uint32_t perm = mu < 2 ? 3u - cs_ : (cs_ ^ 2u);
        // gsign(mu, s) for runtime s
        int gs;
        if constexpr (mu == 0) gs = cs_ < 2 ? 1 : -1;
        else if constexpr (mu == 1) gs = (cs_ == 0 || cs_ == 3) ? -1 : 1;
        else if constexpr (mu == 2) gs = (cs_ == 0 || cs_ == 3) ? 1 : -1;
        else gs = 1;
        const bool diag = cg == cs_, off = cg == perm;
        const float sg = (diag ? 1.f : (fwd ? -1.f : 1.f) * (float)gs * (dag ? -1.f : 1.f)) * bc;
        const bool zim = off && imag;
        const unsigned char* wr = smem + tcs::w_off(NST);
        unsigned char* bbuf = smem + tcs::b_off(NST) + b * tcs::kBBytes;
#pragma unroll
        for (int part = 0; part < 2; part++) {
          uint4 v = make_uint4(0u, 0u, 0u, 0u);
          if (diag || off) {
            const uint32_t src = (uint32_t)part ^ (zim ? 1u : 0u);
            // z real: sign sg on both parts; z = sg i: Re part -sg Im W, Im part +sg Re W
            const bool neg = zim ? (part == 0 ? sg > 0.f : sg < 0.f) : sg < 0.f;
            const uint32_t m = neg ? 0x80008000u : 0u;
            v = *reinterpret_cast<const uint4*>(wr + (src * 8u + ca_) * 16u);
            v.x ^= m;
            v.y ^= m;
            v.z ^= m;
            v.w ^= m;
          }
          *reinterpret_cast<uint4*>(bbuf + (part ? boff1 : boff0)) = v;
        }
      }
      tc::fence_async_smem();
      if (__syncthreads_or(!ok)) return false;
      if (tid == 0) {
        tc::fence_after();
        const uint32_t bb = smem0 + tcs::b_off(NST) + b * tcs::kBBytes;
        // K step j: input spins 2j, 2j + 1 (two 1 KB swizzle atoms of A, two 128 B core-matrix columns of B)
        tc::mma_bf16(tmem, tcs::a_desc(stage_addr), tcs::b_desc(bb), tcs::kIdesc, D > 0);
        tc::mma_bf16(tmem, tcs::a_desc(stage_addr + 2048u), tcs::b_desc(bb + 256u), tcs::kIdesc, 1u);
        tc::commit(bar_mma + 8 * b);
        // refill the stage hop q - 1 used, once its MMAs have completed (the
        // generic reads of its link box were ordered by this hop's barriers)
        if (q >= 1 && !tma::mbar_poll(bar_mma + 8 * ((q - 1) & 1u), ((q - 1) >> 1) & 1u, T.err)) {
          prod_failed = true;  // the CTA stops at the next hop's agreement
        } else {
          tc::fence_async_smem();
          issue(q + NST - 1);
        }
      }
      q++;
      return true;
    };
    failed = !(hop(std::integral_constant<int, 0>{}) && hop(std::integral_constant<int, 1>{}) &&
               hop(std::integral_constant<int, 2>{}) && hop(std::integral_constant<int, 3>{}) &&
               hop(std::integral_constant<int, 4>{}) && hop(std::integral_constant<int, 5>{}) &&
               hop(std::integral_constant<int, 6>{}) && hop(std::integral_constant<int, 7>{}));
    if (failed) break;

    // the commit of the last hop covers all MMAs of this tile
    const uint32_t ql = q - 1;
    const bool ok = tma::mbar_poll(bar_mma + 8 * (ql & 1u), (ql >> 1) & 1u, T.err);
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    tc::fence_after();

    // epilogue, one output spin at a time: lane m = 2 r + ri holds part ri of
    // RHS r; Re (ri = 0) = Re K - partner's Im K, Im (ri = 1) = Re K + partner's Im K
    const uint32_t r = (uint32_t)tid >> 1, ri = (uint32_t)tid & 1u;
    const uint32_t rhs = chunk * (uint32_t)T.rt + r;
    const bool live = r < (uint32_t)T.rt && (!A.mask || A.mask[rhs] != 0);
    const float ca = live ? (A.a_rhs_f ? A.a_rhs_f[rhs] : A.af) : 0.f;
    const __nv_bfloat16* __restrict__ xin = static_cast<const __nv_bfloat16*>(A.x);
    __nv_bfloat16* __restrict__ out = static_cast<__nv_bfloat16*>(A.out);
    const uint32_t cs = vh * nrhs;
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
    for (int s = 0; s < 4; s++) {
      uint32_t re_k[8], im_k[8];
      tcs::ld8(lane_addr + 8u * s, re_k);
      tcs::ld8(lane_addr + 32u + 8u * s, im_k);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int a = 0; a < N; a++) {
        const float other = __shfl_xor_sync(0xffffffffu, __uint_as_float(im_k[a]), 1);
        const float own = __uint_as_float(re_k[a]);
        float val = ca * (ri ? own + other : own - other);
        if (live) {
          const uint32_t idx = 2u * ((uint32_t)(s * N + a) * cs + site * nrhs + rhs) + ri;
          if (xin) val = fmaf(A.bf, __bfloat162float(xin[idx]), val);
          out[idx] = __float2bfloat16_rn(val);
        }
      }
    }
    tc::fence_before();
  }

  if (failed && tid == 0 && q > 0) {
    // let the MMAs in flight finish before the tensor memory is released (bounded)
    const uint32_t ql = q - 1;
    tma::mbar_poll(bar_mma + 8 * (ql & 1u), (ql >> 1) & 1u, T.err);
  }
  // copies still in flight land before the CTA's shared memory is released (bounded)
  if (failed && tid == 0)
    for (uint32_t qq = q; qq < issued; qq++) tma::mbar_poll(bar_ring + 8 * (qq % NST), (qq / NST) & 1u, T.err);
  tc::fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tcs::kTmemCols) : "memory");
}

}  // namespace qcu
