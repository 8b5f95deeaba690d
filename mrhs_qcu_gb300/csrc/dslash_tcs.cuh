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
// Persistent, warp-specialized CTA of 320 threads; the roles hand work to
// each other through mbarriers only:
//   warps 0-3  B builders: per hop, the 4 KB B operand into a ring of NB
//              buffers, each thread two 16-byte chunks: signed copies of one
//              link row of the tile's link record.  They never read the A
//              stage, so a hop's build overlaps the copy of its neighbour
//              block instead of following it; only the MMA waits for both
//              (waiting for the copy as well put the copy latency and the
//              build in series: about 15% slower at nrhs 64)
//   warp 4     MMA issuer (one thread): two MMAs per hop into one of two
//              tensor-memory accumulators; commits free the B buffer and the
//              TMA stage, and hand a finished tile to the epilogue
//   warp 5     TMA producer (one thread): per hop, the neighbour's A block
//              (one box, or two of 32 RHS) into a ring of NST stages, as far
//              ahead as the ring allows; with each tile's first hop, the next
//              tile's link record (one 2 KB bulk copy, layout.h
//              gauge_tc_records_bf16) into one of three record slots
//   warps 6-9  epilogue: tensor memory -> Re/Im combination -> global, one
//              tile behind the MMAs (double-buffered accumulator)
// Every wait is bounded (about 1 s); a timeout sets *err and a shared abort
// flag that every other wait checks, so all roles leave their loops; the
// MMA issuer then waits (bounded) for its MMAs, the producer for its copies,
// and the CTA frees its tensor memory and returns.
#pragma once

#include <type_traits>

#include "dslash_tc.cuh"

namespace qcu {

struct TcsDslashArgs {
  DslashArgs A;
  int rt;      // RHS per tile (<= 64)
  int chunks;  // nrhs / rt
  int ntiles;  // vh * chunks
  int halves;  // A halves of 32 RHS per tile: 1 (rt <= 32) or 2
  int fused;   // 1: the tensor map is 5-D and one box brings both halves (nrhs a multiple of 32)
  int* err;    // set to 1 when a wait times out
  // complex-element strides of the output and xpay fields between components
  // and between sites (component- or site-major layout)
  uint32_t cstr, sstr;
};

namespace tcs {

constexpr uint32_t kHalfBytes = 4096;               // 4 spins x 8 colours x 128 B (32 RHS)
constexpr uint32_t kRecBytes = 2048;                // a site's eight links in row form (layout.h kTcRecordBytes)
constexpr uint32_t kBBytes = 4096;                  // 64 (n) x 32 (k) BF16, K-major
constexpr uint32_t kTmemCols = 128;  // two accumulators of 64 columns
// A stage holds HV A halves of 32 RHS (M rows 64 h .. 64 h + 63).  With
// HV = 1 (tiles of at most 32 RHS) the MMA's rows 64-127 read the 4 KB after
// the half, whatever lies there: their accumulator lanes are never stored,
// and the read stays inside the CTA's shared memory (the link records and
// the B buffers follow the last stage).
__host__ __device__ constexpr uint32_t stage_bytes(int hv) { return (uint32_t)hv * kHalfBytes; }

// Link records: tile k of a CTA uses slot k % 3, fetched during tile k - 1.
// Slot k % 3 was last read in tile k - 3, which the builders have finished
// when the producer, at the first hop of tile k - 1, has seen the MMAs of a
// hop of tile k - 2 complete (rings of at most 8 stages).
constexpr int kRecSlots = 3;
// offsets from the 1024-byte aligned base of dynamic shared memory: TMA
// stages, link records, B buffers, barriers
__host__ __device__ constexpr uint32_t rec_off(int nst, int hv) { return (uint32_t)nst * stage_bytes(hv); }
__host__ __device__ constexpr uint32_t b_off(int nst, int hv) { return rec_off(nst, hv) + kRecSlots * kRecBytes; }
__host__ __device__ constexpr uint32_t bar_off(int nst, int nb, int hv) { return b_off(nst, hv) + (uint32_t)nb * kBBytes; }
// barriers: ring_full[nst], ring_empty[nst], b_full[nb], b_empty[nb],
// tmem_full[2], tmem_empty[2], drain, rec_full[3]; then the tensor-memory slot and the abort flag
__host__ __device__ constexpr uint32_t slot_off(int nst, int nb, int hv) {
  return bar_off(nst, nb, hv) + 8u * (2 * nst + 2 * nb + 5 + kRecSlots);
}
// + 1024 bytes to align the base
__host__ __device__ constexpr uint32_t smem_bytes(int nst, int nb, int hv) { return slot_off(nst, nb, hv) + 16 + 1024; }
constexpr int kThreads = 320;
// epilogue warps with accumulator rows to store: warp w holds rows 32 w .. 32 w + 31,
// RHS 16 w .. 16 w + 15 of the tile; the others leave at once
__host__ __device__ constexpr uint32_t epilogue_warps(int rt) { return (uint32_t)(rt + 15) / 16u; }

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

// L2 policy that keeps lines resident (each neighbour block is read by the
// eight sites around it, a short while apart)
__device__ __forceinline__ uint64_t evict_last_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
// L2 policy for data read once (the link records): evicted first, so that it
// does not displace the neighbour blocks that are read again
__device__ __forceinline__ uint64_t evict_first_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

// 1-D bulk copy global -> shared with an L2 cache policy (16-byte aligned,
// size a multiple of 16), completion counted on bar
__device__ __forceinline__ void bulk_load_hint(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar,
                                               uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(bar), "l"(policy)
      : "memory");
}

// 5-D tiled TMA load into shared memory with an L2 cache policy, completion counted on bar
__device__ __forceinline__ void load_5d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, int c4,
                                        uint32_t bar, uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, "
      "{%2, %3, %4, %5, %6}], [%7], %8;" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar), "l"(policy)
      : "memory");
}

// 4-D tiled TMA load into shared memory with an L2 cache policy, completion counted on bar
__device__ __forceinline__ void load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                        uint32_t bar, uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, "
      "{%2, %3, %4, %5}], [%6], %7;" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar), "l"(policy)
      : "memory");
}

// Bounded wait for the phase of `bar` with the given parity that also gives
// up when another role has set the CTA's abort flag; a timeout (about 1 s)
// sets *err and the abort flag.  Waiting threads are suspended in try_wait
// (suspend-time hint) rather than spinning.
__device__ __forceinline__ bool wait(uint32_t bar, uint32_t parity, int* err, volatile int* abort_flag) {
  uint32_t ok = 0;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  if (ok) return true;
  const uint64_t t0 = tma::now_ns();
  for (uint32_t i = 1;; i++) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(20000u)
        : "memory");
    if (ok) return true;
    if (*abort_flag) return false;
    if ((i & 15u) == 0 && tma::now_ns() - t0 > 1000000000ull) {
      atomicExch(err, 1);
      *abort_flag = 1;
      return false;
    }
  }
}

// The same bounded wait for roles off the critical path: the epilogue waits
// a whole tile for its accumulator and the producer runs a ring ahead of the
// MMAs.  Between polls the warp sleeps (64 ns doubling to 1 us), so it takes
// no issue slots from the builders and the MMA issuer, which poll.
__device__ __forceinline__ bool wait_sleep(uint32_t bar, uint32_t parity, int* err, volatile int* abort_flag) {
  uint32_t ok = 0;
  const uint64_t t0 = tma::now_ns();
  uint32_t ns = 64;
  for (uint32_t i = 1;; i++) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (*abort_flag) return false;
    __nanosleep(ns);
    ns = ns < 1024u ? 2u * ns : 1024u;
    if ((i & 15u) == 0 && tma::now_ns() - t0 > 1000000000ull) {
      atomicExch(err, 1);
      *abort_flag = 1;
      return false;
    }
  }
}

}  // namespace tcs

// map_in: the input field as [site][spin 4][colour N][RHS] of 4-byte complex
// BF16 (strides of either layout), box (32 RHS, 8 colours, 4 spins, 1 site),
// 128-byte swizzle; or, when the RHS count is a multiple of 32 and a tile
// holds 64 RHS (T.fused), as [site][half][spin][colour][RHS 32] with box
// (32, 8, 4, 2, 1), which lands a tile's two halves in one copy.  In the
// site-major layout a box is one contiguous run of the field; in the
// component-major one it gathers rows of 128 bytes from arrays Vh x nrhs x 4
// bytes apart, which the copy engine serves at about half the rate.  The
// links come from A.gauge_tc: one 2 KB record per site (its eight links in
// row form), one bulk copy per tile, a tile ahead.
template <int N, int NST, int NB, int HV>
__global__ void __launch_bounds__(tcs::kThreads, 4)
    wilson_tcs_kernel(const __grid_constant__ TcsDslashArgs T, const __grid_constant__ CUtensorMap map_in) {
  static_assert(N >= 2 && N <= 8, "colours are padded to 8");
  static_assert(NST >= 2 && NST <= 8 && NB >= 2 && NB <= 4, "ring depths");
  static_assert(HV == 1 || HV == 2, "A halves per stage");
  constexpr uint32_t kStage = tcs::stage_bytes(HV);
  using namespace detail;
  const DslashArgs& A = T.A;
  extern __shared__ unsigned char smem_raw[];
  // 1024-byte alignment for the swizzled A blocks
  const uint32_t raw0 = tma::smem_u32(smem_raw);
  const uint32_t smem0 = (raw0 + 1023u) & ~1023u;
  unsigned char* smem = smem_raw + (smem0 - raw0);
  const uint32_t ring_full = smem0 + tcs::bar_off(NST, NB, HV);
  const uint32_t ring_empty = ring_full + 8 * NST;
  const uint32_t b_full = ring_empty + 8 * NST;
  const uint32_t b_empty = b_full + 8 * NB;
  const uint32_t tmem_full = b_empty + 8 * NB;
  const uint32_t tmem_empty = tmem_full + 16;
  const uint32_t drain = tmem_empty + 16;
  const uint32_t rec_full = drain + 8;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + tcs::slot_off(NST, NB, HV));
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + tcs::slot_off(NST, NB, HV) + 8);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    for (int i = 0; i < NST; i++) {
      tma::mbar_init(ring_full + 8 * i, 1);
      tma::mbar_init(ring_empty + 8 * i, 1);
    }
    for (int i = 0; i < NB; i++) {
      tma::mbar_init(b_full + 8 * i, 128);
      tma::mbar_init(b_empty + 8 * i, 1);
    }
    for (int i = 0; i < 2; i++) {
      tma::mbar_init(tmem_full + 8 * i, 1);
      tma::mbar_init(tmem_empty + 8 * i, 32 * tcs::epilogue_warps(T.rt));
    }
    tma::mbar_init(drain, 1);
    for (int i = 0; i < tcs::kRecSlots; i++) tma::mbar_init(rec_full + 8 * i, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 4) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tma::smem_u32(tmem_slot)),
                 "r"(tcs::kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t p = A.parity;
  const int ntiles = T.ntiles;

  if (warp < 4) {
    // ---- B builders --------------------------------------------------------
    // stage 2 assignment: chunks c = tid + 128 i: colour a = c & 7, input spin
    // g = (c >> 3) & 3, output spin s = (c >> 5) & 3, part = c >> 7 = i
    const uint32_t ca_ = (uint32_t)tid & 7u, cg = ((uint32_t)tid >> 3) & 3u, cs_ = ((uint32_t)tid >> 5) & 3u;
    const uint32_t boff0 = cs_ * 512u + cg * 128u + ca_ * 16u;  // (n >> 3) * 512 + g * 128 + (n & 7) * 16
    const uint32_t boff1 = boff0 + 4u * 512u;                   // part 1: n + 32
    const bool dag = A.dagger != 0;
    uint32_t q = 0;
    bool stop = false;
    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles && !stop; tile += gridDim.x, it++) {
      const uint32_t site = (uint32_t)(tile / T.chunks);
      const uint32_t t_coord = EoSite(A.geo, site).t;
      auto hop = [&](auto dc) -> bool {
        constexpr int D = decltype(dc)::value;
        constexpr int mu = D >> 1;
        constexpr bool fwd = (D & 1) == 0;
        constexpr bool imag = gimag(mu);
        const uint32_t b = q % NB;
        // B buffer b is free once the MMAs of hop q - NB have completed; the
        // tile's link record is in place before its first hop is built.  The
        // builders never read the A stage, so the build of a hop overlaps the
        // copy of its neighbour block (the MMA issuer waits for both).
        bool ok = true;
        if (q >= NB) ok = tcs::wait(b_empty + 8 * b, ((q / NB) - 1) & 1u, T.err, abort_flag);
        if (D == 0 && ok) ok = tcs::wait(rec_full + 8 * (it % tcs::kRecSlots), (it / tcs::kRecSlots) & 1u, T.err, abort_flag);
        if (!ok) return false;
        // stage 2: K_hop chunk for output spin s = cs_, input spin g = cg, colour a = ca_:
        // z = P[s][g] = bc (g = s) or bc * sg * (i if imag) (g = perm(s)) or 0
        float bc = 1.f;
        if constexpr (mu == 3) {
          const uint32_t Lt = A.geo.L[3];
          if (A.antiperiodic_t && (fwd ? t_coord == Lt - 1 : t_coord == 0)) bc = -1.f;
        }
        const uint32_t perm = mu < 2 ? 3u - cs_ : (cs_ ^ 2u);
        int gs;  // gsign(mu, s) for runtime s
        if constexpr (mu == 0) gs = cs_ < 2 ? 1 : -1;
        else if constexpr (mu == 1) gs = (cs_ == 0 || cs_ == 3) ? -1 : 1;
        else if constexpr (mu == 2) gs = (cs_ == 0 || cs_ == 3) ? 1 : -1;
        else gs = 1;
        const bool diag = cg == cs_, off = cg == perm;
        const float sg = (diag ? 1.f : (fwd ? -1.f : 1.f) * (float)gs * (dag ? -1.f : 1.f)) * bc;
        const bool zim = off && imag;
        // the hop's link in the tile's record (which arrived with hop 0): row
        // (part, a) of W = U (forward) or of U^T (backward, whose conjugation
        // flips the sign of the Im part)
        const unsigned char* wr =
            smem + tcs::rec_off(NST, HV) + (uint32_t)(it % tcs::kRecSlots) * tcs::kRecBytes + D * 256u;
        unsigned char* bbuf = smem + tcs::b_off(NST, HV) + b * tcs::kBBytes;
#pragma unroll
        for (int part = 0; part < 2; part++) {
          uint4 v = make_uint4(0u, 0u, 0u, 0u);
          if (diag || off) {
            const uint32_t src = (uint32_t)part ^ (zim ? 1u : 0u);
            // z real: sign sg on both parts; z = sg i: Re part -sg Im W, Im part +sg Re W
            const bool neg = (zim ? (part == 0 ? sg > 0.f : sg < 0.f) : sg < 0.f) != (!fwd && src == 1u);
            const uint32_t m = neg ? 0x80008000u : 0u;
            v = *reinterpret_cast<const uint4*>(wr + (src * 8u + ca_) * 16u);
            v.x ^= m;
            v.y ^= m;
            v.z ^= m;
            v.w ^= m;
          }
          *reinterpret_cast<uint4*>(bbuf + (part ? boff1 : boff0)) = v;
        }
        // the tensor core reads B, and the producer refills the stage, only
        // after every builder's generic accesses
        tc::fence_async_smem();
        tma::mbar_arrive(b_full + 8 * b);
        q++;
        return true;
      };
      stop = !(hop(std::integral_constant<int, 0>{}) && hop(std::integral_constant<int, 1>{}) &&
               hop(std::integral_constant<int, 2>{}) && hop(std::integral_constant<int, 3>{}) &&
               hop(std::integral_constant<int, 4>{}) && hop(std::integral_constant<int, 5>{}) &&
               hop(std::integral_constant<int, 6>{}) && hop(std::integral_constant<int, 7>{}));
    }
  } else if (warp == 4) {
    // ---- MMA issuer ----------------------------------------------------------
    if (lane == 0) {
      uint32_t q = 0;
      bool ok = true;
      int it = 0;
      for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, it++) {
        const uint32_t acc = (uint32_t)it & 1u;
        // the epilogue has read this accumulator's previous tile
        if (it >= 2) ok = tcs::wait(tmem_empty + 8 * acc, (((uint32_t)it >> 1) - 1) & 1u, T.err, abort_flag);
        tc::fence_after();
        for (int h = 0; h < 8 && ok; h++, q++) {
          const uint32_t st = q % NST, b = q % NB;
          ok = tcs::wait(b_full + 8 * b, (q / NB) & 1u, T.err, abort_flag) &&
               tcs::wait(ring_full + 8 * st, (q / NST) & 1u, T.err, abort_flag);
          if (!ok) break;
          tc::fence_after();
          const uint32_t sa = smem0 + st * kStage;
          const uint32_t sb = smem0 + tcs::b_off(NST, HV) + b * tcs::kBBytes;
          const uint32_t d = tmem + acc * 64u;
          // K step j: input spins 2j, 2j + 1 (two 1 KB swizzle atoms of A, two 128 B core-matrix columns of B)
          tc::mma_bf16(d, tcs::a_desc(sa), tcs::b_desc(sb), tcs::kIdesc, h > 0);
          tc::mma_bf16(d, tcs::a_desc(sa + 2048u), tcs::b_desc(sb + 256u), tcs::kIdesc, 1u);
          tc::commit(b_empty + 8 * b);
          tc::commit(ring_empty + 8 * st);
        }
        if (ok) tc::commit(tmem_full + 8 * acc);
      }
      // every MMA issued has completed before the tensor memory is released (bounded)
      tc::commit(drain);
      tma::mbar_wait(drain, 0, T.err);
    }
  } else if (warp == 5) {
    // ---- TMA producer --------------------------------------------------------
    if (lane == 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&map_in)) : "memory");
      const unsigned char* gtc = static_cast<const unsigned char*>(A.gauge_tc);
      const uint32_t vh = A.geo.vh;
      const uint32_t tx = (uint32_t)T.halves * tcs::kHalfBytes;
      const uint64_t keep = tcs::evict_last_policy(), once = tcs::evict_first_policy();
      uint32_t qq = 0;
      bool ok = true;
      int it = 0;
      // link record of tile `it` (its site's eight links, 2 KB) into slot it % 3
      auto fetch_record = [&](int tile_r, int it_r) {
        const uint32_t bar = rec_full + 8 * (it_r % tcs::kRecSlots);
        tma::mbar_expect_tx(bar, tcs::kRecBytes);
        tcs::bulk_load_hint(smem0 + tcs::rec_off(NST, HV) + (uint32_t)(it_r % tcs::kRecSlots) * tcs::kRecBytes,
                            gtc + ((uint64_t)p * vh + (uint32_t)(tile_r / T.chunks)) * tcs::kRecBytes, tcs::kRecBytes,
                            bar, once);
      };
      int fetched = 0;  // records issued
      if ((int)blockIdx.x < ntiles) {
        fetch_record(blockIdx.x, 0);
        fetched = 1;
      }
      for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, it++) {
        const uint32_t st_site = (uint32_t)(tile / T.chunks), st_chunk = (uint32_t)(tile % T.chunks);
        const EoSite sc(A.geo, st_site);
#pragma unroll
        for (int d = 0; d < 8; d++, qq++) {
          const uint32_t st = qq % NST;
          // stage st is free once the MMAs of hop qq - NST have completed
          if (qq >= (uint32_t)NST && !tcs::wait_sleep(ring_empty + 8 * st, ((qq / NST) - 1) & 1u, T.err, abort_flag)) {
            ok = false;
            break;
          }
          // with the tile's first hop, the next tile's link record
          if (d == 0 && tile < ntiles - (int)gridDim.x) {
            fetch_record(tile + (int)gridDim.x, it + 1);
            fetched++;
          }
          const uint32_t nbq = sc.nb(A.geo, p, d);
          const uint32_t bar = ring_full + 8 * st, dst = smem0 + st * kStage;
          tma::mbar_expect_tx(bar, tx);
          if (T.fused)
            tcs::load_5d(dst, &map_in, 0, 0, 0, 2 * (int)st_chunk, (int)nbq, bar, keep);
          else
            for (int h = 0; h < T.halves; h++)
              tcs::load_4d(dst + (uint32_t)h * tcs::kHalfBytes, &map_in, (int)(st_chunk * T.rt) + 32 * h, 0, 0,
                           (int)nbq, bar, keep);
        }
      }
      // copies still in flight land before the CTA's shared memory is released (bounded):
      // the last hop issued into each stage
      for (uint32_t k = 0; k < (uint32_t)NST && k < qq; k++) {
        const uint32_t last = qq - 1 - k;
        tma::mbar_wait(ring_full + 8 * (last % NST), (last / NST) & 1u, T.err);
      }
      // and the last record issued into each slot
      for (int k = 0; k < tcs::kRecSlots && k < fetched; k++) {
        const int last = fetched - 1 - k;
        tma::mbar_wait(rec_full + 8 * (last % tcs::kRecSlots), (last / tcs::kRecSlots) & 1u, T.err);
      }
    }
  } else {
    // ---- epilogue (warps 6-9: lane quarter warp % 4) ---------------------------
    const uint32_t lq = (uint32_t)warp & 3u;
    const uint32_t m = lq * 32u + (uint32_t)lane;
    const uint32_t r = m >> 1, ri = m & 1u;
    const uint32_t cstr = T.cstr, sstr = T.sstr;
    const __nv_bfloat16* __restrict__ xin = static_cast<const __nv_bfloat16*>(A.x);
    __nv_bfloat16* __restrict__ out = static_cast<__nv_bfloat16*>(A.out);
    int it = 0;
    // warps whose 32 accumulator lanes are all padding rows (tiles of at most
    // 32 RHS) have nothing to read and take no part in the hand-off
    const int first = lq < tcs::epilogue_warps(T.rt) ? (int)blockIdx.x : ntiles;
    for (int tile = first; tile < ntiles; tile += gridDim.x, it++) {
      const uint32_t site = (uint32_t)(tile / T.chunks), chunk = (uint32_t)(tile % T.chunks);
      const uint32_t rhs = chunk * (uint32_t)T.rt + r;
      const bool live = r < (uint32_t)T.rt && (!A.mask || A.mask[rhs] != 0);
      const float ca = live ? (A.a_rhs_f ? A.a_rhs_f[rhs] : A.af) : 0.f;
      const uint32_t acc = (uint32_t)it & 1u;
      if (!tcs::wait_sleep(tmem_full + 8 * acc, ((uint32_t)it >> 1) & 1u, T.err, abort_flag)) break;
      tc::fence_after();
      const uint32_t lane_addr = tmem + ((lq * 32u) << 16) + acc * 64u;
      // Re (ri = 0) = Re K - partner's Im K, Im (ri = 1) = Re K + partner's Im K;
      // component k of this lane's output at o + k * step (BF16 halves)
      const uint32_t o = 2u * (site * sstr + rhs) + ri, step = 2u * cstr;
      unsigned short* const op = reinterpret_cast<unsigned short*>(out) + o;
      const unsigned short* const xp = xin ? reinterpret_cast<const unsigned short*>(xin) + o : nullptr;
      const float sgn = ri ? 1.f : -1.f, bfx = A.bf;
#pragma unroll
      for (int s = 0; s < 4; s++) {
        uint32_t re_k[8], im_k[8];
        tcs::ld8(lane_addr + 8u * s, re_k);
        tcs::ld8(lane_addr + 32u + 8u * s, im_k);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (s == 3) {
          // the accumulator is free for the tile after next once all its columns are read
          tc::fence_before();
          tma::mbar_arrive(tmem_empty + 8 * acc);
        }
        float val[N];
#pragma unroll
        for (int a = 0; a < N; a++) {
          const float other = __shfl_xor_sync(0xffffffffu, __uint_as_float(im_k[a]), 1);
          val[a] = ca * fmaf(sgn, other, __uint_as_float(re_k[a]));  // ca (own -+ other), one rounding each
        }
        if (live) {
          // streaming stores: the output is not re-read by this launch
          if (xp) {
#pragma unroll
            for (int a = 0; a < N; a++) {
              const uint32_t k = (uint32_t)(s * N + a) * step;
              const float x = __bfloat162float(__ushort_as_bfloat16(xp[k]));
              __stcs(op + k, __bfloat16_as_ushort(__float2bfloat16_rn(fmaf(bfx, x, val[a]))));
            }
          } else {
#pragma unroll
            for (int a = 0; a < N; a++)
              __stcs(op + (uint32_t)(s * N + a) * step, __bfloat16_as_ushort(__float2bfloat16_rn(val[a])));
          }
        }
      }
    }
  }

  tc::fence_before();
  __syncthreads();
  if (warp == 4)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tcs::kTmemCols) : "memory");
}

}  // namespace qcu
