// The register kernel with its links staged through TMA into shared memory.
//
// One CTA = one x-row of output sites (hx = X/2 consecutive even-odd sites at
// fixed y, z, t) x all nrhs RHS (hx * G threads, G = nrhs / R).  Every hop's
// links for the whole row lie in one row of the gauge: forward hops at the
// output row itself, backward hops at the neighbour row (the own row, other
// parity, for x; the y-1, z-1, t-1 row, wrapped, for the others).  So at CTA
// start one thread issues eight tensor copies, one [NN][hx] box per hop (for
// two-row links, out of the row's group of 32 sites), each
// completing on its own mbarrier, and every thread waits only for the hop it
// is about to compute: the links are read from DRAM once per CTA, shared by
// all nrhs RHS of the row from shared memory, and never occupy L1 or
// registers while in flight.  The arithmetic is hop_pk's (packed FP32x2 over
// RHS pairs), operation for operation, so results are bit-identical to the
// register kernel of the same R and link form.
//
// Every wait is bounded (about one second, 10 ms once any CTA timed out;
// then *err is set and the host reports QCU_ERR_DEVICE_TIMEOUT).  No thread
// leaves while a copy of its CTA may be in flight: every thread waits on all
// eight barriers, and a thread whose wait ran out waits once more on each
// (bounded) before it returns.
#pragma once

#include "dslash_tma.h"

namespace qcu {

template <int P, int N, int R, int MINB, bool RC>
__global__ void __maxnreg__(RegCap<MINB>::regs)
    wilson_tmalink_kernel(const DslashArgs A, const __grid_constant__ CUtensorMap gmap, int* err) {
  using S = Store<P>;
  using E = typename S::elem;
  using namespace detail;
  constexpr uint32_t NN = RC ? (N - 1) * N : N * N;  // stored components per link
  extern __shared__ __align__(128) unsigned char smem[];
  const uint32_t hx = A.geo.hx, Ly = A.geo.L[1], Lz = A.geo.L[2], Lt = A.geo.L[3];
  const uint32_t hop_bytes = NN * hx * (uint32_t)sizeof(E);  // one hop's links: [NN][hx]
  const uint32_t hop_stride = (hop_bytes + 127u) & ~127u;     // each hop's box 128-byte aligned
  const uint32_t bar0 = tma::smem_u32(smem + 8 * hop_stride);
  const uint32_t row = blockIdx.x;
  uint32_t y, zt, z, t;
  A.geo.div_y.divmod(row, zt, y);
  A.geo.div_z.divmod(zt, t, z);
  const uint32_t p = A.parity;

  if (threadIdx.x == 0) {
    for (int h = 0; h < 8; h++) tma::mbar_init(bar0 + 8 * h, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t ym = (y == 0 ? Ly - 1 : y - 1), zm = (z == 0 ? Lz - 1 : z - 1), tm = (t == 0 ? Lt - 1 : t - 1);
    const uint32_t back_row[4] = {row, (t * Lz + z) * Ly + ym, (t * Lz + zm) * Ly + y, (tm * Lz + z) * Ly + y};
    for (int h = 0; h < 8; h++) {
      const uint32_t mu = h >> 1;
      const bool fwd = (h & 1) == 0;
      tma::mbar_expect_tx(bar0 + 8 * h, hop_bytes);
      // box {hx sites, NN components, 1}, x in 4-byte units: full links at (row start, 0,
      // 2 mu + parity); two-row links at (row start within its group of 32 sites, 0, group
      // index over all (mu, parity) blocks)
      const uint32_t lrow = fwd ? row : back_row[mu], blk = 2 * mu + (fwd ? p : 1u - p);
      if constexpr (RC)
        tma::load_3d(tma::smem_u32(smem + h * hop_stride), &gmap, (int)(((lrow * hx) & 31u) * (sizeof(E) / 4)), 0,
                     (int)(blk * (two_row_vh(A.geo.vh) >> 5) + ((lrow * hx) >> 5)), bar0 + 8 * h);
      else
        tma::load_3d(tma::smem_u32(smem + h * hop_stride), &gmap, (int)(lrow * hx * (sizeof(E) / 4)), 0, (int)blk,
                     bar0 + 8 * h);
    }
  }
  // after a timeout anywhere in the launch, later CTAs wait 10 ms instead of
  // one second, so a launch whose copies never land ends in seconds
  const uint64_t lim = *reinterpret_cast<volatile int*>(err) ? 10000000ull : 1000000000ull;

  uint32_t xh, grp;
  A.div_groups.divmod(threadIdx.x, xh, grp);
  const uint32_t site = row * hx + xh;
  const uint32_t rhs0 = grp * R;
  bool active = true;
  if (A.mask) {
    active = false;
#pragma unroll
    for (int r = 0; r < R; r++) active |= A.mask[rhs0 + r] != 0;
  }
  auto drain = [&]() {  // a wait ran out: wait (bounded) for every copy before leaving
    for (int h = 0; h < 8; h++) tma::mbar_wait(bar0 + 8 * h, 0, err, lim);
  };
  if (!active) {
    for (int h = 0; h < 8; h++)
      if (!tma::mbar_wait(bar0 + 8 * h, 0, err, lim)) return drain();
    return;
  }

  const uint32_t hx1 = hx - 1, pl = A.geo.plane, cb = A.geo.cube;
  const uint32_t eo = (y + z + t) & 1u;
  const bool top = t == Lt - 1, bot = t == 0;
  const float f = A.dagger ? -1.f : 1.f;
  const E* __restrict__ in = static_cast<const E*>(A.in);
  // neighbour site and the link's place in its staged row, per hop
  const uint32_t nbx_f = (eo != p) ? (xh == hx1 ? site - hx1 : site + 1) : site;
  const uint32_t nbx_b = (eo == p) ? (xh == 0 ? site + hx1 : site - 1) : site;
  const uint32_t nb[8] = {nbx_f,
                          nbx_b,
                          (y == Ly - 1) ? site - (Ly - 1) * hx : site + hx,
                          (y == 0) ? site + (Ly - 1) * hx : site - hx,
                          (z == Lz - 1) ? site - (Lz - 1) * pl : site + pl,
                          (z == 0) ? site + (Lz - 1) * pl : site - pl,
                          top ? site - (Lt - 1) * cb : site + cb,
                          bot ? site + (Lt - 1) * cb : site - cb};
  // the backward x link is at the x-neighbour in the own row; every other link at the thread's xh
  // (byte offsets in the staged [NN][hx] row)
  constexpr uint32_t LB = (uint32_t)sizeof(E);
  const uint32_t lx[8] = {xh * LB, (nbx_b - row * hx) * LB, xh * LB, xh * LB, xh * LB, xh * LB, xh * LB, xh * LB};
  const uint32_t ls_bytes = hx * (uint32_t)sizeof(E);
  const float bcf = (A.antiperiodic_t && top) ? -1.f : 1.f;
  const float bcb = (A.antiperiodic_t && bot) ? -1.f : 1.f;

  float2 re[4][N][R / 2], im[4][N][R / 2];
#pragma unroll
  for (int s = 0; s < 4; s++)
#pragma unroll
    for (int a = 0; a < N; a++)
#pragma unroll
      for (int q = 0; q < R / 2; q++) re[s][a][q] = im[s][a][q] = make_float2(0.f, 0.f);

#define QCU_TMALINK_HOP(H, MU, FWD, BC)                                                                          \
  if (!tma::mbar_wait(bar0 + 8 * (H), 0, err, lim)) return drain();                                             \
  hop_pk<P, N, R, MU, FWD, RC, true>(re, im, A, in,                                                             \
                                     reinterpret_cast<const char*>(smem + (H) * hop_stride) + lx[H],             \
                                     ls_bytes, nb[H], rhs0, BC, f);
  QCU_TMALINK_HOP(0, 0, true, 1.f)
  QCU_TMALINK_HOP(1, 0, false, 1.f)
  QCU_TMALINK_HOP(2, 1, true, 1.f)
  QCU_TMALINK_HOP(3, 1, false, 1.f)
  QCU_TMALINK_HOP(4, 2, true, 1.f)
  QCU_TMALINK_HOP(5, 2, false, 1.f)
  QCU_TMALINK_HOP(6, 3, true, bcf)
  QCU_TMALINK_HOP(7, 3, false, bcb)
#undef QCU_TMALINK_HOP

  C2<float> acc[4][N][R];
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
  store_out<P, N, R>(acc, A, site, rhs0);
}

// Launch over Vh / hx rows of hx * nrhs / R threads; the block argument of
// the registry signature is not used (the CTA is one row).

template <int P, int N, int R, int MINB, bool PK, bool RC>
void launch_wilson_tmalink(const DslashArgs& A, int /*block*/, cudaStream_t st) {
  static_assert(PK, "the link-staged kernel uses the packed arithmetic");
  using E = typename Store<P>::elem;
  constexpr int NN = RC ? (N - 1) * N : N * N;
  QCU_REQUIRE(tmalink_runs(A, R, (int)sizeof(E), NN), QCU_ERR_UNSUPPORTED,
              "link-staged dslash: arguments outside the kernel's limits");
  CUtensorMap mg;
  if constexpr (RC)
    tma_encode_gauge_groups(&mg, A.gauge12, (int)sizeof(E), (int)detail::two_row_vh(A.geo.vh), A.geo.hx);
  else
    tma_encode_gauge(&mg, A.gauge, (int)sizeof(E), A.geo.vh, NN, A.geo.hx);
  const size_t smem = tmalink_smem_bytes(NN, A.geo.hx, (int)sizeof(E));
  const void* k = reinterpret_cast<const void*>(&wilson_tmalink_kernel<P, N, R, MINB, RC>);
  static size_t smem_set = 48 * 1024;  // the attribute only grows; set outside graph capture by the first launch
  if (smem > smem_set) {
    QCU_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    smem_set = smem;
  }
  const int rows = A.geo.vh / A.geo.hx;
  const int threads = A.geo.hx * (A.nrhs / R);
  static int max_threads = 0;
  if (!max_threads) {
    cudaFuncAttributes fa;
    QCU_CHECK_CUDA(cudaFuncGetAttributes(&fa, k));
    max_threads = fa.maxThreadsPerBlock;
  }
  QCU_REQUIRE(threads <= max_threads, QCU_ERR_UNSUPPORTED, "link-staged dslash: row too long for one CTA");
  wilson_tmalink_kernel<P, N, R, MINB, RC><<<rows, threads, smem, st>>>(A, mg, tma_error_flag());
  tma_note_launch();
}

}  // namespace qcu
