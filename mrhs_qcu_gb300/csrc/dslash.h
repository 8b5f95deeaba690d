// Dslash dispatch: runtime (precision, N, RHS per thread) -> kernel instance.
// This is the GB300 counterpart of the reference's instantiateDslash ladder
// (src/qcd/qcu_wilson.cu:61-173): every (precision, N) pair has its own
// instances, N = 6, 7, 8 included (the reference maps them to N = 5,
// src/qcd/qcu_wilson.cu:109-119), and nrhs is a runtime value split into
// groups of R RHS per thread instead of a compile-time 1..5.
#pragma once

#include <vector>

#include "dslash_kernel.cuh"

namespace qcu {

using DslashLauncher = void (*)(const DslashArgs&, int block, cudaStream_t);

// registry filled by the instantiation units (dslash_inst_*.cu); minb is the
// register-cap variant of the kernel (RegCap in dslash_kernel.cuh)
// pk selects the packed FP32x2 arithmetic variant
// rc selects the SU(3) variant that reads two-row links and reconstructs the third
// lt selects the register kernel with its links staged by TMA into shared memory (dslash_tmalink.cuh)
DslashLauncher find_dslash(int prec, int N, int R, int minb = 1, int pk = 0, int rc = 0, int lt = 0);
void register_dslash(int prec, int N, int R, int minb, int pk, DslashLauncher fn);
void register_dslash(int prec, int N, int R, int minb, int pk, int rc, DslashLauncher fn);
void register_dslash(int prec, int N, int R, int minb, int pk, int rc, int lt, DslashLauncher fn);

// RHS-per-thread values compiled for (prec, N), largest first
int dslash_r_options(int prec, int N, int* out, int max);
// The link-staged kernel: dynamic shared memory for NN stored components per
// link, hx sites per row and ebytes per complex; whether it can run A with R
// RHS per thread (alignment, box, block and shared-memory limits).
size_t tmalink_smem_bytes(int nn, int hx, int ebytes);
bool tmalink_runs(const DslashArgs& A, int R, int ebytes, int nn);
// register-cap variants compiled for (prec, N, R, pk, rc, lt), ascending
int dslash_minb_options(int prec, int N, int R, int pk, int* out, int max, int rc = 0, int lt = 0);

struct DslashConfig {
  int R = 1;
  int block = 128;  // <= 256 (launch bounds)
  int minb = 1;
  int pk = 0;
  int tma = 0;   // > 0: the TMA-staged kernel (dslash_tma.cuh) with this many ring stages
  int rcta = 0;  // its RHS per tile (0: the largest that fits)
  int tc = 0;    // tensor-core kernel (dslash_tc.cuh): 1 direct loads, 2 / 3 TMA ring of that depth
  int rc = 0;    // 1: SU(3) two-row links with the third row reconstructed (register kernel)
  int lt = 0;    // 1: the register kernel with its links staged by TMA (one CTA per x-row)
};

// The register kernel's site order and output store policy for B (prec, N):
// slabs of z-planes where whole t-slices of the field overflow L2, evict-first
// output stores where the field is larger than L2.
void plan_site_order(DslashArgs& B, int prec, int N);
// The shape launch_dslash last launched on the calling thread (after its
// fallbacks: a pinned shape the arguments rule out runs another kernel).
DslashConfig last_launched_dslash();

// whether the staged kernel of cfg can run these arguments
bool tma_runs(const DslashArgs& A, int prec, int N, const DslashConfig& cfg);
// whether the tensor-core kernel variant (1 direct, 2 / 3 TMA ring) can run these arguments
bool tc_runs(const DslashArgs& A, int prec, int N, int variant = 1);

// launch with an explicit configuration (throws if not compiled)
void launch_dslash(const DslashArgs& A, int prec, int N, const DslashConfig& cfg, cudaStream_t st);

// Work-list form of the register kernel (wilson_segments_kernel): many
// (lattice, gauge, fields) segments in one launch.
using SegmentsLauncher = void (*)(HopSegments&, int block, cudaStream_t);
void register_segments(int prec, int N, int R, int minb, int pk, int rc, SegmentsLauncher fn);
SegmentsLauncher find_segments(int prec, int N, int R, int minb, int pk, int rc);
// the shapes with a work-list form for (prec, N): up to max (R, minb, pk, rc) in out[4 * i ..]
int segments_options(int prec, int N, int* out, int max);
// The hop on the segments with the kernel shape cfg: those whose nrhs is a
// multiple of its R run in one launch per kMaxHopSegments segments when the
// shape has a work-list form (two-row links only when every one of them has
// them), else one launch each.  The indices of the segments cfg cannot take
// (nrhs not a multiple of R) are returned in *misfits, not launched.
// Returns the number of launches.
int launch_dslash_segments(const std::vector<DslashArgs>& segs, int prec, int N, const DslashConfig& cfg,
                           cudaStream_t st, std::vector<int>* misfits);

}  // namespace qcu
