// Host side of the link-staged register kernel (dslash_tmalink.cuh): limits,
// shared-memory size, and the instances registered at library load.
#include "dslash_tmalink.cuh"

namespace qcu {

size_t tmalink_smem_bytes(int nn, int hx, int ebytes) {
  const size_t hop = ((size_t)nn * hx * ebytes + 127) / 128 * 128;
  return 8 * hop + 8 * sizeof(uint64_t);  // eight hops' boxes, one barrier each
}

bool tmalink_runs(const DslashArgs& A, int R, int ebytes, int nn) {
  const int hx = A.geo.hx;
  if (A.nrhs % R) return false;
  // one CTA per row; the instances cap registers at 128, so at most 512 threads per CTA
  const int64_t threads = (int64_t)hx * (A.nrhs / R);
  if (threads < 1 || threads > 512) return false;
  // TMA: box inner extent (hx complexes) a multiple of 16 bytes and at most 256 4-byte
  // elements, 16-byte aligned rows and strides; two-row links are read out of groups of 32
  // sites, so a row must lie within one group
  const int inner = hx * ebytes;
  if (inner % 16 || inner / 4 > 256 || nn > 256) return false;
  if (nn == 6 && 32 % hx) return false;
  const void* g = (nn == 6) ? A.gauge12 : A.gauge;
  if (!g || (uintptr_t)g % 16 || (nn != 6 && ((int64_t)A.geo.vh * ebytes) % 16)) return false;
  if (tmalink_smem_bytes(nn, hx, ebytes) > 200 * 1024) return false;
  // the register kernel's 32-bit offset limits
  if ((int64_t)4 * 3 * A.geo.vh * A.nrhs >= (1ll << 32)) return false;
  return true;
}

namespace {
struct RegisterTmaLink {
  RegisterTmaLink() {
    register_dslash(PREC_SINGLE, 3, 2, 2, 1, 1, 1, &launch_wilson_tmalink<PREC_SINGLE, 3, 2, 2, true, true>);
    register_dslash(PREC_SINGLE, 3, 2, 2, 1, 0, 1, &launch_wilson_tmalink<PREC_SINGLE, 3, 2, 2, true, false>);
    register_dslash(PREC_BF16, 3, 2, 2, 1, 1, 1, &launch_wilson_tmalink<PREC_BF16, 3, 2, 2, true, true>);
  }
} register_tmalink;
}  // namespace

}  // namespace qcu
