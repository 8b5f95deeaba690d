// Dslash instances with packed FP32x2 arithmetic on two-row SU(3) links (third
// row reconstructed); registered at library load.
#include "dslash.h"

namespace qcu {
namespace {
struct RegisterRcPacked {
  RegisterRcPacked() {
    register_dslash(PREC_SINGLE, 3, 2, 2, 1, 1, &launch_wilson_mrhs<PREC_SINGLE, 3, 2, 2, true, true>);
    register_dslash(PREC_SINGLE, 3, 2, 1, 1, 1, &launch_wilson_mrhs<PREC_SINGLE, 3, 2, 1, true, true>);
    register_dslash(PREC_SINGLE, 3, 4, 1, 1, 1, &launch_wilson_mrhs<PREC_SINGLE, 3, 4, 1, true, true>);
    register_dslash(PREC_HALF, 3, 2, 2, 1, 1, &launch_wilson_mrhs<PREC_HALF, 3, 2, 2, true, true>);
    register_dslash(PREC_BF16, 3, 2, 2, 1, 1, &launch_wilson_mrhs<PREC_BF16, 3, 2, 2, true, true>);
  }
} register_rc_packed;
}  // namespace
}  // namespace qcu
