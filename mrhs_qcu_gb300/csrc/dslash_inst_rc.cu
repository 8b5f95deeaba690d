// Dslash instances on two-row SU(3) links (third row reconstructed); registered
// at library load.
#include "dslash.h"

namespace qcu {
namespace {
struct RegisterRc {
  RegisterRc() {
    register_dslash(PREC_SINGLE, 3, 1, 1, 0, 1, &launch_wilson_mrhs<PREC_SINGLE, 3, 1, 1, false, true>);
    register_dslash(PREC_SINGLE, 3, 1, 2, 0, 1, &launch_wilson_mrhs<PREC_SINGLE, 3, 1, 2, false, true>);
    register_dslash(PREC_SINGLE, 3, 2, 1, 0, 1, &launch_wilson_mrhs<PREC_SINGLE, 3, 2, 1, false, true>);
    register_dslash(PREC_SINGLE, 3, 2, 2, 0, 1, &launch_wilson_mrhs<PREC_SINGLE, 3, 2, 2, false, true>);
    register_dslash(PREC_SINGLE, 3, 4, 1, 0, 1, &launch_wilson_mrhs<PREC_SINGLE, 3, 4, 1, false, true>);
    register_dslash(PREC_DOUBLE, 3, 1, 1, 0, 1, &launch_wilson_mrhs<PREC_DOUBLE, 3, 1, 1, false, true>);
    register_dslash(PREC_DOUBLE, 3, 1, 2, 0, 1, &launch_wilson_mrhs<PREC_DOUBLE, 3, 1, 2, false, true>);
    register_dslash(PREC_HALF, 3, 2, 2, 0, 1, &launch_wilson_mrhs<PREC_HALF, 3, 2, 2, false, true>);
    register_dslash(PREC_HALF, 3, 4, 1, 0, 1, &launch_wilson_mrhs<PREC_HALF, 3, 4, 1, false, true>);
    register_dslash(PREC_BF16, 3, 2, 2, 0, 1, &launch_wilson_mrhs<PREC_BF16, 3, 2, 2, false, true>);
    register_dslash(PREC_BF16, 3, 4, 1, 0, 1, &launch_wilson_mrhs<PREC_BF16, 3, 4, 1, false, true>);
  }
} register_rc;
}  // namespace
}  // namespace qcu
