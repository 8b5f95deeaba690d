// Dslash instances for PREC_HALF; registered at library load.
#include "dslash.h"

namespace qcu {
namespace {
struct Register_h3 {
  Register_h3() {
    register_dslash(PREC_HALF, 3, 1, 1, 0, &launch_wilson_mrhs<PREC_HALF, 3, 1, 1, false>);
    register_dslash(PREC_HALF, 3, 1, 2, 0, &launch_wilson_mrhs<PREC_HALF, 3, 1, 2, false>);
    register_dslash(PREC_HALF, 3, 2, 1, 0, &launch_wilson_mrhs<PREC_HALF, 3, 2, 1, false>);
    register_dslash(PREC_HALF, 3, 2, 2, 0, &launch_wilson_mrhs<PREC_HALF, 3, 2, 2, false>);
    register_dslash(PREC_HALF, 3, 4, 1, 0, &launch_wilson_mrhs<PREC_HALF, 3, 4, 1, false>);
    register_dslash(PREC_HALF, 3, 4, 2, 0, &launch_wilson_mrhs<PREC_HALF, 3, 4, 2, false>);
  }
} register_h3;
}  // namespace
}  // namespace qcu
