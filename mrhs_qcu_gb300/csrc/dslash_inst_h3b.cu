// Dslash instances for PREC_HALF; registered at library load.
#include "dslash.h"

namespace qcu {
namespace {
struct Register_h3b {
  Register_h3b() {
    register_dslash(PREC_HALF, 3, 1, 3, 0, &launch_wilson_mrhs<PREC_HALF, 3, 1, 3, false>);
    register_dslash(PREC_HALF, 3, 3, 1, 0, &launch_wilson_mrhs<PREC_HALF, 3, 3, 1, false>);
    register_dslash(PREC_HALF, 3, 2, 2, 1, &launch_wilson_mrhs<PREC_HALF, 3, 2, 2, true>);
    register_dslash(PREC_HALF, 3, 4, 1, 1, &launch_wilson_mrhs<PREC_HALF, 3, 4, 1, true>);
    register_dslash(PREC_HALF, 3, 2, 4, 0, &launch_wilson_mrhs<PREC_HALF, 3, 2, 4, false>);
    register_dslash(PREC_HALF, 3, 1, 5, 0, &launch_wilson_mrhs<PREC_HALF, 3, 1, 5, false>);
  }
} register_h3b;
}  // namespace
}  // namespace qcu
