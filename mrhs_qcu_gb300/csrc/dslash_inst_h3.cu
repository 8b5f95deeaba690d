// Dslash instances for PREC_HALF; registered at library load.
#include "dslash.h"

namespace qcu {
namespace {
struct Register_h3 {
  Register_h3() {
    register_dslash(PREC_HALF, 3, 1, 1, &launch_wilson_mrhs<PREC_HALF, 3, 1, 1>);
    register_dslash(PREC_HALF, 3, 1, 2, &launch_wilson_mrhs<PREC_HALF, 3, 1, 2>);
    register_dslash(PREC_HALF, 3, 1, 3, &launch_wilson_mrhs<PREC_HALF, 3, 1, 3>);
    register_dslash(PREC_HALF, 3, 2, 1, &launch_wilson_mrhs<PREC_HALF, 3, 2, 1>);
    register_dslash(PREC_HALF, 3, 2, 2, &launch_wilson_mrhs<PREC_HALF, 3, 2, 2>);
    register_dslash(PREC_HALF, 3, 3, 1, &launch_wilson_mrhs<PREC_HALF, 3, 3, 1>);
    register_dslash(PREC_HALF, 3, 4, 1, &launch_wilson_mrhs<PREC_HALF, 3, 4, 1>);
    register_dslash(PREC_HALF, 3, 4, 2, &launch_wilson_mrhs<PREC_HALF, 3, 4, 2>);
  }
} register_h3;
}  // namespace
}  // namespace qcu
