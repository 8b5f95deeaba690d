// Dslash instances for PREC_SINGLE; registered at library load.
#include "dslash.h"

namespace qcu {
namespace {
struct Register_s3 {
  Register_s3() {
    register_dslash(PREC_SINGLE, 3, 1, 1, 0, &launch_wilson_mrhs<PREC_SINGLE, 3, 1, 1, false>);
    register_dslash(PREC_SINGLE, 3, 1, 2, 0, &launch_wilson_mrhs<PREC_SINGLE, 3, 1, 2, false>);
    register_dslash(PREC_SINGLE, 3, 2, 1, 0, &launch_wilson_mrhs<PREC_SINGLE, 3, 2, 1, false>);
    register_dslash(PREC_SINGLE, 3, 2, 2, 0, &launch_wilson_mrhs<PREC_SINGLE, 3, 2, 2, false>);
    register_dslash(PREC_SINGLE, 3, 4, 1, 0, &launch_wilson_mrhs<PREC_SINGLE, 3, 4, 1, false>);
    register_dslash(PREC_SINGLE, 3, 2, 2, 1, &launch_wilson_mrhs<PREC_SINGLE, 3, 2, 2, true>);
  }
} register_s3;
}  // namespace
}  // namespace qcu
