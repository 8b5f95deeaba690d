// Dslash instances for PREC_SINGLE; registered at library load.
#include "dslash.h"

namespace qcu {
namespace {
struct Register_s3b {
  Register_s3b() {
    register_dslash(PREC_SINGLE, 3, 1, 3, 0, &launch_wilson_mrhs<PREC_SINGLE, 3, 1, 3, false>);
    register_dslash(PREC_SINGLE, 3, 3, 1, 0, &launch_wilson_mrhs<PREC_SINGLE, 3, 3, 1, false>);
    register_dslash(PREC_SINGLE, 3, 3, 2, 0, &launch_wilson_mrhs<PREC_SINGLE, 3, 3, 2, false>);
    register_dslash(PREC_SINGLE, 3, 4, 2, 0, &launch_wilson_mrhs<PREC_SINGLE, 3, 4, 2, false>);
    register_dslash(PREC_SINGLE, 3, 2, 1, 1, &launch_wilson_mrhs<PREC_SINGLE, 3, 2, 1, true>);
    register_dslash(PREC_SINGLE, 3, 2, 4, 0, &launch_wilson_mrhs<PREC_SINGLE, 3, 2, 4, false>);
    register_dslash(PREC_SINGLE, 3, 2, 6, 0, &launch_wilson_mrhs<PREC_SINGLE, 3, 2, 6, false>);
    register_dslash(PREC_SINGLE, 3, 1, 5, 0, &launch_wilson_mrhs<PREC_SINGLE, 3, 1, 5, false>);
  }
} register_s3b;
}  // namespace
}  // namespace qcu
