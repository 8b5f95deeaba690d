// Dslash instances for PREC_HALF; registered at library load.
#include "dslash.h"

namespace qcu {
namespace {
struct Register_hn {
  Register_hn() {
    register_dslash(PREC_HALF, 4, 1, 1, 0, &launch_wilson_mrhs<PREC_HALF, 4, 1, 1, false>);
    register_dslash(PREC_HALF, 4, 2, 1, 0, &launch_wilson_mrhs<PREC_HALF, 4, 2, 1, false>);
    register_dslash(PREC_HALF, 4, 4, 1, 0, &launch_wilson_mrhs<PREC_HALF, 4, 4, 1, false>);
    register_dslash(PREC_HALF, 5, 1, 1, 0, &launch_wilson_mrhs<PREC_HALF, 5, 1, 1, false>);
    register_dslash(PREC_HALF, 5, 2, 1, 0, &launch_wilson_mrhs<PREC_HALF, 5, 2, 1, false>);
    register_dslash(PREC_HALF, 6, 1, 1, 0, &launch_wilson_mrhs<PREC_HALF, 6, 1, 1, false>);
    register_dslash(PREC_HALF, 6, 2, 1, 0, &launch_wilson_mrhs<PREC_HALF, 6, 2, 1, false>);
    register_dslash(PREC_HALF, 7, 1, 1, 0, &launch_wilson_mrhs<PREC_HALF, 7, 1, 1, false>);
    register_dslash(PREC_HALF, 8, 1, 1, 0, &launch_wilson_mrhs<PREC_HALF, 8, 1, 1, false>);
    register_dslash(PREC_HALF, 8, 2, 1, 0, &launch_wilson_mrhs<PREC_HALF, 8, 2, 1, false>);
  }
} register_hn;
}  // namespace
}  // namespace qcu
