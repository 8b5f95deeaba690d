// Dslash instances for PREC_SINGLE; registered at library load.
#include "dslash.h"

namespace qcu {
namespace {
struct Register_sn {
  Register_sn() {
    register_dslash(PREC_SINGLE, 4, 1, 1, 0, &launch_wilson_mrhs<PREC_SINGLE, 4, 1, 1, false>);
    register_dslash(PREC_SINGLE, 4, 2, 1, 0, &launch_wilson_mrhs<PREC_SINGLE, 4, 2, 1, false>);
    register_dslash(PREC_SINGLE, 4, 4, 1, 0, &launch_wilson_mrhs<PREC_SINGLE, 4, 4, 1, false>);
    register_dslash(PREC_SINGLE, 5, 1, 1, 0, &launch_wilson_mrhs<PREC_SINGLE, 5, 1, 1, false>);
    register_dslash(PREC_SINGLE, 5, 2, 1, 0, &launch_wilson_mrhs<PREC_SINGLE, 5, 2, 1, false>);
    register_dslash(PREC_SINGLE, 6, 1, 1, 0, &launch_wilson_mrhs<PREC_SINGLE, 6, 1, 1, false>);
    register_dslash(PREC_SINGLE, 6, 2, 1, 0, &launch_wilson_mrhs<PREC_SINGLE, 6, 2, 1, false>);
    register_dslash(PREC_SINGLE, 7, 1, 1, 0, &launch_wilson_mrhs<PREC_SINGLE, 7, 1, 1, false>);
    register_dslash(PREC_SINGLE, 8, 1, 1, 0, &launch_wilson_mrhs<PREC_SINGLE, 8, 1, 1, false>);
    register_dslash(PREC_SINGLE, 8, 2, 1, 0, &launch_wilson_mrhs<PREC_SINGLE, 8, 2, 1, false>);
  }
} register_sn;
}  // namespace
}  // namespace qcu
