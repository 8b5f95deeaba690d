// Dslash instances for PREC_DOUBLE; registered at library load.
#include "dslash.h"

namespace qcu {
namespace {
struct Register_d3 {
  Register_d3() {
    register_dslash(PREC_DOUBLE, 3, 1, 1, 0, &launch_wilson_mrhs<PREC_DOUBLE, 3, 1, 1, false>);
    register_dslash(PREC_DOUBLE, 3, 1, 2, 0, &launch_wilson_mrhs<PREC_DOUBLE, 3, 1, 2, false>);
    register_dslash(PREC_DOUBLE, 3, 2, 1, 0, &launch_wilson_mrhs<PREC_DOUBLE, 3, 2, 1, false>);
    register_dslash(PREC_DOUBLE, 3, 3, 1, 0, &launch_wilson_mrhs<PREC_DOUBLE, 3, 3, 1, false>);
    register_dslash(PREC_DOUBLE, 3, 4, 1, 0, &launch_wilson_mrhs<PREC_DOUBLE, 3, 4, 1, false>);
    register_dslash(PREC_DOUBLE, 3, 1, 4, 0, &launch_wilson_mrhs<PREC_DOUBLE, 3, 1, 4, false>);
  }
} register_d3;
}  // namespace
}  // namespace qcu
