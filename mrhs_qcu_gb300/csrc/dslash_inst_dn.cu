// Dslash instances for PREC_DOUBLE; registered at library load.
#include "dslash.h"

namespace qcu {
namespace {
struct Register_dn {
  Register_dn() {
    register_dslash(PREC_DOUBLE, 4, 1, 1, 0, &launch_wilson_mrhs<PREC_DOUBLE, 4, 1, 1, false>);
    register_dslash(PREC_DOUBLE, 4, 2, 1, 0, &launch_wilson_mrhs<PREC_DOUBLE, 4, 2, 1, false>);
    register_dslash(PREC_DOUBLE, 5, 1, 1, 0, &launch_wilson_mrhs<PREC_DOUBLE, 5, 1, 1, false>);
    register_dslash(PREC_DOUBLE, 6, 1, 1, 0, &launch_wilson_mrhs<PREC_DOUBLE, 6, 1, 1, false>);
    register_dslash(PREC_DOUBLE, 7, 1, 1, 0, &launch_wilson_mrhs<PREC_DOUBLE, 7, 1, 1, false>);
    register_dslash(PREC_DOUBLE, 8, 1, 1, 0, &launch_wilson_mrhs<PREC_DOUBLE, 8, 1, 1, false>);
  }
} register_dn;
}  // namespace
}  // namespace qcu
