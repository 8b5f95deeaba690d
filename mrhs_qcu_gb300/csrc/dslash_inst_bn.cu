// Dslash instances for PREC_BF16; registered at library load.
#include "dslash.h"

namespace qcu {
namespace {
struct Register_bn {
  Register_bn() {
    register_dslash(PREC_BF16, 4, 1, 1, 0, &launch_wilson_mrhs<PREC_BF16, 4, 1, 1, false>);
    register_dslash(PREC_BF16, 4, 2, 1, 0, &launch_wilson_mrhs<PREC_BF16, 4, 2, 1, false>);
    register_dslash(PREC_BF16, 4, 4, 1, 0, &launch_wilson_mrhs<PREC_BF16, 4, 4, 1, false>);
    register_dslash(PREC_BF16, 5, 1, 1, 0, &launch_wilson_mrhs<PREC_BF16, 5, 1, 1, false>);
    register_dslash(PREC_BF16, 5, 2, 1, 0, &launch_wilson_mrhs<PREC_BF16, 5, 2, 1, false>);
    register_dslash(PREC_BF16, 6, 1, 1, 0, &launch_wilson_mrhs<PREC_BF16, 6, 1, 1, false>);
    register_dslash(PREC_BF16, 6, 2, 1, 0, &launch_wilson_mrhs<PREC_BF16, 6, 2, 1, false>);
    register_dslash(PREC_BF16, 7, 1, 1, 0, &launch_wilson_mrhs<PREC_BF16, 7, 1, 1, false>);
    register_dslash(PREC_BF16, 8, 1, 1, 0, &launch_wilson_mrhs<PREC_BF16, 8, 1, 1, false>);
    register_dslash(PREC_BF16, 8, 2, 1, 0, &launch_wilson_mrhs<PREC_BF16, 8, 2, 1, false>);
  }
} register_bn;
}  // namespace
}  // namespace qcu
