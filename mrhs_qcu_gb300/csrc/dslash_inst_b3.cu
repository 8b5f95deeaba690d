// Dslash instances for PREC_BF16; registered at library load.
#include "dslash.h"

namespace qcu {
namespace {
struct Register_b3 {
  Register_b3() {
    register_dslash(PREC_BF16, 3, 1, 1, 0, &launch_wilson_mrhs<PREC_BF16, 3, 1, 1, false>);
    register_dslash(PREC_BF16, 3, 1, 2, 0, &launch_wilson_mrhs<PREC_BF16, 3, 1, 2, false>);
    register_dslash(PREC_BF16, 3, 2, 1, 0, &launch_wilson_mrhs<PREC_BF16, 3, 2, 1, false>);
    register_dslash(PREC_BF16, 3, 2, 2, 0, &launch_wilson_mrhs<PREC_BF16, 3, 2, 2, false>);
    register_dslash(PREC_BF16, 3, 4, 1, 0, &launch_wilson_mrhs<PREC_BF16, 3, 4, 1, false>);
    register_dslash(PREC_BF16, 3, 4, 2, 0, &launch_wilson_mrhs<PREC_BF16, 3, 4, 2, false>);
  }
} register_b3;
}  // namespace
}  // namespace qcu
