// Instances of the TMA-staged dslash (dslash_tma.cuh); registered at library
// load.  (R, stages) per (precision, N).
#include "dslash_tma.h"

namespace qcu {
namespace {
struct RegisterTma {
  RegisterTma() {
    register_tma(PREC_SINGLE, 3, 2, 2, &launch_wilson_tma<PREC_SINGLE, 3, 2, 2>);
    register_tma(PREC_SINGLE, 3, 2, 3, &launch_wilson_tma<PREC_SINGLE, 3, 2, 3>);
    register_tma(PREC_SINGLE, 3, 2, 4, &launch_wilson_tma<PREC_SINGLE, 3, 2, 4>);
    register_tma(PREC_SINGLE, 3, 1, 3, &launch_wilson_tma<PREC_SINGLE, 3, 1, 3>);
    register_tma(PREC_DOUBLE, 3, 1, 2, &launch_wilson_tma<PREC_DOUBLE, 3, 1, 2>);
    register_tma(PREC_DOUBLE, 3, 1, 3, &launch_wilson_tma<PREC_DOUBLE, 3, 1, 3>);
    register_tma(PREC_SINGLE, 4, 2, 3, &launch_wilson_tma<PREC_SINGLE, 4, 2, 3>);
    register_tma(PREC_HALF, 3, 2, 3, &launch_wilson_tma<PREC_HALF, 3, 2, 3>);
    register_tma(PREC_HALF, 3, 4, 3, &launch_wilson_tma<PREC_HALF, 3, 4, 3>);
    register_tma(PREC_BF16, 3, 2, 3, &launch_wilson_tma<PREC_BF16, 3, 2, 3>);
    register_tma(PREC_BF16, 3, 4, 3, &launch_wilson_tma<PREC_BF16, 3, 4, 3>);
  }
} register_tma_instances;
}  // namespace
}  // namespace qcu
