// Instances of the spinor-operand tensor-core dslash (dslash_tcs.cuh):
// tensor-core variants 4-8 (ring depths in dslash_tc.h), BF16 in either
// layout, N = 3..8.
#include "dslash_tc.h"

namespace qcu {
namespace {

// the same launchers serve both BF16 layouts (the plan reads the layout)
template <int N>
void register_n() {
  for (int prec : {(int)PREC_BF16, (int)PREC_BF16S}) {
    register_tc(prec, N, 4, &launch_wilson_tcs<N, 4>);
    register_tc(prec, N, 5, &launch_wilson_tcs<N, 5>);
    register_tc(prec, N, 6, &launch_wilson_tcs<N, 6>);
    register_tc(prec, N, 7, &launch_wilson_tcs<N, 7>);
    register_tc(prec, N, 8, &launch_wilson_tcs<N, 8>);
  }
}

struct RegisterTcs {
  RegisterTcs() {
    register_n<3>();
    register_n<4>();
    register_n<5>();
    register_n<6>();
    register_n<7>();
    register_n<8>();
  }
} register_tcs_instances;

}  // namespace
}  // namespace qcu
