// Work-list (segment) forms of the register-kernel shapes the autotuner picks
// most; registered at library load.  Other shapes run one launch per segment.
#include "dslash.h"

namespace qcu {
namespace {
template <int P, int N, int R, int MINB, bool PK, bool RC>
void reg() {
  register_segments(P, N, R, MINB, PK ? 1 : 0, RC ? 1 : 0, &launch_wilson_segments<P, N, R, MINB, PK, RC>);
}
struct RegisterSegments {
  RegisterSegments() {
    reg<PREC_SINGLE, 3, 2, 2, true, true>();
    reg<PREC_SINGLE, 3, 2, 2, true, false>();
    reg<PREC_SINGLE, 3, 2, 2, false, true>();
    reg<PREC_SINGLE, 3, 2, 2, false, false>();
    reg<PREC_SINGLE, 3, 1, 1, false, false>();
    reg<PREC_SINGLE, 4, 2, 1, false, false>();
    reg<PREC_DOUBLE, 3, 1, 1, false, true>();
    reg<PREC_DOUBLE, 3, 1, 1, false, false>();
    reg<PREC_BF16, 3, 2, 2, true, true>();
  }
} register_segments_at_load;
}  // namespace
}  // namespace qcu
