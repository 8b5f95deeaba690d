// qcu::storage::shiftVectorStorage / shiftGaugeStorage with the reference's
// signatures and semantics (src/storage/qcu_storage.cu:9-35 of the
// reference), implemented as shared-memory tiled transposes.  Errors are
// reported through qcuGetLastError() instead of exit(1).
#pragma GCC visibility push(default)  // the public headers: exported
#include "../../include/qcu_gb300.h"
#include "../../include/qcu_storage.h"
#pragma GCC visibility pop
#include "layout.h"

extern "C" void qcu_record_error(int code, const char* msg);

namespace qcu {
namespace storage {

void shiftVectorStorage(void* dstVec, void* srcVec, ShiftDirection shift_direction, int subLx, int Ly, int Lz,
                        int Lt) {
  try {
    const int vh = subLx * Ly * Lz * Lt;
    QCU_REQUIRE(vh > 0 && dstVec && srcVec, QCU_ERR_INVALID_ARGUMENT, "shiftVectorStorage: bad arguments");
    if (shift_direction == TO_COALESCE)
      transpose_c64(srcVec, dstVec, vh, 12, 0);  // [Vh][12] -> [12][Vh]
    else
      transpose_c64(srcVec, dstVec, 12, vh, 0);  // [12][Vh] -> [Vh][12]
    QCU_CHECK_CUDA(cudaStreamSynchronize(0));
  } catch (const Error& e) {
    qcu_record_error(e.code, e.what());
  }
}

void shiftGaugeStorage(void* dst_vec, void* src_vec, ShiftDirection shift_direction, int Lx, int Ly, int Lz, int Lt) {
  try {
    const int vh = Lx / 2 * Ly * Lz * Lt;
    QCU_REQUIRE(vh > 0 && dst_vec && src_vec, QCU_ERR_INVALID_ARGUMENT, "shiftGaugeStorage: bad arguments");
    for (int mp = 0; mp < 8; mp++) {
      const double2* s = static_cast<const double2*>(src_vec) + (size_t)mp * vh * 9;
      double2* d = static_cast<double2*>(dst_vec) + (size_t)mp * vh * 9;
      if (shift_direction == TO_COALESCE)
        transpose_c64(s, d, vh, 9, 0);
      else
        transpose_c64(s, d, 9, vh, 0);
    }
    QCU_CHECK_CUDA(cudaStreamSynchronize(0));
  } catch (const Error& e) {
    qcu_record_error(e.code, e.what());
  }
}

}  // namespace storage
}  // namespace qcu
