/*
 * qcu_storage.h -- C++ layout-transform API with the reference's exact
 * signatures (include/storage/qcu_storage.h:5-6 of the reference; the
 * ShiftDirection enum is in qcu_enum.h), so C++ callers of
 * qcu::storage::shiftVectorStorage / shiftGaugeStorage link against libqcu.so
 * unchanged.  Same semantics: complex double SU(3), one RHS, caller layout
 * [Vh][4][3] <-> coalesced [12][Vh], gauge [4][2][Vh][9] <-> [4][2][9][Vh];
 * synchronous on the legacy default stream.
 */
#pragma once

#include "qcu_enum.h"

namespace qcu {
namespace storage {
void shiftVectorStorage(void *dstVec, void *srcVec, ShiftDirection shift_direction, int subLx, int Ly, int Lz, int Lt);
void shiftGaugeStorage(void *dst_vec, void *src_vec, ShiftDirection shift_direction, int Lx, int Ly, int Lz, int Lt);
}  // namespace storage
}  // namespace qcu
