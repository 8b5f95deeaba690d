/*
 * qcu_enum.h -- the enumerations of the reference's C++ interface, same
 * names and values (include/qcu_enum.h:3-22 of the reference), used by the
 * C++ entry points (qcu_dirac.h, qcd/qcu_dslash.h, qcu_storage.h).
 *
 * qcu_gb300.h defines QCU_HALF/SINGLE/DOUBLE_PRECISION as macros for C
 * callers; this header removes those macros so the enumerators of the same
 * names and values take their place, in either include order.
 */
#pragma once
#define QCU_ENUM_H_INCLUDED 1

#undef QCU_HALF_PRECISION
#undef QCU_SINGLE_PRECISION
#undef QCU_DOUBLE_PRECISION

enum QCU_PRECISION { QCU_HALF_PRECISION = 0, QCU_SINGLE_PRECISION = 1, QCU_DOUBLE_PRECISION = 2, QCU_PRECISION_UNDEFINED };
enum QCU_PC { QCU_NO_PRECONDITION = 0, QCU_EO_PC_4D };
enum QCU_PARITY { EVEN_PARITY = 0, ODD_PARITY = 1, PARITY = 2 };
enum DIMS { X_DIM = 0, Y_DIM, Z_DIM, T_DIM, Nd };
enum DIRS { BWD = 0, FWD = 1, DIRECTIONS };
enum QCU_DAGGER_FLAG { QCU_DAGGER_NO = 0, QCU_DAGGER_YES, QCU_DAGGER_UNDEFINED };
enum DSLASH_TYPE { DSLASH_WILSON = 0, DSLASH_CLOVER, DSLASH_UNKNOWN };
enum MemoryStorage { NON_COALESCED = 0, COALESCED = 1 };
enum ShiftDirection { TO_COALESCE = 0, TO_NON_COALESCE = 1 };
