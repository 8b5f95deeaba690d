/*
 * qcuDesc/qcu_desc.h -- lattice and process-grid descriptors of the
 * reference's C++ interface (include/qcuDesc/qcu_desc.h:9-97 of the
 * reference): class templates in the global namespace over the number of
 * dimensions, dim[] in X, Y, Z, T order, constructible from four extents or
 * from the C structs of qcu.h.  Same layout (one int per dimension), so they
 * pass by reference between code built against either header.
 */
#pragma once

#include <cassert>

#include "../qcu.h"
#include "../qcu_enum.h"

template <int _Ndim>
struct QcuLattDesc {
  int dim[_Ndim];

  QcuLattDesc(int x, int y, int z, int t) {
    const int v[4] = {x, y, z, t};
    for (int i = 0; i < _Ndim && i < 4; i++) dim[i] = v[i];
  }
  QcuLattDesc(QcuParam *param) {
    for (int i = 0; i < _Ndim && i < 4; i++) dim[i] = param->lattice_size[i];
  }
  int X() { return dim[X_DIM]; }
  int Y() { return at(Y_DIM); }
  int Z() { return at(Z_DIM); }
  int T() { return at(T_DIM); }

 private:
  int at(int d) {
    assert(d < _Ndim && "dimension beyond the descriptor");
    return d < _Ndim ? dim[d] : 0;
  }
};

template <int _Ndim>
struct QcuProcDesc {
  int dim[_Ndim];

  QcuProcDesc(int x, int y, int z, int t) {
    const int v[4] = {x, y, z, t};
    for (int i = 0; i < _Ndim && i < 4; i++) dim[i] = v[i];
  }
  QcuProcDesc(QcuGrid *grid) {
    for (int i = 0; i < _Ndim && i < 4; i++) dim[i] = grid->grid_size[i];
  }
  int X() { return dim[X_DIM]; }
  int Y() { return at(Y_DIM); }
  int Z() { return at(Z_DIM); }
  int T() { return at(T_DIM); }

 private:
  int at(int d) {
    assert(d < _Ndim && "dimension beyond the descriptor");
    return d < _Ndim ? dim[d] : 0;
  }
};
