// ref_fields.cpp -- TEST INFRASTRUCTURE ONLY.
//
// The reference's src/geometry/FIELD_3D.cpp and VECTOR3_FIELD_3D.cpp include
// OpenGL headers, so they are not compiled for the oracle.  This file restates
// the member functions that the reference's FLUID_3D_MIC.cpp calls, against
// the reference's own class declarations (FIELD_3D.h, VECTOR3_FIELD_3D.h),
// each following the cited reference definition.  BOX.cpp includes OpenGL for
// BOX::draw as well, so the BOX members that FLUID_3D_MIC.cpp and the headless
// driver call are restated here too (draw is left out).
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <zlib.h>

#include "BOX.h"
#include "FIELD_3D.h"
#include "VECTOR3_FIELD_3D.h"

int FIELD_3D::_quinticClamps = 0;

// ------------------------------------------------------------------ FIELD_3D
// FIELD_3D.cpp:202-205
FIELD_3D::FIELD_3D() : _xRes(-1), _yRes(-1), _zRes(-1), _totalCells(-1), _data(NULL) {}

// FIELD_3D.cpp:22-51 (zero-filled)
FIELD_3D::FIELD_3D(const int& xRes, const int& yRes, const int& zRes, const VEC3F& center,
                   const VEC3F& lengths)
    : _xRes(xRes), _yRes(yRes), _zRes(zRes), _center(center), _lengths(lengths) {
  _totalCells = _xRes * _yRes * _zRes;
  _slabSize = _xRes * _yRes;
  _data = new Real[_totalCells];
  for (int x = 0; x < _totalCells; x++) _data[x] = 0;
  _dx = _lengths[0] / _xRes;
  _dy = _lengths[1] / _yRes;
  _dz = _lengths[2] / _zRes;
  _invDx = 1.0 / _dx;
  _invDy = 1.0 / _dy;
  _invDz = 1.0 / _dz;
  { int m = _xRes > _yRes ? _xRes : _yRes; m = _zRes > m ? _zRes : m; _outside = m * m; }
}

// copy constructor: same dimensions, center, lengths and values
FIELD_3D::FIELD_3D(const FIELD_3D& m)
    : _xRes(m.xRes()), _yRes(m.yRes()), _zRes(m.zRes()), _center(m.center()),
      _lengths(m.lengths()) {
  _totalCells = _xRes * _yRes * _zRes;
  _slabSize = _xRes * _yRes;
  _data = new Real[_totalCells];
  for (int x = 0; x < _totalCells; x++) _data[x] = m[x];
  _dx = _lengths[0] / _xRes;
  _dy = _lengths[1] / _yRes;
  _dz = _lengths[2] / _zRes;
  _invDx = 1.0 / _dx;
  _invDy = 1.0 / _dy;
  _invDz = 1.0 / _dz;
  { int m = _xRes > _yRes ? _xRes : _yRes; m = _zRes > m ? _zRes : m; _outside = m * m; }
}

// FIELD_3D.cpp:257-263
FIELD_3D::~FIELD_3D() {
  if (_data) {
    delete[] _data;
    _data = NULL;
  }
}

// FIELD_3D.cpp:787-... : reallocate on size change, then copy everything
FIELD_3D& FIELD_3D::operator=(const FIELD_3D& A) {
  if (A.xRes() != _xRes || A.yRes() != _yRes || A.zRes() != _zRes || _data == NULL) {
    if (_data) delete[] _data;
    _xRes = A.xRes();
    _yRes = A.yRes();
    _zRes = A.zRes();
    _slabSize = _xRes * _yRes;
    _totalCells = _xRes * _yRes * _zRes;
    _data = new Real[_totalCells];
  }
  for (int x = 0; x < _totalCells; x++) _data[x] = A[x];
  _center = A.center();
  _lengths = A.lengths();
  _dx = _lengths[0] / _xRes;
  _dy = _lengths[1] / _yRes;
  _dz = _lengths[2] / _zRes;
  _invDx = 1.0 / _dx;
  _invDy = 1.0 / _dy;
  _invDz = 1.0 / _dz;
  { int m = _xRes > _yRes ? _xRes : _yRes; m = _zRes > m ? _zRes : m; _outside = m * m; }
  return *this;
}

// FIELD_3D.cpp:576-...
FIELD_3D& FIELD_3D::operator*=(const Real& alpha) {
  for (int x = 0; x < _totalCells; x++) _data[x] *= alpha;
  return *this;
}

// FIELD_3D.cpp:637-...
FIELD_3D& FIELD_3D::operator+=(const FIELD_3D& input) {
  for (int x = 0; x < _totalCells; x++) _data[x] += input[x];
  return *this;
}

// FIELD_3D.cpp:5724-5733
void FIELD_3D::axpy(const Real& alpha, const FIELD_3D& input) {
  const int totalCells = input.totalCells();
  for (int x = 0; x < totalCells; x++) _data[x] += alpha * input[x];
}

// FIELD_3D.cpp:1382-1420 (z faces, then y faces, then x faces)
void FIELD_3D::copyBorderAll() {
  int index;
  for (int y = 0; y < _yRes; y++)
    for (int x = 0; x < _xRes; x++) {
      index = x + y * _xRes;
      _data[index] = _data[index + _slabSize];
      index += _totalCells - _slabSize;
      _data[index] = _data[index - _slabSize];
    }
  for (int z = 0; z < _zRes; z++)
    for (int x = 0; x < _xRes; x++) {
      index = x + z * _slabSize;
      _data[index] = _data[index + _xRes];
      index += _slabSize - _xRes;
      _data[index] = _data[index - _xRes];
    }
  for (int z = 0; z < _zRes; z++)
    for (int y = 0; y < _yRes; y++) {
      index = y * _xRes + z * _slabSize;
      _data[index] = _data[index + 1];
      index += _xRes - 1;
      _data[index] = _data[index - 1];
    }
}

// FIELD_3D.cpp:6591-6602
Real FIELD_3D::dot(const FIELD_3D& input) const {
  Real final = 0;
  for (int x = 0; x < _totalCells; x++) final += input[x] * _data[x];
  return final;
}

// FIELD_3D.cpp:1529-1538 (signed maximum)
Real FIELD_3D::max() {
  Real final = _data[0];
  for (int i = 0; i < _totalCells; i++)
    if (_data[i] > final) final = _data[i];
  return final;
}

// FIELD_3D.cpp:6722-6733
VECTOR FIELD_3D::flattened() const {
  VECTOR final(_totalCells);
  for (int i = 0; i < _totalCells; i++) final[i] = _data[i];
  return final;
}

// FIELD_3D.cpp:6679-6689
FIELD_3D FIELD_3D::peelBoundary() const {
  FIELD_3D final(_xRes - 2, _yRes - 2, _zRes - 2);
  for (int z = 1; z < _zRes - 1; z++)
    for (int y = 1; y < _yRes - 1; y++)
      for (int x = 1; x < _xRes - 1; x++) final(x - 1, y - 1, z - 1) = (*this)(x, y, z);
  return final;
}

// FIELD_3D.cpp:5993-6014: 3 ints, center, lengths, then the doubles
void FIELD_3D::writeGz(gzFile& file) const {
  gzwrite(file, (void*)&_xRes, sizeof(int));
  gzwrite(file, (void*)&_yRes, sizeof(int));
  gzwrite(file, (void*)&_zRes, sizeof(int));
  _center.writeGz(file);
  _lengths.writeGz(file);
  gzwrite(file, (void*)_data, _totalCells * sizeof(Real));
}

// FIELD_3D.cpp:6019-6050
void FIELD_3D::readGz(gzFile& file) {
  gzread(file, (void*)&_xRes, sizeof(int));
  gzread(file, (void*)&_yRes, sizeof(int));
  gzread(file, (void*)&_zRes, sizeof(int));
  _center.readGz(file);
  _lengths.readGz(file);
  _dx = _lengths[0] / _xRes;
  _dy = _lengths[1] / _yRes;
  _dz = _lengths[2] / _zRes;
  _invDx = 1.0 / _dx;
  _invDy = 1.0 / _dy;
  _invDz = 1.0 / _dz;
  { int m = _xRes > _yRes ? _xRes : _yRes; m = _zRes > m ? _zRes : m; _outside = m * m; }
  _slabSize = _xRes * _yRes;
  _totalCells = _xRes * _yRes * _zRes;
  if (_data) delete[] _data;
  _data = new Real[_totalCells];
  gzread(file, (void*)_data, _totalCells * sizeof(Real));
}

// FIELD_3D.cpp:6408-6444
void FIELD_3D::setZeroBorder() {
  int index;
  for (int z = 0; z < _zRes; z++)
    for (int y = 0; y < _yRes; y++) {
      index = y * _xRes + z * _slabSize;
      _data[index] = 0.0f;
      index += _xRes - 1;
      _data[index] = 0.0f;
    }
  for (int z = 0; z < _zRes; z++)
    for (int x = 0; x < _xRes; x++) {
      index = x + z * _slabSize;
      _data[index] = 0.0f;
      index += _slabSize - _xRes;
      _data[index] = 0.0f;
    }
  for (int y = 0; y < _yRes; y++)
    for (int x = 0; x < _xRes; x++) {
      index = x + y * _xRes;
      _data[index] = 0.0f;
      index += _totalCells - _slabSize;
      _data[index] = 0.0f;
    }
}

// FIELD_3D.cpp:6449-6458
void FIELD_3D::swapPointers(FIELD_3D& field) {
  Real* temp = _data;
  _data = field._data;
  field._data = temp;
}

// ----------------------------------------------------------- VECTOR3_FIELD_3D
// VECTOR3_FIELD_3D.cpp:141-145
VECTOR3_FIELD_3D::VECTOR3_FIELD_3D()
    : _xRes(0), _yRes(0), _zRes(0), _totalCells(0), _data(NULL), _initialized(false) {}

// VECTOR3_FIELD_3D.cpp:16-27 (VEC3F default-constructs to zero)
VECTOR3_FIELD_3D::VECTOR3_FIELD_3D(const int& xRes, const int& yRes, const int& zRes,
                                   const VEC3F& center, const VEC3F& lengths)
    : _xRes(xRes), _yRes(yRes), _zRes(zRes), _center(center), _lengths(lengths),
      _initialized(true) {
  _totalCells = _xRes * _yRes * _zRes;
  _slabSize = _xRes * _yRes;
  _data = new VEC3F[_totalCells];
  _dx = _lengths[0] / _xRes;
  _dy = _lengths[1] / _yRes;
  _dz = _lengths[2] / _zRes;
}

// VECTOR3_FIELD_3D.cpp:109-123
VECTOR3_FIELD_3D::VECTOR3_FIELD_3D(const VECTOR3_FIELD_3D& m)
    : _xRes(m.xRes()), _yRes(m.yRes()), _zRes(m.zRes()), _center(m.center()),
      _lengths(m.lengths()), _initialized(true) {
  _totalCells = _xRes * _yRes * _zRes;
  _slabSize = _xRes * _yRes;
  _data = new VEC3F[_totalCells];
  _dx = _lengths[0] / _xRes;
  _dy = _lengths[1] / _yRes;
  _dz = _lengths[2] / _zRes;
  for (int x = 0; x < _totalCells; x++) _data[x] = m[x];
}

// VECTOR3_FIELD_3D.cpp:199-202
VECTOR3_FIELD_3D::~VECTOR3_FIELD_3D() { delete[] _data; }

// VECTOR3_FIELD_3D.cpp:1143-1173
VECTOR3_FIELD_3D& VECTOR3_FIELD_3D::operator=(const VECTOR3_FIELD_3D& input) {
  if (input.xRes() != _xRes || input.yRes() != _yRes || input.zRes() != _zRes) {
    delete[] _data;
    _xRes = input.xRes();
    _yRes = input.yRes();
    _zRes = input.zRes();
    _totalCells = _xRes * _yRes * _zRes;
    _slabSize = _xRes * _yRes;
    _data = new VEC3F[_totalCells];
  }
  _center = input.center();
  _lengths = input.lengths();
  _dx = _lengths[0] / _xRes;
  _dy = _lengths[1] / _yRes;
  _dz = _lengths[2] / _zRes;
  for (int x = 0; x < _totalCells; x++) _data[x] = input[x];
  _initialized = input._initialized;
  return *this;
}

// VECTOR3_FIELD_3D.cpp:206-211
void VECTOR3_FIELD_3D::clear() {
  for (int x = 0; x < _totalCells; x++) _data[x] = 0.0;
}

// VECTOR3_FIELD_3D.cpp:353-361
FIELD_3D VECTOR3_FIELD_3D::magnitudeField() const {
  FIELD_3D final(_xRes, _yRes, _zRes, _center, _lengths);
  for (int x = 0; x < _totalCells; x++) final[x] = norm(_data[x]);
  return final;
}

// VECTOR3_FIELD_3D.cpp:459-471
VECTOR3_FIELD_3D operator-(const VECTOR3_FIELD_3D& u, const VECTOR3_FIELD_3D& v) {
  VECTOR3_FIELD_3D final(u.xRes(), u.yRes(), u.zRes(), u.center(), u.lengths());
  const int totalCells = u.totalCells();
  for (int x = 0; x < totalCells; x++) final[x] = u[x] - v[x];
  return final;
}

// VECTOR3_FIELD_3D.cpp:2001-2077 and 2082-2158: first-order semi-Lagrangian,
// backtrace clamped to [1.5, res-2.5], trilinear weights, same evaluation order.
template <class FIELD, class VALUE>
static void advect_impl(const Real dt, const VECTOR3_FIELD_3D& velocityGrid,
                        const FIELD& oldField, FIELD& newField) {
  const int xRes = velocityGrid.xRes();
  const int yRes = velocityGrid.yRes();
  const int zRes = velocityGrid.zRes();
  const int slabSize = velocityGrid.slabSize();
  for (int z = 0; z < zRes; z++)
    for (int y = 0; y < yRes; y++)
      for (int x = 0; x < xRes; x++) {
        const int index = x + y * xRes + z * slabSize;
        const VEC3F velocity = velocityGrid[index];
        Real xTrace = x - dt * velocity[0];
        Real yTrace = y - dt * velocity[1];
        Real zTrace = z - dt * velocity[2];
        xTrace = (xTrace < 1.5) ? 1.5 : xTrace;
        xTrace = (xTrace > xRes - 2.5) ? xRes - 2.5 : xTrace;
        yTrace = (yTrace < 1.5) ? 1.5 : yTrace;
        yTrace = (yTrace > yRes - 2.5) ? yRes - 2.5 : yTrace;
        zTrace = (zTrace < 1.5) ? 1.5 : zTrace;
        zTrace = (zTrace > zRes - 2.5) ? zRes - 2.5 : zTrace;
        const int x0 = (int)xTrace;
        const int x1 = x0 + 1;
        const int y0 = (int)yTrace;
        const int y1 = y0 + 1;
        const int z0 = (int)zTrace;
        const int z1 = z0 + 1;
        const Real s1 = xTrace - x0;
        const Real s0 = 1.0f - s1;
        const Real t1 = yTrace - y0;
        const Real t0 = 1.0f - t1;
        const Real u1 = zTrace - z0;
        const Real u0 = 1.0f - u1;
        const int i000 = x0 + y0 * xRes + z0 * slabSize;
        const int i010 = x0 + y1 * xRes + z0 * slabSize;
        const int i100 = x1 + y0 * xRes + z0 * slabSize;
        const int i110 = x1 + y1 * xRes + z0 * slabSize;
        const int i001 = x0 + y0 * xRes + z1 * slabSize;
        const int i011 = x0 + y1 * xRes + z1 * slabSize;
        const int i101 = x1 + y0 * xRes + z1 * slabSize;
        const int i111 = x1 + y1 * xRes + z1 * slabSize;
        newField[index] = u0 * (s0 * (t0 * oldField[i000] + t1 * oldField[i010]) +
                                s1 * (t0 * oldField[i100] + t1 * oldField[i110])) +
                          u1 * (s0 * (t0 * oldField[i001] + t1 * oldField[i011]) +
                                s1 * (t0 * oldField[i101] + t1 * oldField[i111]));
      }
}

void VECTOR3_FIELD_3D::advect(const Real dt, const VECTOR3_FIELD_3D& velocityGrid,
                              const VECTOR3_FIELD_3D& oldField, VECTOR3_FIELD_3D& newField) {
  advect_impl<VECTOR3_FIELD_3D, VEC3F>(dt, velocityGrid, oldField, newField);
}

void VECTOR3_FIELD_3D::advect(const Real dt, const VECTOR3_FIELD_3D& velocityGrid,
                              const FIELD_3D& oldField, FIELD_3D& newField) {
  advect_impl<FIELD_3D, Real>(dt, velocityGrid, oldField, newField);
}

// VECTOR3_FIELD_3D.cpp:3113-3120
void VECTOR3_FIELD_3D::axpy(const Real& alpha, const VECTOR3_FIELD_3D& field) {
  for (int x = 0; x < _totalCells; x++) _data[x] += alpha * field[x];
}

// VECTOR3_FIELD_3D.cpp:3125-3134
void VECTOR3_FIELD_3D::swapPointers(VECTOR3_FIELD_3D& field) {
  VEC3F* temp = _data;
  _data = field._data;
  field._data = temp;
}

// VECTOR3_FIELD_3D.cpp:3139-3151
VECTOR VECTOR3_FIELD_3D::flattened() const {
  VECTOR final(_totalCells * 3);
  int index = 0;
  for (int z = 0; z < _zRes; z++)
    for (int y = 0; y < _yRes; y++)
      for (int x = 0; x < _xRes; x++)
        for (int i = 0; i < 3; i++, index++) final[index] = (*this)(x, y, z)[i];
  return final;
}

// VECTOR3_FIELD_3D.cpp:3156-3168
VectorXd VECTOR3_FIELD_3D::flattenedEigen() const {
  VectorXd final(_totalCells * 3);
  int index = 0;
  for (int z = 0; z < _zRes; z++)
    for (int y = 0; y < _yRes; y++)
      for (int x = 0; x < _xRes; x++)
        for (int i = 0; i < 3; i++, index++) final(index) = (*this)(x, y, z)[i];
  return final;
}

// VECTOR3_FIELD_3D.cpp:3222-3232
VECTOR3_FIELD_3D VECTOR3_FIELD_3D::peelBoundary() const {
  VECTOR3_FIELD_3D final(_xRes - 2, _yRes - 2, _zRes - 2);
  for (int z = 1; z < _zRes - 1; z++)
    for (int y = 1; y < _yRes - 1; y++)
      for (int x = 1; x < _xRes - 1; x++) final(x - 1, y - 1, z - 1) = (*this)(x, y, z);
  return final;
}

// VECTOR3_FIELD_3D.cpp:3415-3429
void VECTOR3_FIELD_3D::setWithPeeled(const VectorXd& data) {
  int index = 0;
  for (int z = 1; z < _zRes - 1; z++)
    for (int y = 1; y < _yRes - 1; y++)
      for (int x = 1; x < _xRes - 1; x++, index++) {
        (*this)(x, y, z)[0] = data[3 * index];
        (*this)(x, y, z)[1] = data[3 * index + 1];
        (*this)(x, y, z)[2] = data[3 * index + 2];
      }
}

// VECTOR3_FIELD_3D.cpp:2828-2867
void VECTOR3_FIELD_3D::setZeroBorder() {
  int index;
  for (int z = 0; z < _zRes; z++)
    for (int y = 0; y < _yRes; y++) {
      index = y * _xRes + z * _slabSize;
      _data[index] = 0.0f;
      index += _xRes - 1;
      _data[index] = 0.0f;
    }
  for (int z = 0; z < _zRes; z++)
    for (int x = 0; x < _xRes; x++) {
      index = x + z * _slabSize;
      _data[index] = 0.0f;
      index += _slabSize - _xRes;
      _data[index] = 0.0f;
    }
  for (int y = 0; y < _yRes; y++)
    for (int x = 0; x < _xRes; x++) {
      index = x + y * _xRes;
      _data[index] = 0.0f;
      index += _totalCells - _slabSize;
      _data[index] = 0.0f;
    }
}

// VECTOR3_FIELD_3D.cpp:2872-2924: one component of one pair of faces to zero
void VECTOR3_FIELD_3D::setZeroX() {
  for (int z = 0; z < _zRes; z++)
    for (int y = 0; y < _yRes; y++) {
      int index = y * _xRes + z * _slabSize;
      _data[index][0] = 0.0f;
      index += _xRes - 1;
      _data[index][0] = 0.0f;
    }
}
void VECTOR3_FIELD_3D::setZeroY() {
  for (int z = 0; z < _zRes; z++)
    for (int x = 0; x < _xRes; x++) {
      int index = x + z * _slabSize;
      _data[index][1] = 0.0f;
      index += _slabSize - _xRes;
      _data[index][1] = 0.0f;
    }
}
void VECTOR3_FIELD_3D::setZeroZ() {
  for (int y = 0; y < _yRes; y++)
    for (int x = 0; x < _xRes; x++) {
      int index = x + y * _xRes;
      _data[index][2] = 0.0f;
      index += _totalCells - _slabSize;
      _data[index][2] = 0.0f;
    }
}

// VECTOR3_FIELD_3D.cpp:2929-3000: copy from two cells in
void VECTOR3_FIELD_3D::setNeumannX() {
  for (int z = 0; z < _zRes; z++)
    for (int y = 0; y < _yRes; y++) {
      int index = y * _xRes + z * _slabSize;
      _data[index][0] = _data[index + 2][0];
      index += _xRes - 1;
      _data[index][0] = _data[index - 2][0];
    }
}
void VECTOR3_FIELD_3D::setNeumannY() {
  for (int z = 0; z < _zRes; z++)
    for (int x = 0; x < _xRes; x++) {
      int index = x + z * _slabSize;
      _data[index][1] = _data[index + 2 * _xRes][1];
      index += _slabSize - _xRes;
      _data[index][1] = _data[index - 2 * _xRes][1];
    }
}
void VECTOR3_FIELD_3D::setNeumannZ() {
  for (int y = 0; y < _yRes; y++)
    for (int x = 0; x < _xRes; x++) {
      int index = x + y * _xRes;
      _data[index][2] = _data[index + 2 * _slabSize][2];
      index += _totalCells - _slabSize;
      _data[index][2] = _data[index - 2 * _slabSize][2];
    }
}

// VECTOR3_FIELD_3D.cpp:3005-3053: copy from one cell in
void VECTOR3_FIELD_3D::copyBorderX() {
  for (int z = 0; z < _zRes; z++)
    for (int y = 0; y < _yRes; y++) {
      int index = y * _xRes + z * _slabSize;
      _data[index][0] = _data[index + 1][0];
      index += _xRes - 1;
      _data[index][0] = _data[index - 1][0];
    }
}
void VECTOR3_FIELD_3D::copyBorderY() {
  for (int z = 0; z < _zRes; z++)
    for (int x = 0; x < _xRes; x++) {
      int index = x + z * _slabSize;
      _data[index][1] = _data[index + _xRes][1];
      index += _slabSize - _xRes;
      _data[index][1] = _data[index - _xRes][1];
    }
}
void VECTOR3_FIELD_3D::copyBorderZ() {
  for (int y = 0; y < _yRes; y++)
    for (int x = 0; x < _xRes; x++) {
      int index = x + y * _xRes;
      _data[index][2] = _data[index + _slabSize][2];
      index += _totalCells - _slabSize;
      _data[index][2] = _data[index - _slabSize][2];
    }
}

// VECTOR3_FIELD_3D.cpp:1327-1346: interleaved doubles
void VECTOR3_FIELD_3D::writeGz(gzFile& file) const {
  gzwrite(file, (void*)&_xRes, sizeof(int));
  gzwrite(file, (void*)&_yRes, sizeof(int));
  gzwrite(file, (void*)&_zRes, sizeof(int));
  _center.writeGz(file);
  _lengths.writeGz(file);
  gzwrite(file, (void*)_data, sizeof(double) * 3 * _totalCells);
}

// VECTOR3_FIELD_3D.cpp:1351-1383
void VECTOR3_FIELD_3D::readGz(gzFile& file) {
  gzread(file, (void*)&_xRes, sizeof(int));
  gzread(file, (void*)&_yRes, sizeof(int));
  gzread(file, (void*)&_zRes, sizeof(int));
  _center.readGz(file);
  _lengths.readGz(file);
  _dx = _lengths[0] / _xRes;
  _dy = _lengths[1] / _yRes;
  _dz = _lengths[2] / _zRes;
  _slabSize = _xRes * _yRes;
  _totalCells = _xRes * _yRes * _zRes;
  if (_data) delete[] _data;
  _data = new VEC3F[_totalCells];
  gzread(file, (void*)_data, sizeof(double) * 3 * _totalCells);
}

// ----------------------------------------------------------------------- BOX
// BOX.cpp:26-41
BOX::BOX(const VEC3F& center, const VEC3F& lengths, double period, double translationPeriod)
    : _center(center), _lengths(lengths), _period(period), _translationPeriod(translationPeriod) {
  set_halfLengths();
  set_angularVelocity();
  initialize_rotationMatrix();
  _theta = 0.0;
  _phi = 0.0;
  _currentTime = 0.0;
  _dt = 0.0;
  _rotationAxis = VEC3F(0.0, 0.0, 1.0);
  _displacement = VEC3F(0.0, 0.0, 0.0);
  _displacementVelocity = VEC3F(0.0, 0.0, 0.0);
  _original_center = _center;
}
BOX::~BOX() {}

// BOX.cpp:50-57
void BOX::initialize_rotationMatrix() { _rotation = MATRIX3::I(); }
void BOX::update_rotationMatrix() { _rotation = MATRIX3::rotation(_rotationAxis, -1 * _theta); }

// BOX.cpp:59-70
bool BOX::inside(const VEC3F& point) const {
  VEC3F t = point - _center;
  t = _rotation * t;
  return fabs(t[0]) <= _halfLengths[0] && fabs(t[1]) <= _halfLengths[1] &&
         fabs(t[2]) <= _halfLengths[2];
}

// BOX.cpp:72-81
void BOX::update_r(const VEC3F& point, VEC3F* r) {
  VEC3F u = point - _center;
  *r = u - project_onto(u, _rotationAxis);
}

// BOX.cpp:84-91
void BOX::calculate_displacementVelocity() {
  _displacementVelocity[0] = 0.25 * 2 * M_PI / _translationPeriod * cos(_phi);
}

// BOX.cpp:93-101
void BOX::spin() {
  _theta += 2 * M_PI * _dt / _period;
  if (_theta >= 2 * M_PI) _theta = 0.0;
  update_rotationMatrix();
}

// BOX.cpp:104-113
void BOX::translate_center() {
  _phi += 2 * M_PI * _dt / _translationPeriod;
  if (_phi >= 2 * M_PI) _phi = 0.0;
  _displacement[0] = 0.25 * sin(_phi);
  _center[0] = _original_center[0] + _displacement[0];
}

// BOX.cpp:43-45
BOX::BOX() {}

// --------------------------------------------- members the reduced step calls
// FIELD_3D.cpp:6753-6764
VectorXd FIELD_3D::flattenedEigen() const {
  VectorXd final(_totalCells);
  int index = 0;
  for (int z = 0; z < _zRes; z++)
    for (int y = 0; y < _yRes; y++)
      for (int x = 0; x < _xRes; x++, index++) final[index] = (*this)(x, y, z);
  return final;
}

// VECTOR3_FIELD_3D.cpp:3434-3553: U^T times the peeled field (x fastest,
// components interleaved), accumulated in the reference's grouping: per row
// (y, z) four partial sums over x = 0, 4, ... (and x + 1, + 2, + 3), added to
// the total in that order, then the leftover x one at a time.
VectorXd VECTOR3_FIELD_3D::peeledProject(const MatrixXd& U) {
  const int xPeeled = _xRes - 2;
  const int slabPeeled = (_xRes - 2) * (_yRes - 2);
  const int totalColumns = U.cols();
  VectorXd final = VectorXd::Zero(totalColumns);
  VectorXd unroll[4];
  for (int k = 0; k < 4; k++) unroll[k].resize(totalColumns);
  const int stride = 4;
  for (int z = 0; z < _zRes - 2; z++) {
    const int zCached = 3 * z * slabPeeled;
    for (int y = 0; y < _yRes - 2; y++) {
      const int yzCached = 3 * y * xPeeled + zCached;
      const int xEnd = (_xRes - 2) / stride * stride;
      for (int k = 0; k < 4; k++) unroll[k].setZero();
      for (int x = 0; x < xEnd; x += stride)
        for (int k = 0; k < 4; k++) {
          const int index = 3 * (x + k) + yzCached;
          const VEC3F v3 = (*this)(x + k + 1, y + 1, z + 1);
          const Vector3d v(v3[0], v3[1], v3[2]);
          unroll[k].noalias() += U.block(index, 0, 3, totalColumns).transpose() * v;
        }
      for (int k = 0; k < 4; k++) final.noalias() += unroll[k];
      for (int x = xEnd; x < _xRes - 2; x++) {
        const int index = 3 * x + yzCached;
        const VEC3F v3 = (*this)(x + 1, y + 1, z + 1);
        const Vector3d v(v3[0], v3[1], v3[2]);
        final.noalias() += U.block(index, 0, 3, totalColumns).transpose() * v;
      }
    }
  }
  return final;
}

// VECTOR3_FIELD_3D.cpp:3558-3605: each peeled cell = (U row 3i, 3i+1, 3i+2) . q
void VECTOR3_FIELD_3D::peeledUnproject(const MatrixXd& U, const VectorXd& q) {
  const int xPeeled = _xRes - 2;
  const int slabPeeled = (_xRes - 2) * (_yRes - 2);
  for (int z = 0; z < _zRes - 2; z++) {
    const int zCached = 3 * z * slabPeeled;
    for (int y = 0; y < _yRes - 2; y++) {
      const int yzCached = 3 * y * xPeeled + zCached;
      for (int x = 0; x < _xRes - 2; x++) {
        const int index = 3 * x + yzCached;
        const Real fx = U.row(index).dot(q);
        const Real fy = U.row(index + 1).dot(q);
        const Real fz = U.row(index + 2).dot(q);
        (*this)(x + 1, y + 1, z + 1) = VEC3F(fx, fy, fz);
      }
    }
  }
}
