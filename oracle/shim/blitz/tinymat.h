/*
 * Minimal stand-in for blitz-0.9's TinyMatrix, written for this project (see
 * tinyvec-et.h). TEST INFRASTRUCTURE ONLY: builds the reference as the parity
 * oracle. Row-major storage, element access M(i,j), data(), scalar broadcast
 * and comma initialisation ("M = a, b, c, ...;"). The reference defines its own
 * Mat3_t + - and scalar* operators (External/matvec.h:549-575), so none are
 * declared here.
 */
#ifndef PSPH_SHIM_BLITZ_TINYMAT_H
#define PSPH_SHIM_BLITZ_TINYMAT_H

#include <iostream>

#include "tinyvec-et.h"

namespace blitz {

template <typename T, int R, int C>
class TinyMatrix;

template <typename T, int R, int C>
class TinyMatCommaInit {
 public:
  TinyMatCommaInit(TinyMatrix<T, R, C>* m, int next) : m_(m), i_(next) {}
  TinyMatCommaInit& operator,(T value) {
    if (i_ < R * C) m_->data()[i_] = value;
    ++i_;
    return *this;
  }

 private:
  TinyMatrix<T, R, C>* m_;
  int i_;
};

template <typename T, int R, int C>
class TinyMatrix {
 public:
  typedef T T_numtype;
  TinyMatrix() {
    for (int i = 0; i < R * C; ++i) d_[i] = T();
  }
  TinyMatrix(const TinyMatrix& o) {
    for (int i = 0; i < R * C; ++i) d_[i] = o.d_[i];
  }
  TinyMatrix& operator=(const TinyMatrix& o) {
    for (int i = 0; i < R * C; ++i) d_[i] = o.d_[i];
    return *this;
  }
  TinyMatCommaInit<T, R, C> operator=(T s) {
    for (int i = 0; i < R * C; ++i) d_[i] = s;
    return TinyMatCommaInit<T, R, C>(this, 1);
  }
  T& operator()(int i, int j) { return d_[i * C + j]; }
  const T& operator()(int i, int j) const { return d_[i * C + j]; }
  T* data() { return d_; }
  const T* data() const { return d_; }
  static int rows() { return R; }
  static int columns() { return C; }

 private:
  T d_[R * C];
};

template <typename T, int R, int C>
inline std::ostream& operator<<(std::ostream& os, const TinyMatrix<T, R, C>& m) {
  for (int i = 0; i < R; ++i) {
    for (int j = 0; j < C; ++j) os << m(i, j) << (j + 1 < C ? " " : "");
    os << "\n";
  }
  return os;
}

}  // namespace blitz

#endif
