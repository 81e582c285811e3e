/*
 * Minimal stand-in for blitz-0.9's TinyVector, written for this project so that
 * the reference's header-only sources compile in a container without blitz.
 * TEST INFRASTRUCTURE ONLY: used to build the reference itself as the parity
 * oracle (oracle/_ref); nothing in the product includes it.
 *
 * It provides exactly the TinyVector surface the reference uses: element
 * access, scalar broadcast and comma initialisation, element-wise + - * /,
 * compound assignment, dot() and norm(). Element-wise expressions evaluate
 * per element in source order, which is what blitz's expression templates do;
 * dot() sums the three products left to right (blitz unrolls the same three
 * products; only the association of the two additions may differ, a last-bit
 * effect far below the 1e-12 parity tolerance).
 */
#ifndef PSPH_SHIM_BLITZ_TINYVEC_H
#define PSPH_SHIM_BLITZ_TINYVEC_H

#include <cmath>
#include <cstddef>
#include <iostream>

namespace blitz {

template <typename T, int N>
class TinyVector;

/* Comma initialiser: "V = a, b, c;" assigns successive elements. */
template <typename T, int N>
class TinyVecCommaInit {
 public:
  TinyVecCommaInit(TinyVector<T, N>* v, int next) : v_(v), i_(next) {}
  TinyVecCommaInit& operator,(T value) {
    if (i_ < N) (*v_)[i_] = value;
    ++i_;
    return *this;
  }

 private:
  TinyVector<T, N>* v_;
  int i_;
};

template <typename T, int N>
class TinyVector {
 public:
  typedef T T_numtype;
  TinyVector() {
    for (int i = 0; i < N; ++i) d_[i] = T();
  }
  TinyVector(T s) {  // implicit: "Vec3_t v = 0.0;" broadcasts
    for (int i = 0; i < N; ++i) d_[i] = s;
  }
  TinyVector(T a, T b) {
    d_[0] = a;
    d_[1] = b;
  }
  TinyVector(T a, T b, T c) {
    d_[0] = a;
    d_[1] = b;
    d_[2] = c;
  }
  TinyVector(const TinyVector& o) {
    for (int i = 0; i < N; ++i) d_[i] = o.d_[i];
  }
  TinyVector& operator=(const TinyVector& o) {
    for (int i = 0; i < N; ++i) d_[i] = o.d_[i];
    return *this;
  }
  TinyVecCommaInit<T, N> operator=(T s) {
    for (int i = 0; i < N; ++i) d_[i] = s;
    return TinyVecCommaInit<T, N>(this, 1);
  }

  T& operator()(int i) { return d_[i]; }
  const T& operator()(int i) const { return d_[i]; }
  T& operator[](int i) { return d_[i]; }
  const T& operator[](int i) const { return d_[i]; }
  T* data() { return d_; }
  const T* data() const { return d_; }
  static int length() { return N; }

  TinyVector& operator+=(const TinyVector& o) {
    for (int i = 0; i < N; ++i) d_[i] += o.d_[i];
    return *this;
  }
  TinyVector& operator-=(const TinyVector& o) {
    for (int i = 0; i < N; ++i) d_[i] -= o.d_[i];
    return *this;
  }
  TinyVector& operator*=(T s) {
    for (int i = 0; i < N; ++i) d_[i] *= s;
    return *this;
  }
  TinyVector& operator/=(T s) {
    for (int i = 0; i < N; ++i) d_[i] /= s;
    return *this;
  }
  TinyVector& operator+=(T s) {
    for (int i = 0; i < N; ++i) d_[i] += s;
    return *this;
  }
  TinyVector& operator-=(T s) {
    for (int i = 0; i < N; ++i) d_[i] -= s;
    return *this;
  }

 private:
  T d_[N];
};

#define PSPH_TV_BINOP(OP)                                                          \
  template <typename T, int N>                                                     \
  inline TinyVector<T, N> operator OP(const TinyVector<T, N>& a,                   \
                                      const TinyVector<T, N>& b) {                 \
    TinyVector<T, N> r;                                                            \
    for (int i = 0; i < N; ++i) r[i] = a[i] OP b[i];                               \
    return r;                                                                      \
  }                                                                                \
  template <typename T, int N>                                                     \
  inline TinyVector<T, N> operator OP(const TinyVector<T, N>& a, double s) {       \
    TinyVector<T, N> r;                                                            \
    for (int i = 0; i < N; ++i) r[i] = a[i] OP s;                                  \
    return r;                                                                      \
  }                                                                                \
  template <typename T, int N>                                                     \
  inline TinyVector<T, N> operator OP(double s, const TinyVector<T, N>& a) {       \
    TinyVector<T, N> r;                                                            \
    for (int i = 0; i < N; ++i) r[i] = s OP a[i];                                  \
    return r;                                                                      \
  }

PSPH_TV_BINOP(+)
PSPH_TV_BINOP(-)
PSPH_TV_BINOP(*)
PSPH_TV_BINOP(/)
#undef PSPH_TV_BINOP

template <typename T, int N>
inline TinyVector<T, N> operator-(const TinyVector<T, N>& a) {
  TinyVector<T, N> r;
  for (int i = 0; i < N; ++i) r[i] = -a[i];
  return r;
}

template <typename T, int N>
inline T dot(const TinyVector<T, N>& a, const TinyVector<T, N>& b) {
  T s = a[0] * b[0];
  for (int i = 1; i < N; ++i) s = s + a[i] * b[i];
  return s;
}

template <typename T, int N>
inline T sum(const TinyVector<T, N>& a) {
  T s = a[0];
  for (int i = 1; i < N; ++i) s = s + a[i];
  return s;
}

template <typename T, int N>
inline T norm(const TinyVector<T, N>& a) {
  return std::sqrt(dot(a, a));
}

template <typename T, int N>
inline TinyVector<T, N> cross(const TinyVector<T, N>& a, const TinyVector<T, N>& b) {
  TinyVector<T, N> r;
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
  return r;
}

template <typename T, int N>
inline std::ostream& operator<<(std::ostream& os, const TinyVector<T, N>& v) {
  os << "(";
  for (int i = 0; i < N; ++i) os << (i ? "," : "") << v[i];
  return os << ")";
}

}  // namespace blitz

using blitz::dot;
using blitz::norm;

#endif
