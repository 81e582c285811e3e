/*
 * Small value types with the names and operators PersianSPH drivers use
 * (Vec3_t, Mat3_t, Array<T>, String, Fatal, MECHSYS_CATCH), so that a driver
 * written against the reference's Domain.h compiles unchanged against this
 * library's SPH::Domain (include/persiansph/Domain.h).
 *
 * The reference gets these from blitz TinyVector/TinyMatrix and its own
 * External/ headers (External/matvec.h, External/array.h, External/fatal.h,
 * External/string.h). These are independent implementations of the same
 * interface: element access x(i) / M(i,j), blitz-style comma initialisation
 * (`v = a, b, c;`, and `v = s;` filling every element), element-wise
 * arithmetic, dot/norm, Array::Size/Push/Resize, String::Printf/CStr,
 * `throw new Fatal(fmt, ...)` caught by MECHSYS_CATCH.
 */
#ifndef PERSIANSPH_MATVEC_H
#define PERSIANSPH_MATVEC_H

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <iostream>
#include <string>
#include <vector>

class Vec3_t {
 public:
  Vec3_t() : d_{0.0, 0.0, 0.0} {}
  Vec3_t(double a, double b, double c) : d_{a, b, c} {}
  double& operator()(int i) { return d_[i]; }
  double operator()(int i) const { return d_[i]; }
  double& operator[](int i) { return d_[i]; }
  double operator[](int i) const { return d_[i]; }
  double* data() { return d_; }
  const double* data() const { return d_; }

  // `v = a, b, c;` sets the elements in turn; `v = s;` alone sets all three.
  class Init {
   public:
    Init(Vec3_t* v, int k, bool fill) : v_(v), k_(k), fill_(fill) {}
    Init operator,(double x) {
      fill_ = false;
      if (k_ < 3) v_->d_[k_] = x;
      return Init(v_, k_ + 1, false);
    }
    ~Init() {
      if (fill_) v_->d_[1] = v_->d_[2] = v_->d_[0];
    }

   private:
    Vec3_t* v_;
    int k_;
    bool fill_;
  };
  Init operator=(double x) {
    d_[0] = x;
    return Init(this, 1, true);
  }
  Vec3_t& operator=(const Vec3_t& o) = default;
  Vec3_t(const Vec3_t& o) = default;

  Vec3_t& operator+=(const Vec3_t& o) {
    for (int i = 0; i < 3; ++i) d_[i] += o.d_[i];
    return *this;
  }
  Vec3_t& operator-=(const Vec3_t& o) {
    for (int i = 0; i < 3; ++i) d_[i] -= o.d_[i];
    return *this;
  }
  Vec3_t& operator*=(double s) {
    for (int i = 0; i < 3; ++i) d_[i] *= s;
    return *this;
  }
  Vec3_t& operator/=(double s) {
    for (int i = 0; i < 3; ++i) d_[i] /= s;
    return *this;
  }

 private:
  double d_[3];
};

inline Vec3_t operator+(const Vec3_t& a, const Vec3_t& b) { return Vec3_t(a(0) + b(0), a(1) + b(1), a(2) + b(2)); }
inline Vec3_t operator-(const Vec3_t& a, const Vec3_t& b) { return Vec3_t(a(0) - b(0), a(1) - b(1), a(2) - b(2)); }
inline Vec3_t operator-(const Vec3_t& a) { return Vec3_t(-a(0), -a(1), -a(2)); }
inline Vec3_t operator*(double s, const Vec3_t& a) { return Vec3_t(s * a(0), s * a(1), s * a(2)); }
inline Vec3_t operator*(const Vec3_t& a, double s) { return Vec3_t(a(0) * s, a(1) * s, a(2) * s); }
inline Vec3_t operator/(const Vec3_t& a, double s) { return Vec3_t(a(0) / s, a(1) / s, a(2) / s); }
inline double dot(const Vec3_t& a, const Vec3_t& b) { return a(0) * b(0) + a(1) * b(1) + a(2) * b(2); }
inline double norm(const Vec3_t& a) { return std::sqrt(dot(a, a)); }

class Mat3_t {
 public:
  Mat3_t() {
    for (double& x : d_) x = 0.0;
  }
  double& operator()(int i, int j) { return d_[3 * i + j]; }
  double operator()(int i, int j) const { return d_[3 * i + j]; }
  double* data() { return d_; }
  const double* data() const { return d_; }

  class Init {
   public:
    Init(Mat3_t* m, int k, bool fill) : m_(m), k_(k), fill_(fill) {}
    Init operator,(double x) {
      fill_ = false;
      if (k_ < 9) m_->d_[k_] = x;
      return Init(m_, k_ + 1, false);
    }
    ~Init() {
      if (fill_)
        for (int k = 1; k < 9; ++k) m_->d_[k] = m_->d_[0];
    }

   private:
    Mat3_t* m_;
    int k_;
    bool fill_;
  };
  Init operator=(double x) {
    d_[0] = x;
    return Init(this, 1, true);
  }
  Mat3_t& operator=(const Mat3_t& o) = default;
  Mat3_t(const Mat3_t& o) = default;

 private:
  double d_[9];
};

inline void set_to_zero(Mat3_t& m) { m = 0.0; }
inline void set_to_zero(Vec3_t& v) { v = 0.0; }

template <class T>
class Array : public std::vector<T> {
 public:
  Array() {}
  explicit Array(size_t n) : std::vector<T>(n) {}
  size_t Size() const { return this->size(); }
  void Push(const T& x) { this->push_back(x); }
  void Resize(size_t n) { this->resize(n); }
  void Clear() { this->clear(); }
  T& Last() { return this->back(); }
};

class String : public std::string {
 public:
  String() {}
  String(const std::string& o) : std::string(o) {}
  String(const char* o) : std::string(o) {}
  int Printf(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    char buf[4096];
    const int n = vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    this->assign(buf);
    return n;
  }
  const char* CStr() const { return this->c_str(); }
};

class Fatal {
 public:
  explicit Fatal(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    char buf[4096];
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    msg_ = buf;
  }
  void Cout() const { std::printf("Fatal: %s\n", msg_.c_str()); }
  String Msg() const { return msg_; }

 private:
  String msg_;
};

#define MECHSYS_CATCH                                            \
  catch (Fatal * e) {                                            \
    e->Cout();                                                   \
    delete e;                                                    \
    return 1;                                                    \
  }                                                              \
  catch (char const* m) {                                        \
    std::printf("Fatal: %s\n", m);                               \
    return 1;                                                    \
  }                                                              \
  catch (std::exception & e) {                                   \
    std::printf("Fatal: %s\n", e.what());                        \
    return 1;                                                    \
  }                                                              \
  catch (...) {                                                  \
    std::printf("Fatal: Some exception (...) occurred\n");      \
    return 1;                                                    \
  }

#endif  // PERSIANSPH_MATVEC_H
