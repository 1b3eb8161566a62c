// Minimal fixed-size dense-matrix header providing the subset of the Eigen 3
// API that MST-CFD's density-based path uses, so that the reference's own
// sources compile here (Eigen is not installed and cannot be fetched).
//
// TEST INFRASTRUCTURE ONLY: this header is used solely to build the reference
// oracle under oracle/_ref.  It is written from the documented Eigen API
// semantics, not from Eigen's sources, and it fixes the arithmetic order of
// every reduction, so that the CUDA parity kernels can follow the same order:
//
//   * products        c_ij = a_i0*b_0j, then += a_ik*b_kj for k = 1..K-1
//   * dot / norm      s = x_0*y_0, then += x_k*y_k ascending; norm = sqrt(s)
//   * inverse (2..4)  adjugate (cofactor) formula: each 3x3 minor by
//                     first-row expansion a(ei-fh) - b(di-fg) + c(dh-eg),
//                     det = sum_j a_0j*C_0j (j ascending),
//                     inv_ij = C_ji * (1/det)
//   * scalar ops      coefficient-wise, no reassociation
//
// Real Eigen may vectorise reductions (pairwise order) and uses its own 4x4
// inverse, so results are pinned to this header, not to a particular Eigen.
#pragma once
// Eigen/Core pulls these standard headers in; the reference relies on that.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <iostream>
#include <limits>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

namespace Eigen {

template <typename T, int R, int C>
class Matrix;

template <typename T, int R, int C>
class ColRef {
 public:
  ColRef(Matrix<T, R, C>& m, int j) : m_(m), j_(j) {}
  ColRef& operator=(const Matrix<T, R, 1>& v) {
    for (int i = 0; i < R; ++i) m_(i, j_) = v(i);
    return *this;
  }
  ColRef& operator+=(const Matrix<T, R, 1>& v) {
    for (int i = 0; i < R; ++i) m_(i, j_) += v(i);
    return *this;
  }
  ColRef& operator-=(const Matrix<T, R, 1>& v) {
    for (int i = 0; i < R; ++i) m_(i, j_) -= v(i);
    return *this;
  }
  Matrix<T, R, 1> eval() const {
    Matrix<T, R, 1> v;
    for (int i = 0; i < R; ++i) v(i) = m_(i, j_);
    return v;
  }
  operator Matrix<T, R, 1>() const { return eval(); }

 private:
  Matrix<T, R, C>& m_;
  int j_;
};

template <typename T, int R, int C>
class RowRef {
 public:
  RowRef(Matrix<T, R, C>& m, int i) : m_(m), i_(i) {}
  RowRef& operator=(const Matrix<T, 1, C>& v) {
    for (int j = 0; j < C; ++j) m_(i_, j) = v(0, j);
    return *this;
  }
  Matrix<T, 1, C> eval() const {
    Matrix<T, 1, C> v;
    for (int j = 0; j < C; ++j) v(0, j) = m_(i_, j);
    return v;
  }
  operator Matrix<T, 1, C>() const { return eval(); }

 private:
  Matrix<T, R, C>& m_;
  int i_;
};

template <typename T, int R, int C>
class CommaInit {
 public:
  CommaInit(Matrix<T, R, C>& m, T first) : m_(m), k_(0) { put(first); }
  template <typename S>
  CommaInit& operator,(const S& x) {
    put(static_cast<T>(x));
    return *this;
  }

 private:
  void put(T x) {
    // Row-major fill, as Eigen's comma initializer does.
    if (k_ < R * C) m_(k_ / C, k_ % C) = x;
    ++k_;
  }
  Matrix<T, R, C>& m_;
  int k_;
};

template <typename T, int R, int C>
class Matrix {
 public:
  Matrix() {}
  static Matrix Zero() {
    Matrix m;
    for (int k = 0; k < R * C; ++k) m.v_[k] = T(0);
    return m;
  }
  static Matrix Identity() {
    Matrix m = Zero();
    for (int k = 0; k < (R < C ? R : C); ++k) m(k, k) = T(1);
    return m;
  }
  // column-major storage
  T& operator()(int i, int j) { return v_[j * R + i]; }
  const T& operator()(int i, int j) const { return v_[j * R + i]; }
  T& operator()(int k) { return v_[k]; }
  const T& operator()(int k) const { return v_[k]; }
  T& operator[](int k) { return v_[k]; }
  const T& operator[](int k) const { return v_[k]; }

  int rows() const { return R; }
  int cols() const { return C; }
  int size() const { return R * C; }

  ColRef<T, R, C> col(int j) { return ColRef<T, R, C>(*this, j); }
  Matrix<T, R, 1> col(int j) const {
    Matrix<T, R, 1> v;
    for (int i = 0; i < R; ++i) v(i) = (*this)(i, j);
    return v;
  }
  RowRef<T, R, C> row(int i) { return RowRef<T, R, C>(*this, i); }
  Matrix<T, 1, C> row(int i) const {
    Matrix<T, 1, C> v;
    for (int j = 0; j < C; ++j) v(0, j) = (*this)(i, j);
    return v;
  }

  Matrix<T, C, R> transpose() const {
    Matrix<T, C, R> t;
    for (int i = 0; i < R; ++i)
      for (int j = 0; j < C; ++j) t(j, i) = (*this)(i, j);
    return t;
  }

  T squaredNorm() const {
    T s = v_[0] * v_[0];
    for (int k = 1; k < R * C; ++k) s += v_[k] * v_[k];
    return s;
  }
  T norm() const { return std::sqrt(squaredNorm()); }
  T dot(const Matrix& o) const {
    T s = v_[0] * o.v_[0];
    for (int k = 1; k < R * C; ++k) s += v_[k] * o.v_[k];
    return s;
  }
  Matrix cross(const Matrix& o) const {
    Matrix r = Zero();
    if (R * C == 3) {
      r(0) = v_[1] * o.v_[2] - v_[2] * o.v_[1];
      r(1) = v_[2] * o.v_[0] - v_[0] * o.v_[2];
      r(2) = v_[0] * o.v_[1] - v_[1] * o.v_[0];
    }
    return r;
  }
  T sum() const {
    T s = v_[0];
    for (int k = 1; k < R * C; ++k) s += v_[k];
    return s;
  }

  Matrix inverse() const;

  // 1x1 results of row*column products convert to their scalar
  operator T() const
    requires(R == 1 && C == 1)
  {
    return v_[0];
  }

  template <typename S, typename = std::enable_if_t<std::is_arithmetic_v<S>>>
  CommaInit<T, R, C> operator<<(const S& first) {
    return CommaInit<T, R, C>(*this, static_cast<T>(first));
  }

  Matrix& operator+=(const Matrix& o) {
    for (int k = 0; k < R * C; ++k) v_[k] += o.v_[k];
    return *this;
  }
  Matrix& operator-=(const Matrix& o) {
    for (int k = 0; k < R * C; ++k) v_[k] -= o.v_[k];
    return *this;
  }
  template <typename S, typename = std::enable_if_t<std::is_arithmetic_v<S>>>
  Matrix& operator*=(S s) {
    for (int k = 0; k < R * C; ++k) v_[k] *= static_cast<T>(s);
    return *this;
  }
  template <typename S, typename = std::enable_if_t<std::is_arithmetic_v<S>>>
  Matrix& operator/=(S s) {
    for (int k = 0; k < R * C; ++k) v_[k] /= static_cast<T>(s);
    return *this;
  }
  Matrix operator-() const {
    Matrix r;
    for (int k = 0; k < R * C; ++k) r.v_[k] = -v_[k];
    return r;
  }

 private:
  T v_[R * C];
};

template <typename T, int R, int C>
Matrix<T, R, C> operator+(const Matrix<T, R, C>& a, const Matrix<T, R, C>& b) {
  Matrix<T, R, C> r;
  for (int k = 0; k < R * C; ++k) r(k) = a(k) + b(k);
  return r;
}
template <typename T, int R, int C>
Matrix<T, R, C> operator-(const Matrix<T, R, C>& a, const Matrix<T, R, C>& b) {
  Matrix<T, R, C> r;
  for (int k = 0; k < R * C; ++k) r(k) = a(k) - b(k);
  return r;
}
template <typename S, typename T, int R, int C,
          typename = std::enable_if_t<std::is_arithmetic_v<S>>>
Matrix<T, R, C> operator*(S s, const Matrix<T, R, C>& a) {
  Matrix<T, R, C> r;
  for (int k = 0; k < R * C; ++k) r(k) = static_cast<T>(s) * a(k);
  return r;
}
template <typename S, typename T, int R, int C,
          typename = std::enable_if_t<std::is_arithmetic_v<S>>>
Matrix<T, R, C> operator*(const Matrix<T, R, C>& a, S s) {
  Matrix<T, R, C> r;
  for (int k = 0; k < R * C; ++k) r(k) = a(k) * static_cast<T>(s);
  return r;
}
template <typename S, typename T, int R, int C,
          typename = std::enable_if_t<std::is_arithmetic_v<S>>>
Matrix<T, R, C> operator/(const Matrix<T, R, C>& a, S s) {
  Matrix<T, R, C> r;
  for (int k = 0; k < R * C; ++k) r(k) = a(k) / static_cast<T>(s);
  return r;
}
template <typename T, int R, int K, int C>
Matrix<T, R, C> operator*(const Matrix<T, R, K>& a, const Matrix<T, K, C>& b) {
  Matrix<T, R, C> r;
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) {
      T s = a(i, 0) * b(0, j);
      for (int k = 1; k < K; ++k) s += a(i, k) * b(k, j);
      r(i, j) = s;
    }
  return r;
}
// column views used as vectors
template <typename S, typename T, int R, int C,
          typename = std::enable_if_t<std::is_arithmetic_v<S>>>
Matrix<T, R, 1> operator*(S s, const ColRef<T, R, C>& c) {
  return s * c.eval();
}
template <typename S, typename T, int R, int C,
          typename = std::enable_if_t<std::is_arithmetic_v<S>>>
Matrix<T, R, 1> operator*(const ColRef<T, R, C>& c, S s) {
  return c.eval() * s;
}

namespace shim_detail {
template <typename T>
inline T det3(T a, T b, T c, T d, T e, T f, T g, T h, T i) {
  return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}
}  // namespace shim_detail

template <typename T, int R, int C>
Matrix<T, R, C> Matrix<T, R, C>::inverse() const {
  static_assert(R == C, "inverse of a non-square matrix");
  Matrix<T, R, C> inv;
  const Matrix& a = *this;
  if constexpr (R == 1) {
    inv(0, 0) = T(1) / a(0, 0);
  } else if constexpr (R == 2) {
    T det = a(0, 0) * a(1, 1) - a(0, 1) * a(1, 0);
    T id = T(1) / det;
    inv(0, 0) = a(1, 1) * id;
    inv(0, 1) = -a(0, 1) * id;
    inv(1, 0) = -a(1, 0) * id;
    inv(1, 1) = a(0, 0) * id;
  } else if constexpr (R == 3) {
    T cof[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        int r0 = (i == 0) ? 1 : 0, r1 = (i == 2) ? 1 : 2;
        int c0 = (j == 0) ? 1 : 0, c1 = (j == 2) ? 1 : 2;
        T m = a(r0, c0) * a(r1, c1) - a(r0, c1) * a(r1, c0);
        cof[i][j] = ((i + j) & 1) ? -m : m;
      }
    T det = a(0, 0) * cof[0][0] + a(0, 1) * cof[0][1] + a(0, 2) * cof[0][2];
    T id = T(1) / det;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) inv(i, j) = cof[j][i] * id;
  } else if constexpr (R == 4) {
    T cof[4][4];
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        int rr[3], cc[3];
        for (int k = 0, n = 0; k < 4; ++k)
          if (k != i) rr[n++] = k;
        for (int k = 0, n = 0; k < 4; ++k)
          if (k != j) cc[n++] = k;
        T m = shim_detail::det3(a(rr[0], cc[0]), a(rr[0], cc[1]), a(rr[0], cc[2]),
                                a(rr[1], cc[0]), a(rr[1], cc[1]), a(rr[1], cc[2]),
                                a(rr[2], cc[0]), a(rr[2], cc[1]), a(rr[2], cc[2]));
        cof[i][j] = ((i + j) & 1) ? -m : m;
      }
    T det = a(0, 0) * cof[0][0];
    for (int j = 1; j < 4; ++j) det += a(0, j) * cof[0][j];
    T id = T(1) / det;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) inv(i, j) = cof[j][i] * id;
  } else {
    // Gauss-Jordan with partial pivoting for larger blocks (not on the
    // 2D reference path).
    Matrix<T, R, 2 * R> w;
    for (int i = 0; i < R; ++i)
      for (int j = 0; j < 2 * R; ++j)
        w(i, j) = (j < R) ? a(i, j) : (j - R == i ? T(1) : T(0));
    for (int p = 0; p < R; ++p) {
      int best = p;
      for (int i = p + 1; i < R; ++i)
        if (std::fabs(w(i, p)) > std::fabs(w(best, p))) best = i;
      if (best != p)
        for (int j = 0; j < 2 * R; ++j) {
          T t = w(p, j);
          w(p, j) = w(best, j);
          w(best, j) = t;
        }
      T piv = w(p, p);
      for (int j = 0; j < 2 * R; ++j) w(p, j) /= piv;
      for (int i = 0; i < R; ++i)
        if (i != p) {
          T f = w(i, p);
          for (int j = 0; j < 2 * R; ++j) w(i, j) -= f * w(p, j);
        }
    }
    for (int i = 0; i < R; ++i)
      for (int j = 0; j < R; ++j) inv(i, j) = w(i, j + R);
  }
  return inv;
}

template <typename T, int R, int C>
std::ostream& operator<<(std::ostream& os, const Matrix<T, R, C>& m) {
  for (int i = 0; i < R; ++i) {
    for (int j = 0; j < C; ++j) {
      if (j) os << ' ';
      os << m(i, j);
    }
    if (i + 1 < R) os << '\n';
  }
  return os;
}

typedef Matrix<double, 2, 1> Vector2d;
typedef Matrix<double, 3, 1> Vector3d;
typedef Matrix<double, 4, 1> Vector4d;
typedef Matrix<double, 4, 4> Matrix4d;

}  // namespace Eigen
