// RenderToy/rtmath.h — math types of the RenderToy-compatible C++ API.
//
// Same names, members and results as RenderToy's include/RenderToy/rtmath.h
// (Vector, Matrix, Convert, AffineTransformation, convolution kernels), so a
// program written against RenderToy compiles unchanged.  Arithmetic keeps the
// reference's evaluation order (dot products accumulate from zero, matrix
// products sum k = 0..N-1) so that cameras and world-space vertices computed
// here equal the reference's; build with -ffp-contract=off for that.
// Vector<float, 3> is three packed floats, as RenderContext::buffer requires.
#ifndef RTX_COMPAT_RTMATH_H
#define RTX_COMPAT_RTMATH_H

#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <initializer_list>
#include <istream>
#include <type_traits>
#include <vector>

namespace RenderToy {

template <typename T = float>
inline constexpr T kPi = T(3.14159265358979323846L);
inline constexpr float kFloatEpsilon = 1e-7f;
inline constexpr float kFloatInfinity = 1e7f;

enum class Orientation { X = 0, Y = 1, All = 2 };

template <typename T, std::size_t N>
struct Vector;
template <typename T, std::size_t N>
struct Matrix;

template <typename T, std::size_t N>
struct VectorConstants {};

template <typename T>
struct VectorConstants<T, 2> {
  static const Vector<T, 2> O, X, Y;
};
template <typename T>
struct VectorConstants<T, 3> {
  static const Vector<T, 3> O, X, Y, Z, White;
};
template <typename T>
struct VectorConstants<T, 4> {
  static const Vector<T, 4> O, X, Y, Z, W;
};

template <typename T, std::size_t N>
struct Vector : public VectorConstants<T, N> {
  std::array<T, N> arr = {};

  constexpr Vector() = default;
  template <typename... A>
    requires(sizeof...(A) == N && N > 1)
  constexpr Vector(A&&... v) : arr{static_cast<T>(std::forward<A>(v))...} {}
  Vector(const T& v) { arr.fill(v); }

  constexpr const T& operator[](std::size_t i) const { return arr[i]; }
  constexpr T& operator[](std::size_t i) { return arr[i]; }
  constexpr T& x() { return arr[0]; }
  constexpr const T& x() const { return arr[0]; }
  constexpr T& y() requires(N > 1) { return arr[1]; }
  constexpr const T& y() const requires(N > 1) { return arr[1]; }
  constexpr T& z() requires(N > 2) { return arr[2]; }
  constexpr const T& z() const requires(N > 2) { return arr[2]; }
  constexpr T& w() requires(N > 3) { return arr[3]; }
  constexpr const T& w() const requires(N > 3) { return arr[3]; }

  bool IsZero() const {
    for (T a : arr)
      if (std::abs(a) > kFloatEpsilon) return false;
    return true;
  }
  static Vector Abs(const Vector& v) {
    Vector r;
    for (std::size_t i = 0; i < N; ++i) r.arr[i] = std::abs(v.arr[i]);
    return r;
  }
  T Length2() const {
    T r = T(0);
    for (T a : arr) r += a * a;
    return r;
  }
  T Length() const { return std::sqrt(Length2()); }
  void Normalize() {
    T l = Length();
    for (T& a : arr) a /= l;
  }
  Vector Normalized() const {
    Vector r(*this);
    r.Normalize();
    return r;
  }
  Vector Normalized_s() const { return IsZero() ? Vector() : Normalized(); }

  Vector operator+(const Vector& b) const {
    Vector r;
    for (std::size_t i = 0; i < N; ++i) r.arr[i] = arr[i] + b.arr[i];
    return r;
  }
  Vector operator-(const Vector& b) const {
    Vector r;
    for (std::size_t i = 0; i < N; ++i) r.arr[i] = arr[i] - b.arr[i];
    return r;
  }
  Vector operator-() const {
    Vector r;
    for (std::size_t i = 0; i < N; ++i) r.arr[i] = -arr[i];
    return r;
  }
  Vector operator*(const T s) const {
    Vector r;
    for (std::size_t i = 0; i < N; ++i) r.arr[i] = arr[i] * s;
    return r;
  }
  Vector operator*(const Vector& b) const {
    Vector r;
    for (std::size_t i = 0; i < N; ++i) r.arr[i] = arr[i] * b.arr[i];
    return r;
  }
  Vector operator/(const T s) const {
    Vector r;
    for (std::size_t i = 0; i < N; ++i) r.arr[i] = arr[i] / s;
    return r;
  }
  Vector operator/(const Vector& b) const {
    Vector r;
    for (std::size_t i = 0; i < N; ++i) r.arr[i] = arr[i] / b.arr[i];
    return r;
  }
  const Vector& operator+=(const Vector& b) {
    for (std::size_t i = 0; i < N; ++i) arr[i] += b.arr[i];
    return *this;
  }
  const Vector& operator-=(const Vector& b) {
    for (std::size_t i = 0; i < N; ++i) arr[i] -= b.arr[i];
    return *this;
  }
  const Vector& operator*=(const T s) {
    for (T& a : arr) a *= s;
    return *this;
  }
  const Vector& operator/=(const T s) {
    for (T& a : arr) a /= s;
    return *this;
  }
  // epsilon comparison, as the reference's
  bool operator==(const Vector& b) const {
    for (std::size_t i = 0; i < N; ++i)
      if (std::abs(arr[i] - b.arr[i]) > kFloatEpsilon) return false;
    return true;
  }
  bool operator!=(const Vector& b) const { return !(*this == b); }

  static T Dot(const Vector& a, const Vector& b) {
    T r(0);
    for (std::size_t i = 0; i < N; ++i) r += a.arr[i] * b.arr[i];
    return r;
  }
  T Dot(const Vector& b) const { return Dot(*this, b); }
  static Vector Pow(const Vector& a, const Vector& b) {
    Vector r;
    for (std::size_t i = 0; i < N; ++i) r.arr[i] = std::pow(a.arr[i], b.arr[i]);
    return r;
  }
  static Vector Log(const Vector& a) {
    Vector r;
    for (std::size_t i = 0; i < N; ++i) r.arr[i] = std::log(a.arr[i]);
    return r;
  }
  static constexpr Vector Cross(const Vector& a, const Vector& b) requires(N == 3) {
    return Vector(a.arr[1] * b.arr[2] - a.arr[2] * b.arr[1], a.arr[2] * b.arr[0] - a.arr[0] * b.arr[2],
                  a.arr[0] * b.arr[1] - a.arr[1] * b.arr[0]);
  }
  constexpr Vector Cross(const Vector& b) const requires(N == 3) { return Cross(*this, b); }

  Vector TransformEach(const std::function<T(T)>& f) const {
    Vector r;
    for (std::size_t i = 0; i < N; ++i) r.arr[i] = f(arr[i]);
    return r;
  }
  Vector Floor() const { return TransformEach([](T v) { return T(std::floor(v)); }); }
  Vector Fract() const { return TransformEach([](T v) { return v - T(std::floor(v)); }); }
  Vector Sin() const { return TransformEach([](T v) { return T(std::sin(v)); }); }
  Vector Cos() const { return TransformEach([](T v) { return T(std::cos(v)); }); }

  friend Vector operator*(const float s, const Vector& a) {
    Vector r(a);
    for (auto& v : r.arr) v *= s;
    return r;
  }
  friend std::istream& operator>>(std::istream& is, Vector& a) {
    for (std::size_t i = 0; i < N; ++i) is >> a.arr[i];
    return is;
  }
};

template <typename T>
const Vector<T, 2> VectorConstants<T, 2>::O = Vector<T, 2>(T(0), T(0));
template <typename T>
const Vector<T, 2> VectorConstants<T, 2>::X = Vector<T, 2>(T(1), T(0));
template <typename T>
const Vector<T, 2> VectorConstants<T, 2>::Y = Vector<T, 2>(T(0), T(1));
template <typename T>
const Vector<T, 3> VectorConstants<T, 3>::O = Vector<T, 3>(T(0), T(0), T(0));
template <typename T>
const Vector<T, 3> VectorConstants<T, 3>::X = Vector<T, 3>(T(1), T(0), T(0));
template <typename T>
const Vector<T, 3> VectorConstants<T, 3>::Y = Vector<T, 3>(T(0), T(1), T(0));
template <typename T>
const Vector<T, 3> VectorConstants<T, 3>::Z = Vector<T, 3>(T(0), T(0), T(1));
template <typename T>
const Vector<T, 3> VectorConstants<T, 3>::White = Vector<T, 3>(T(1), T(1), T(1));
template <typename T>
const Vector<T, 4> VectorConstants<T, 4>::O = Vector<T, 4>(T(0), T(0), T(0), T(0));
template <typename T>
const Vector<T, 4> VectorConstants<T, 4>::X = Vector<T, 4>(T(1), T(0), T(0), T(0));
template <typename T>
const Vector<T, 4> VectorConstants<T, 4>::Y = Vector<T, 4>(T(0), T(1), T(0), T(0));
template <typename T>
const Vector<T, 4> VectorConstants<T, 4>::Z = Vector<T, 4>(T(0), T(0), T(1), T(0));
template <typename T>
const Vector<T, 4> VectorConstants<T, 4>::W = Vector<T, 4>(T(0), T(0), T(0), T(1));

template <typename T>
using Vector2 = Vector<T, 2>;
template <typename T>
using Vector3 = Vector<T, 3>;
template <typename T>
using Vector4 = Vector<T, 4>;
using Vector2f = Vector2<float>;
using Vector3f = Vector3<float>;
using Vector4f = Vector4<float>;
using Vector2d = Vector2<double>;
using Vector3d = Vector3<double>;
using Vector4d = Vector4<double>;
static_assert(sizeof(Vector3f) == 12, "Vector3f must be three packed floats");

template <typename T, std::size_t N>
struct MatrixConstants {
  static const Matrix<T, N> I, O;
};

template <typename T, std::size_t N>
struct Matrix : public MatrixConstants<T, N> {
  using VectorType = Vector<T, N>;
  std::array<VectorType, N> row = {};

  constexpr Matrix() = default;
  constexpr Matrix(const VectorType& r0, const VectorType& r1) requires(N == 2) : row{r0, r1} {}
  constexpr Matrix(const VectorType& r0, const VectorType& r1, const VectorType& r2) requires(N == 3)
      : row{r0, r1, r2} {}
  constexpr Matrix(const VectorType& r0, const VectorType& r1, const VectorType& r2,
                   const VectorType& r3) requires(N == 4)
      : row{r0, r1, r2, r3} {}
  constexpr Matrix(const std::array<VectorType, N>& rows) : row(rows) {}

  constexpr VectorType& operator[](std::size_t i) { return row[i]; }
  constexpr const VectorType& operator[](std::size_t i) const { return row[i]; }
  bool operator==(const Matrix& b) const {
    for (std::size_t i = 0; i < N; ++i)
      if (row[i] != b.row[i]) return false;
    return true;
  }
  bool operator!=(const Matrix& b) const { return !(*this == b); }
  Matrix operator+(const Matrix& b) const {
    Matrix r;
    for (std::size_t i = 0; i < N; ++i) r.row[i] = row[i] + b.row[i];
    return r;
  }
  Matrix operator-(const Matrix& b) const {
    Matrix r;
    for (std::size_t i = 0; i < N; ++i) r.row[i] = row[i] - b.row[i];
    return r;
  }
  Matrix operator-() const {
    Matrix r;
    for (std::size_t i = 0; i < N; ++i) r.row[i] = -row[i];
    return r;
  }
  // each output component is the row's dot product, accumulated from zero
  VectorType operator*(const VectorType& v) const {
    VectorType r;
    for (std::size_t i = 0; i < N; ++i) r.arr[i] = row[i].Dot(v);
    return r;
  }
  Matrix operator*(const Matrix& b) const {
    Matrix r;
    for (std::size_t i = 0; i < N; ++i)
      for (std::size_t j = 0; j < N; ++j)
        for (std::size_t k = 0; k < N; ++k) r.row[i][j] += row[i][k] * b.row[k][j];
    return r;
  }
  Matrix Transposed() const {
    Matrix r;
    for (std::size_t i = 0; i < N; ++i)
      for (std::size_t j = 0; j < N; ++j) r.row[i][j] = row[j][i];
    return r;
  }
  void Transpose() { *this = Transposed(); }
  Matrix<T, N - 1> ComplementMinor(std::size_t ri, std::size_t ci) const requires(N >= 3) {
    Matrix<T, N - 1> r;
    for (std::size_t x = 0, rx = 0; x < N; ++x) {
      if (x == ri) continue;
      for (std::size_t y = 0, ry = 0; y < N; ++y) {
        if (y == ci) continue;
        r[rx][ry++] = row[x][y];
      }
      ++rx;
    }
    return r;
  }
  static constexpr float Determinant(const Matrix& m) requires(N == 2) {
    return m.row[0][0] * m.row[1][1] - m.row[0][1] * m.row[1][0];
  }
  static constexpr float Determinant(const Matrix& m) requires(N == 3) {
    return m.row[0][0] * m.row[1][1] * m.row[2][2] + m.row[0][1] * m.row[1][2] * m.row[2][0] +
           m.row[0][2] * m.row[1][0] * m.row[2][1] - m.row[0][2] * m.row[1][1] * m.row[2][0] -
           m.row[0][0] * m.row[1][2] * m.row[2][1] - m.row[2][2] * m.row[0][1] * m.row[1][0];
  }
};

template <typename T, std::size_t N>
constexpr Matrix<T, N> make_identity() {
  Matrix<T, N> m;
  for (std::size_t i = 0; i < N; ++i) m.row[i][i] = T(1);
  return m;
}
template <typename T, std::size_t N>
const Matrix<T, N> MatrixConstants<T, N>::I = make_identity<T, N>();
template <typename T, std::size_t N>
const Matrix<T, N> MatrixConstants<T, N>::O = Matrix<T, N>();

using Matrix2x2f = Matrix<float, 2>;
using Matrix3x3f = Matrix<float, 3>;
using Matrix4x4f = Matrix<float, 4>;
using Matrix2x2d = Matrix<double, 2>;
using Matrix3x3d = Matrix<double, 3>;
using Matrix4x4d = Matrix<double, 4>;

// Run-time sized vectors and matrices (convolution kernels)
template <typename T>
struct GeneralizedVector {
  std::size_t column;
  GeneralizedVector(std::size_t c, T v = T(0)) : column(c), data(c, v) {}
  GeneralizedVector(std::initializer_list<T> d) : column(d.size()), data(d) {}
  const T& operator[](std::size_t c) const { return data[c]; }
  T& operator[](std::size_t c) { return data[c]; }

 private:
  std::vector<T> data;
};

template <typename T>
struct GeneralizedMatrix {
  std::size_t row, column;
  std::vector<GeneralizedVector<T>> data;
  GeneralizedMatrix(std::size_t r = 2, std::size_t c = 2, T v = T(0))
      : row(r), column(c), data(r, GeneralizedVector<T>(c, v)) {}
  GeneralizedMatrix(std::initializer_list<GeneralizedVector<T>> d)
      : row(d.size()), column(d.begin()->column), data(d) {}
  const GeneralizedVector<T>& operator[](std::size_t r) const { return data[r]; }
  GeneralizedVector<T>& operator[](std::size_t r) { return data[r]; }
};

template <typename T>
struct IConvolutionKernel {
  GeneralizedMatrix<T> kernel_mat;
  IConvolutionKernel() = default;
  IConvolutionKernel(std::size_t r, std::size_t c) : kernel_mat(r, c) {}
  IConvolutionKernel(const GeneralizedMatrix<T>& m) : kernel_mat(m) {}
};

// Normalised Gaussian; weights exp(-(d^2) / (2 sigma^2)) / sum, d from size/2
template <typename T, Orientation O = Orientation::All>
struct UnitizedGaussianKernel : public IConvolutionKernel<T> {
  UnitizedGaussianKernel(std::size_t size, T sigma)
      : IConvolutionKernel<T>(O == Orientation::X ? 1 : size, O == Orientation::Y ? 1 : size) {
    T mid = T(size >> 1);
    T sum = T(0);
    auto& k = this->kernel_mat;
    for (std::size_t i = 0; i < k.row; ++i)
      for (std::size_t j = 0; j < k.column; ++j) {
        T d2;
        if (O == Orientation::X)
          d2 = std::pow(T(j) - mid, T(2));
        else if (O == Orientation::Y)
          d2 = std::pow(T(i) - mid, T(2));
        else
          d2 = std::pow(T(j) - mid, T(2)) + std::pow(T(i) - mid, T(2));
        T g = std::exp(-(d2) / (T(2) * sigma * sigma));
        sum += g;
        k[i][j] = g;
      }
    for (std::size_t i = 0; i < k.row; ++i)
      for (std::size_t j = 0; j < k.column; ++j) k[i][j] /= sum;
  }
};

template <typename T, Orientation O>
struct PrewittKernel : public IConvolutionKernel<T> {
  PrewittKernel()
      : IConvolutionKernel<T>(O == Orientation::X
                                  ? GeneralizedMatrix<T>({{T(-1), T(0), T(1)}, {T(-1), T(0), T(1)}, {T(-1), T(0), T(1)}})
                                  : GeneralizedMatrix<T>({{T(1), T(1), T(1)}, {T(0), T(0), T(0)}, {T(-1), T(-1), T(-1)}})) {}
};

template <typename T, Orientation O>
struct SobelKernel : public IConvolutionKernel<T> {
  SobelKernel()
      : IConvolutionKernel<T>(O == Orientation::X
                                  ? GeneralizedMatrix<T>({{T(-1), T(0), T(1)}, {T(-2), T(0), T(2)}, {T(-1), T(0), T(1)}})
                                  : GeneralizedMatrix<T>({{T(1), T(2), T(1)}, {T(0), T(0), T(0)}, {T(-1), T(-2), T(-1)}})) {}
};

namespace Convert {
template <typename P = float, typename R = float>
constexpr R InchToMM(const P inch) {
  return R(inch) * R(25.4);
}
template <typename P = int, typename R = float>
constexpr R DegreeToRadians(const P deg) {
  return R(deg) * kPi<R> / R(180);
}
enum class ColorStandard { kITURBT709 = 0, kITURBT601 = 1, kITURBT2020 = 2, kSMPTE240M = 3, kAverage = 4 };
template <ColorStandard CS = ColorStandard::kITURBT709>
constexpr float Luma(const Vector3f& v) {
  if constexpr (CS == ColorStandard::kITURBT709) return 0.2126f * v.x() + 0.7152f * v.y() + 0.0722f * v.z();
  if constexpr (CS == ColorStandard::kITURBT601) return 0.299f * v.x() + 0.587f * v.y() + 0.114f * v.z();
  if constexpr (CS == ColorStandard::kITURBT2020) return 0.2627f * v.x() + 0.6780f * v.y() + 0.0593f * v.z();
  if constexpr (CS == ColorStandard::kSMPTE240M) return 0.2122f * v.x() + 0.7013f * v.y() + 0.0865f * v.z();
  if constexpr (CS == ColorStandard::kAverage) return (v.x() + v.y() + v.z()) / 3.0f;
  return 0.0f;
}
template <ColorStandard CS = ColorStandard::kITURBT709>
Vector3f Tonemap(const Vector3f& v, const float limit) {
  return v * 1.0f / (1.0f + Luma<CS>(v) / limit);
}
// Planckian-locus colour of a black body at temperature t (Krystek 1985),
// normalised to a maximum component of 1
Vector3f BlackBody(const float t);
Vector3f XYZToSRGB(const Vector3f& xyz);
}  // namespace Convert

struct SizeN;
struct PointN {
  int x, y;
  PointN();
  PointN(int x_, int y_);
  PointN(const Vector2f& v);
  PointN(const std::array<int, 2>& t);
  PointN operator+(const PointN& p) const;
  void SizeClamp(const SizeN& size);
};

struct SizeN {
  std::size_t width, height;
  SizeN();
  SizeN(std::size_t w, std::size_t h);
  SizeN(const Vector2f& v);
  SizeN(const std::array<std::size_t, 2>& t);
  std::size_t Area() const;
  float AspectRatio() const;
  PointN Center() const;
  bool operator==(const SizeN& a) const;
  bool operator!=(const SizeN& a) const;
};

namespace AffineTransformation {
Matrix4x4f Translation(const Vector3f& origin);
// Z * Y * X of the Euler angles, with RenderToy's sign conventions
Matrix4x4f RotationEulerXYZ(const Vector3f& euler_xyz);
}  // namespace AffineTransformation

template <typename T, typename C>
T Lerp(const T x, const T y, const C a) {
  return x * (C(1) - a) + y * a;
}

namespace Random {
int Int(int min, int max);
float Float();
}  // namespace Random

}  // namespace RenderToy

#endif
