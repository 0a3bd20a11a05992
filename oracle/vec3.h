// Small FP64 vector helpers that evaluate in the order Eigen 3.3 uses for
// Vector3d/Matrix3d expressions in the reference:
//   dot / squaredNorm : (a0*b0 + a1*b1) + a2*b2
//   norm              : sqrt(squaredNorm)
//   normalized        : v / sqrt(squaredNorm) when squaredNorm > 0, else v
//   cross             : (a1 b2 - a2 b1, a2 b0 - a0 b2, a0 b1 - a1 b0)
// Oracle-internal (test infrastructure).
#ifndef EOLC_ORACLE_VEC3_H_
#define EOLC_ORACLE_VEC3_H_
#include <cmath>

namespace orc {

struct V3 {
  double v[3];
  double &operator[](int i) { return v[i]; }
  double operator[](int i) const { return v[i]; }
};

inline V3 mk(double a, double b, double c) { return V3{{a, b, c}}; }
inline V3 ld(const double *p) { return V3{{p[0], p[1], p[2]}}; }
inline V3 operator+(const V3 &a, const V3 &b) {
  return mk(a[0] + b[0], a[1] + b[1], a[2] + b[2]);
}
inline V3 operator-(const V3 &a, const V3 &b) {
  return mk(a[0] - b[0], a[1] - b[1], a[2] - b[2]);
}
inline V3 operator-(const V3 &a) { return mk(-a[0], -a[1], -a[2]); }
inline V3 operator*(double s, const V3 &a) {
  return mk(s * a[0], s * a[1], s * a[2]);
}
inline V3 operator/(const V3 &a, double s) {
  return mk(a[0] / s, a[1] / s, a[2] / s);
}
inline double dot(const V3 &a, const V3 &b) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}
inline double sqn(const V3 &a) { return dot(a, a); }
inline double norm(const V3 &a) { return std::sqrt(sqn(a)); }
inline V3 normalized(const V3 &a) {
  double z = sqn(a);
  return z > 0.0 ? a / std::sqrt(z) : a;
}
inline V3 cross(const V3 &a, const V3 &b) {
  return mk(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
            a[0] * b[1] - a[1] * b[0]);
}

}  // namespace orc
#endif
