// Small float vector / rotation algebra for the host side of the apps (the
// reference uses Eigen's Vector3f, Matrix3f and Quaternionf; Eigen is not a
// dependency here).  The formulas are the textbook ones: Hamilton product,
// the quaternion-to-matrix map, Shepperd's matrix-to-quaternion branch on
// the largest diagonal term, and Rodrigues' axis-angle matrix.
#pragma once
#include <cmath>

namespace dvs_app {

struct V3 {
  float x = 0, y = 0, z = 0;
  V3() = default;
  V3(float a, float b, float c) : x(a), y(b), z(c) {}
  float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  float &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(float s, V3 a) { return V3(s * a.x, s * a.y, s * a.z); }
inline V3 operator*(V3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
inline V3 operator/(V3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float norm(V3 a) { return std::sqrt(dot(a, a)); }
inline bool all_finite(V3 a) { return std::isfinite(a.x) && std::isfinite(a.y) && std::isfinite(a.z); }

// Row-major 3x3: m[row][col].
struct M3 {
  float m[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  float operator()(int r, int c) const { return m[r][c]; }
  float &operator()(int r, int c) { return m[r][c]; }
};
inline M3 operator*(const M3 &a, const M3 &b) {
  M3 o;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) o.m[r][c] = a.m[r][0] * b.m[0][c] + a.m[r][1] * b.m[1][c] + a.m[r][2] * b.m[2][c];
  return o;
}
inline V3 operator*(const M3 &a, V3 v) {
  return V3(a.m[0][0] * v.x + a.m[0][1] * v.y + a.m[0][2] * v.z, a.m[1][0] * v.x + a.m[1][1] * v.y + a.m[1][2] * v.z,
            a.m[2][0] * v.x + a.m[2][1] * v.y + a.m[2][2] * v.z);
}
inline M3 transpose(const M3 &a) {
  M3 o;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) o.m[r][c] = a.m[c][r];
  return o;
}
inline float determinant(const M3 &a) {
  return a.m[0][0] * (a.m[1][1] * a.m[2][2] - a.m[1][2] * a.m[2][1]) -
         a.m[0][1] * (a.m[1][0] * a.m[2][2] - a.m[1][2] * a.m[2][0]) +
         a.m[0][2] * (a.m[1][0] * a.m[2][1] - a.m[1][1] * a.m[2][0]);
}
// Frobenius norm.
inline float frobenius(const M3 &a) {
  float s = 0;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) s += a.m[r][c] * a.m[r][c];
  return std::sqrt(s);
}
inline bool all_finite(const M3 &a) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      if (!std::isfinite(a.m[r][c])) return false;
  return true;
}

// Rodrigues: rotation by angle about a unit axis.
inline M3 axis_angle(float angle, V3 axis) {
  const float s = std::sin(angle), c = std::cos(angle), k = 1.0f - c;
  M3 o;
  o.m[0][0] = k * axis.x * axis.x + c;
  o.m[1][1] = k * axis.y * axis.y + c;
  o.m[2][2] = k * axis.z * axis.z + c;
  o.m[0][1] = k * axis.x * axis.y - s * axis.z;
  o.m[1][0] = k * axis.x * axis.y + s * axis.z;
  o.m[0][2] = k * axis.x * axis.z + s * axis.y;
  o.m[2][0] = k * axis.x * axis.z - s * axis.y;
  o.m[1][2] = k * axis.y * axis.z - s * axis.x;
  o.m[2][1] = k * axis.y * axis.z + s * axis.x;
  return o;
}

struct Quat {
  float w = 1, x = 0, y = 0, z = 0;
  Quat() = default;
  Quat(float w_, float x_, float y_, float z_) : w(w_), x(x_), y(y_), z(z_) {}
};
inline float qdot(const Quat &a, const Quat &b) { return a.w * b.w + a.x * b.x + a.y * b.y + a.z * b.z; }
inline Quat qnormalized(const Quat &q) {
  const float n2 = qdot(q, q);
  if (!(n2 > 0)) return q;
  const float n = std::sqrt(n2);
  return Quat(q.w / n, q.x / n, q.y / n, q.z / n);
}
inline Quat qneg(const Quat &q) { return Quat(-q.w, -q.x, -q.y, -q.z); }
inline Quat qconj(const Quat &q) { return Quat(q.w, -q.x, -q.y, -q.z); }
inline Quat qmul(const Quat &a, const Quat &b) {
  return Quat(a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z, a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
              a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z, a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x);
}
inline M3 qmatrix(const Quat &q) {
  const float tx = 2 * q.x, ty = 2 * q.y, tz = 2 * q.z;
  const float twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
  const float txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
  const float tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
  M3 o;
  o.m[0][0] = 1 - (tyy + tzz);
  o.m[0][1] = txy - twz;
  o.m[0][2] = txz + twy;
  o.m[1][0] = txy + twz;
  o.m[1][1] = 1 - (txx + tzz);
  o.m[1][2] = tyz - twx;
  o.m[2][0] = txz - twy;
  o.m[2][1] = tyz + twx;
  o.m[2][2] = 1 - (txx + tyy);
  return o;
}
// Shepperd's method: the branch on the largest of trace and diagonal keeps
// the square root away from cancellation.
inline Quat quat_from_matrix(const M3 &R) {
  Quat q;
  const float trace = R(0, 0) + R(1, 1) + R(2, 2);
  if (trace > 0) {
    float t = std::sqrt(trace + 1.0f);
    q.w = 0.5f * t;
    t = 0.5f / t;
    q.x = (R(2, 1) - R(1, 2)) * t;
    q.y = (R(0, 2) - R(2, 0)) * t;
    q.z = (R(1, 0) - R(0, 1)) * t;
  } else {
    int i = 0;
    if (R(1, 1) > R(0, 0)) i = 1;
    if (R(2, 2) > R(i, i)) i = 2;
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    float t = std::sqrt(R(i, i) - R(j, j) - R(k, k) + 1.0f);
    float v[3];
    v[i] = 0.5f * t;
    t = 0.5f / t;
    q.w = (R(k, j) - R(j, k)) * t;
    v[j] = (R(j, i) + R(i, j)) * t;
    v[k] = (R(k, i) + R(i, k)) * t;
    q.x = v[0];
    q.y = v[1];
    q.z = v[2];
  }
  return q;
}

}  // namespace dvs_app
