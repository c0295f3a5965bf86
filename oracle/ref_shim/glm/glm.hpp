// Minimal stand-in for the GLM headers the reference includes (glmInclude.h),
// written for this repository — TEST INFRASTRUCTURE, used only to compile the
// reference's own instrumented traversal and SAH builder here (oracle/ref/).
//
// GLM itself is not vendored in the reference and is absent from this image.
// This header declares the subset of GLM's API the compiled reference files
// name, with the arithmetic GLM documents for each function, in GLM's
// evaluation order where it decides the float result:
//   min(a, b) = (b < a) ? b : a;  max(a, b) = (a < b) ? b : a  (per component)
//   abs(x)    = x >= 0 ? x : -x   (per component)
//   dot(a, b) = (a.x * b.x + a.y * b.y) + a.z * b.z
//   normalize(v) = v * (1 / sqrt(dot(v, v)))
//   length(v) = sqrt(dot(v, v))
//   cross(a, b) = (a.y b.z - b.y a.z, a.z b.x - b.z a.x, a.x b.y - b.x a.y)
//   compMin / compMax fold min / max over the components from the first.
// Matrix and quaternion types exist so that the scene-graph headers compile;
// the parity driver passes world-space triangles and explicit rays, so none
// of their arithmetic is on the compared path.
#pragma once
#include <cassert>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <limits>

namespace glm {

typedef int length_t;

struct vec2 {
  float x, y;
  vec2() : x(0), y(0) {}
  explicit vec2(float s) : x(s), y(s) {}
  vec2(float a, float b) : x(a), y(b) {}
  float& operator[](length_t i) { return (&x)[i]; }
  const float& operator[](length_t i) const { return (&x)[i]; }
  static constexpr length_t length() { return 2; }
};

struct vec4;

struct vec3 {
  float x, y, z;
  vec3() : x(0), y(0), z(0) {}
  explicit vec3(float s) : x(s), y(s), z(s) {}
  vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  vec3(const vec4& v);  // implicit, as in GLM without GLM_FORCE_EXPLICIT_CTOR
  float& operator[](length_t i) { return (&x)[i]; }
  const float& operator[](length_t i) const { return (&x)[i]; }
  static constexpr length_t length() { return 3; }
  vec3& operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
  vec3& operator-=(const vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
  vec3& operator*=(const vec3& o) { x *= o.x; y *= o.y; z *= o.z; return *this; }
  vec3& operator/=(const vec3& o) { x /= o.x; y /= o.y; z /= o.z; return *this; }
  vec3& operator+=(float s) { x += s; y += s; z += s; return *this; }
  vec3& operator-=(float s) { x -= s; y -= s; z -= s; return *this; }
  vec3& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
  vec3& operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
};
typedef vec3 fvec3;

struct vec4 {
  float x, y, z, w;
  vec4() : x(0), y(0), z(0), w(0) {}
  explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
  vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
  float& operator[](length_t i) { return (&x)[i]; }
  const float& operator[](length_t i) const { return (&x)[i]; }
  static constexpr length_t length() { return 4; }
};
inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

#define GLMSHIM_BIN(T, OP)                                                              \
  inline T operator OP(const T& a, const T& b) { T r(a); for (length_t i = 0; i < T::length(); ++i) r[i] = a[i] OP b[i]; return r; } \
  inline T operator OP(const T& a, float s) { T r(a); for (length_t i = 0; i < T::length(); ++i) r[i] = a[i] OP s; return r; }      \
  inline T operator OP(float s, const T& a) { T r(a); for (length_t i = 0; i < T::length(); ++i) r[i] = s OP a[i]; return r; }
GLMSHIM_BIN(vec2, +) GLMSHIM_BIN(vec2, -) GLMSHIM_BIN(vec2, *) GLMSHIM_BIN(vec2, /)
GLMSHIM_BIN(vec3, +) GLMSHIM_BIN(vec3, -) GLMSHIM_BIN(vec3, *) GLMSHIM_BIN(vec3, /)
GLMSHIM_BIN(vec4, +) GLMSHIM_BIN(vec4, -) GLMSHIM_BIN(vec4, *) GLMSHIM_BIN(vec4, /)
#undef GLMSHIM_BIN

inline vec2 operator-(const vec2& a) { return vec2(-a.x, -a.y); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec4 operator-(const vec4& a) { return vec4(-a.x, -a.y, -a.z, -a.w); }
inline bool operator==(const vec3& a, const vec3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline bool operator!=(const vec3& a, const vec3& b) { return !(a == b); }
inline bool operator==(const vec2& a, const vec2& b) { return a.x == b.x && a.y == b.y; }
inline bool operator==(const vec4& a, const vec4& b) { return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w; }

// scalar forms
inline float min(float a, float b) { return (b < a) ? b : a; }
inline float max(float a, float b) { return (a < b) ? b : a; }
inline float abs(float a) { return a >= 0.0f ? a : -a; }
inline int min(int a, int b) { return (b < a) ? b : a; }
inline int max(int a, int b) { return (a < b) ? b : a; }

template <class T> inline T min(const T& a, const T& b) {
  T r(a); for (length_t i = 0; i < T::length(); ++i) r[i] = (b[i] < a[i]) ? b[i] : a[i]; return r;
}
template <class T> inline T max(const T& a, const T& b) {
  T r(a); for (length_t i = 0; i < T::length(); ++i) r[i] = (a[i] < b[i]) ? b[i] : a[i]; return r;
}
template <class T> inline T min(const T& a, float b) { return min(a, T(b)); }
template <class T> inline T max(const T& a, float b) { return max(a, T(b)); }
template <class T> inline T abs(const T& a) {
  T r(a); for (length_t i = 0; i < T::length(); ++i) r[i] = a[i] >= 0.0f ? a[i] : -a[i]; return r;
}
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec4& a, const vec4& b) { return (a.x * b.x + a.y * b.y) + (a.z * b.z + a.w * b.w); }
inline vec3 cross(const vec3& a, const vec3& b) {
  return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline float length(const vec2& v) { return std::sqrt(dot(v, v)); }
inline float inversesqrt(float x) { return 1.0f / std::sqrt(x); }
inline vec3 normalize(const vec3& v) { return v * inversesqrt(dot(v, v)); }
inline vec2 normalize(const vec2& v) { return v * inversesqrt(dot(v, v)); }
template <class T> inline float compMin(const T& v) {
  float r = v[0]; for (length_t i = 1; i < T::length(); ++i) r = min(r, v[i]); return r;
}
template <class T> inline float compMax(const T& v) {
  float r = v[0]; for (length_t i = 1; i < T::length(); ++i) r = max(r, v[i]); return r;
}

// ---- matrices and quaternions (scene graph only) -------------------------
struct quat;

struct mat3 {
  vec3 c[3];
  mat3() {}
  explicit mat3(float s) { c[0] = vec3(s, 0, 0); c[1] = vec3(0, s, 0); c[2] = vec3(0, 0, s); }
  vec3& operator[](length_t i) { return c[i]; }
  const vec3& operator[](length_t i) const { return c[i]; }
};

struct mat4 {
  vec4 c[4];
  mat4() {}
  explicit mat4(float s) {
    c[0] = vec4(s, 0, 0, 0); c[1] = vec4(0, s, 0, 0); c[2] = vec4(0, 0, s, 0); c[3] = vec4(0, 0, 0, s);
  }
  mat4(const quat& q);  // implicit, as in GLM
  vec4& operator[](length_t i) { return c[i]; }
  const vec4& operator[](length_t i) const { return c[i]; }
};

struct quat {
  float x, y, z, w;
  quat() : x(0), y(0), z(0), w(1) {}
  quat(float w_, float x_, float y_, float z_) : x(x_), y(y_), z(z_), w(w_) {}
  quat(const mat4& m);  // implicit, as in GLM
  float& operator[](length_t i) { return (&x)[i]; }
  const float& operator[](length_t i) const { return (&x)[i]; }
};

inline vec4 operator*(const mat4& m, const vec4& v) {
  return (m[0] * v.x + m[1] * v.y) + (m[2] * v.z + m[3] * v.w);
}
inline mat4 operator*(const mat4& a, const mat4& b) {
  mat4 r;
  for (int i = 0; i < 4; ++i) r[i] = a * b[i];
  return r;
}

inline mat4::mat4(const quat& q) {
  const float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
  const float xz = q.x * q.z, xy = q.x * q.y, yz = q.y * q.z;
  const float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
  c[0] = vec4(1 - 2 * (yy + zz), 2 * (xy + wz), 2 * (xz - wy), 0);
  c[1] = vec4(2 * (xy - wz), 1 - 2 * (xx + zz), 2 * (yz + wx), 0);
  c[2] = vec4(2 * (xz + wy), 2 * (yz - wx), 1 - 2 * (xx + yy), 0);
  c[3] = vec4(0, 0, 0, 1);
}

inline quat::quat(const mat4& m) {
  // Shepperd's method on the upper 3x3 (a rotation matrix).
  const float t = m[0][0] + m[1][1] + m[2][2];
  if (t > 0) {
    const float s = std::sqrt(t + 1.0f) * 2;
    w = 0.25f * s; x = (m[1][2] - m[2][1]) / s; y = (m[2][0] - m[0][2]) / s; z = (m[0][1] - m[1][0]) / s;
  } else if (m[0][0] > m[1][1] && m[0][0] > m[2][2]) {
    const float s = std::sqrt(1.0f + m[0][0] - m[1][1] - m[2][2]) * 2;
    w = (m[1][2] - m[2][1]) / s; x = 0.25f * s; y = (m[1][0] + m[0][1]) / s; z = (m[2][0] + m[0][2]) / s;
  } else if (m[1][1] > m[2][2]) {
    const float s = std::sqrt(1.0f + m[1][1] - m[0][0] - m[2][2]) * 2;
    w = (m[2][0] - m[0][2]) / s; x = (m[1][0] + m[0][1]) / s; y = 0.25f * s; z = (m[2][1] + m[1][2]) / s;
  } else {
    const float s = std::sqrt(1.0f + m[2][2] - m[0][0] - m[1][1]) * 2;
    w = (m[0][1] - m[1][0]) / s; x = (m[2][0] + m[0][2]) / s; y = (m[2][1] + m[1][2]) / s; z = 0.25f * s;
  }
}

inline mat4 translate(const mat4& m, const vec3& v) {
  mat4 r(m);
  r[3] = m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3];
  return r;
}
inline mat4 scale(const mat4& m, const vec3& v) {
  mat4 r;
  r[0] = m[0] * v.x; r[1] = m[1] * v.y; r[2] = m[2] * v.z; r[3] = m[3];
  return r;
}
// General 4x4 inverse by cofactors (scene graph only).
inline mat4 inverse(const mat4& m) {
  float a[16], inv[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) a[i * 4 + j] = m[i][j];
  inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
  inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
  inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
  inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
  inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
  inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
  inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
  inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
  inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
  inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
  inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
  inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
  inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
  inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
  inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
  inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
  const float det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
  mat4 r;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) r[i][j] = inv[i * 4 + j] / det;
  return r;
}

inline const float* value_ptr(const vec3& v) { return &v.x; }
inline const float* value_ptr(const mat4& m) { return &m[0].x; }
inline quat make_quat(const float* p) { return quat(p[3], p[0], p[1], p[2]); }
inline quat make_quat(const double* p) {
  return quat((float)p[3], (float)p[0], (float)p[1], (float)p[2]);
}
inline vec3 make_vec3(const float* p) { return vec3(p[0], p[1], p[2]); }
inline vec3 make_vec3(const double* p) { return vec3((float)p[0], (float)p[1], (float)p[2]); }
inline mat4 make_mat4(const float* p) {
  mat4 r;
  for (int i = 0; i < 16; ++i) r[i / 4][i % 4] = p[i];
  return r;
}
inline mat4 make_mat4(const double* p) {
  mat4 r;
  for (int i = 0; i < 16; ++i) r[i / 4][i % 4] = (float)p[i];
  return r;
}
// Translation, rotation and scale of an affine transform without shear or
// perspective (scene graph only).
inline bool decompose(const mat4& m, vec3& scale_, quat& rot, vec3& trans, vec3& skew, vec4& persp) {
  trans = vec3(m[3]);
  for (int i = 0; i < 3; ++i) scale_[i] = length(vec3(m[i]));
  mat4 r(1.0f);
  for (int i = 0; i < 3; ++i) r[i] = vec4(vec3(m[i]) / scale_[i], 0);
  rot = quat(r);
  skew = vec3(0);
  persp = vec4(0, 0, 0, 1);
  return true;
}

}  // namespace glm

namespace std {
template <> struct hash<glm::vec3> {
  size_t operator()(const glm::vec3& v) const noexcept {
    size_t h = hash<float>()(v.x);
    h ^= hash<float>()(v.y) + 0x9e3779b9 + (h << 6) + (h >> 2);
    h ^= hash<float>()(v.z) + 0x9e3779b9 + (h << 6) + (h >> 2);
    return h;
  }
};
}  // namespace std
