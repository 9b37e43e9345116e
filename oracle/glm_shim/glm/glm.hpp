// Minimal stand-in for the parts of glm 1.0.1 that the reference's bake-path sources use
// (src/convert/tri_box_overlap.h, src/convert/voxelize.cpp, src/io/mesh_weld.cpp,
// src/io/mesh_validate.cpp, src/io/mesh_asset.h). Test infrastructure only: it lets those
// files compile unmodified into oracle/_ref so the CPU oracle can be checked against them.
//
// Every operation evaluates in glm's scalar order, which is what makes the compiled
// reference bit-exact with glm itself when built with -ffp-contract=off:
//   * arithmetic is component-wise, one rounding per operation;
//   * dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z;
//   * cross(a, b) = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y);
//   * min(x, y) = (y < x) ? y : x;  max(x, y) = (x < y) ? y : x;
//   * length(v) = sqrt(dot(v, v)).
#pragma once

#include <cmath>
#include <cstdint>

namespace glm {

struct vec2 {
  float x = 0.0f, y = 0.0f;
  vec2() = default;
  explicit vec2(float s) : x(s), y(s) {}
  vec2(float a, float b) : x(a), y(b) {}
};
inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator/(vec2 a, float s) { return vec2(a.x / s, a.y / s); }

struct ivec3;

struct vec3 {
  union {
    struct { float x, y, z; };
    struct { float r, g, b; };
  };
  vec3() : x(0.0f), y(0.0f), z(0.0f) {}
  explicit vec3(float s) : x(s), y(s), z(s) {}
  vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  vec3(int a, int b, int c) : x(static_cast<float>(a)), y(static_cast<float>(b)), z(static_cast<float>(c)) {}
  explicit vec3(const ivec3 &v);
  float &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  const float &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  vec3 &operator+=(const vec3 &o) {
    x += o.x;
    y += o.y;
    z += o.z;
    return *this;
  }
};

struct vec4 {
  float x = 0.0f, y = 0.0f, z = 0.0f, w = 0.0f;
};

struct ivec3 {
  int x = 0, y = 0, z = 0;
  ivec3() = default;
  explicit ivec3(int s) : x(s), y(s), z(s) {}
  ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
  explicit ivec3(const vec3 &v) : x(static_cast<int>(v.x)), y(static_cast<int>(v.y)), z(static_cast<int>(v.z)) {}
  bool operator==(const ivec3 &o) const { return x == o.x && y == o.y && z == o.z; }
};

inline vec3::vec3(const ivec3 &v) : x(static_cast<float>(v.x)), y(static_cast<float>(v.y)), z(static_cast<float>(v.z)) {}

inline vec3 operator+(const vec3 &a, const vec3 &b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3 &a, const vec3 &b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3 &a, const vec3 &b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator+(const vec3 &a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3 operator*(const vec3 &a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator/(const vec3 &a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }

template <typename T> inline T min(T a, T b) { return (b < a) ? b : a; }
template <typename T> inline T max(T a, T b) { return (a < b) ? b : a; }
inline vec3 min(const vec3 &a, const vec3 &b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(const vec3 &a, const vec3 &b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline ivec3 clamp(const ivec3 &v, const ivec3 &lo, const ivec3 &hi) {
  return ivec3(min(max(v.x, lo.x), hi.x), min(max(v.y, lo.y), hi.y), min(max(v.z, lo.z), hi.z));
}
inline vec3 floor(const vec3 &v) { return vec3(std::floor(v.x), std::floor(v.y), std::floor(v.z)); }

inline float dot(const vec3 &a, const vec3 &b) {
  const vec3 t = a * b;
  return t.x + t.y + t.z;
}
inline vec3 cross(const vec3 &a, const vec3 &b) {
  return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(const vec3 &v) { return std::sqrt(dot(v, v)); }
inline vec3 normalize(const vec3 &v) { return v / length(v); }

} // namespace glm
