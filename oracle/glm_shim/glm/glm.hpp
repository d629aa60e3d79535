// Minimal glm-compatible vector/matrix shim, written for this project.
//
// Test infrastructure only: it exists so the reference's own
// srcCommon/scene/geometry/{bvh,triangle}.cpp compile unmodified into the
// oracle's reference library (the real glm is not installed here).  It
// provides exactly the glm surface those two files use: vec3, vec4, mat4
// (column-major), component-wise arithmetic, scalar*matrix, matrix*vector,
// glm::distance and glm::to_string.
//
// Arithmetic order follows glm >= 0.9.9 (the version the reference pins is
// not recorded; its CMakeLists only says find_package(glm)):
//   * vec + vec, vec - vec, vec * s, s * vec, vec / s: per component;
//   * s * mat4: every element multiplied by s;
//   * mat4 * vec4: (c0*v.x + c1*v.y) + (c2*v.z + c3*v.w), column vectors c_i.
// Compile with -ffp-contract=off so no multiply-add is fused.
#pragma once

#include <cmath>
#include <cstdint>
#include <string>

namespace glm {

struct vec4;

struct vec3 {
    float x, y, z;
    vec3() : x(0.f), y(0.f), z(0.f) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit vec3(const vec4& v);
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const float& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

struct vec4 {
    float x, y, z, w;
    vec4() : x(0.f), y(0.f), z(0.f), w(0.f) {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    const float& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }

inline vec4 operator+(const vec4& a, const vec4& b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator-(const vec4& a, const vec4& b) { return vec4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline vec4 operator*(const vec4& a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline vec4 operator*(float s, const vec4& a) { return vec4(s * a.x, s * a.y, s * a.z, s * a.w); }
inline vec4 operator/(const vec4& a, float s) { return vec4(a.x / s, a.y / s, a.z / s, a.w / s); }

struct mat4 {
    vec4 c[4];  // columns
    mat4() : mat4(1.f) {}
    explicit mat4(float d) {
        c[0] = vec4(d, 0.f, 0.f, 0.f);
        c[1] = vec4(0.f, d, 0.f, 0.f);
        c[2] = vec4(0.f, 0.f, d, 0.f);
        c[3] = vec4(0.f, 0.f, 0.f, d);
    }
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};

inline mat4 operator*(float s, const mat4& m) {
    mat4 r;
    for (int i = 0; i < 4; ++i) r.c[i] = m.c[i] * s;
    return r;
}
inline mat4 operator*(const mat4& m, float s) { return s * m; }

inline vec4 operator*(const mat4& m, const vec4& v) {
    const vec4 a = m.c[0] * v.x + m.c[1] * v.y;
    const vec4 b = m.c[2] * v.z + m.c[3] * v.w;
    return a + b;
}

inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(const vec3& a) { return std::sqrt(dot(a, a)); }
inline float distance(const vec3& a, const vec3& b) { return length(b - a); }

}  // namespace glm
