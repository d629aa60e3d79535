// Minimal GLSL-vocabulary shim for C++, written for this project.
//
// Test infrastructure only: it lets the reference's compute shader
// srcCommon/shaders/raytracer.glsl compile as C++ (after the declaration
// rewrites of oracle/glsl_to_cpp.py), so the oracle's traversal restatement
// can be checked against the shader's own code.  It provides exactly what
// that shader uses:
//   * vec2, vec3, vec4, ivec2, uvec2, uvec3 and mat4 (column-major), with the
//     read-only swizzles the shader takes (.xyz of vec4, .xy of vec3 / vec4 /
//     uvec3) as conversions;
//   * per-component +, -, *, / (vector-vector and vector-scalar);
//   * dot, cross, normalize, abs, min, max as the GLSL 4.60 specification
//     defines them, min(x, y) = y < x ? y : x and max(x, y) = x < y ? y : x;
//   * image2D / imageStore into a host RGBA32F array;
//   * gl_GlobalInvocationID (per host thread) and gl_NumWorkGroups.
// Where the specification leaves the order of operations open, the shim
// fixes it as the CUDA path and the oracle do (compile with
// -ffp-contract=off, so every operation rounds once):
//   * dot(a, b) = ((a.x b.x + a.y b.y) + a.z b.z) [+ a.w b.w];
//   * normalize(v) = v * (1 / sqrt(dot(v, v)));
//   * mat4 * vec4 = (c0 v.x + c1 v.y) + (c2 v.z + c3 v.w) per row (glm's order).
// A default-constructed vector holds NaN in every component: the shader's
// uninitialised Hit._Coords.w then compares false, so a miss never replaces
// a hit (raytracer.glsl:279-281), the canonical reading the CUDA path uses.
//
// This header is meant to be included inside a namespace (after the system
// headers), so that its abs / min / max hide the C library's.
#pragma once

typedef uint32_t uint;

struct vec2;
struct vec3;
struct vec4;
struct uvec2;

constexpr float kShimNaN = __builtin_nanf("");

// Read-only swizzles: views of N floats that convert to the smaller vector.
template <int N, int A, int B>
struct swizzle2 {
    float v[N];
    operator vec2() const;
};
template <int N, int A, int B, int C>
struct swizzle3 {
    float v[N];
    operator vec3() const;
};
template <int N, int A, int B>
struct uswizzle2 {
    uint v[N];
    operator uvec2() const;
};

struct vec2 {
    union {
        struct { float x, y; };
    };
    vec2() : x(kShimNaN), y(kShimNaN) {}
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
};

struct alignas(16) vec3 {
    union {
        struct { float x, y, z; };
        swizzle2<3, 0, 1> xy;
    };
    vec3() : x(kShimNaN), y(kShimNaN), z(kShimNaN) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(const vec2& v, float c) : x(v.x), y(v.y), z(c) {}
};

struct alignas(16) vec4 {
    union {
        struct { float x, y, z, w; };
        swizzle3<4, 0, 1, 2> xyz;
        swizzle2<4, 0, 1> xy;
    };
    vec4() : x(kShimNaN), y(kShimNaN), z(kShimNaN), w(kShimNaN) {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
};

struct uvec2 {
    uint x, y;
    uvec2() : x(0), y(0) {}
    uvec2(uint a, uint b) : x(a), y(b) {}
};

struct uvec3 {
    union {
        struct { uint x, y, z; };
        uswizzle2<3, 0, 1> xy;
    };
    uvec3() : x(0), y(0), z(0) {}
    uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
};

struct ivec2 {
    int x, y;
    ivec2() : x(0), y(0) {}
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(const uvec2& v) : x(static_cast<int>(v.x)), y(static_cast<int>(v.y)) {}
};

template <int N, int A, int B>
swizzle2<N, A, B>::operator vec2() const { return vec2(v[A], v[B]); }
template <int N, int A, int B, int C>
swizzle3<N, A, B, C>::operator vec3() const { return vec3(v[A], v[B], v[C]); }
template <int N, int A, int B>
uswizzle2<N, A, B>::operator uvec2() const { return uvec2(v[A], v[B]); }

// Column-major 4x4: c[i] is column i.
struct alignas(16) mat4 {
    vec4 c[4];
    mat4() : c{vec4(1.f, 0.f, 0.f, 0.f), vec4(0.f, 1.f, 0.f, 0.f), vec4(0.f, 0.f, 1.f, 0.f), vec4(0.f, 0.f, 0.f, 1.f)} {}
};

// ---- arithmetic (per component)
inline vec2 operator-(const vec2& a, float s) { return vec2(a.x - s, a.y - s); }
inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec4 operator+(const vec4& a, const vec4& b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator-(const vec4& a, const vec4& b) { return vec4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline vec4 operator*(const vec4& a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline vec4 operator/(const vec4& a, float s) { return vec4(a.x / s, a.y / s, a.z / s, a.w / s); }
inline vec4& operator+=(vec4& a, const vec4& b) {
    a = a + b;
    return a;
}

inline vec4 operator*(const mat4& m, const vec4& v) {
    const vec4* c = m.c;
    return vec4((c[0].x * v.x + c[1].x * v.y) + (c[2].x * v.z + c[3].x * v.w),
                (c[0].y * v.x + c[1].y * v.y) + (c[2].y * v.z + c[3].y * v.w),
                (c[0].z * v.x + c[1].z * v.y) + (c[2].z * v.z + c[3].z * v.w),
                (c[0].w * v.x + c[1].w * v.y) + (c[2].w * v.z + c[3].w * v.w));
}

// ---- built-in functions
inline float abs(float a) { return __builtin_fabsf(a); }
inline float min(float a, float b) { return b < a ? b : a; }
inline float max(float a, float b) { return a < b ? b : a; }
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float dot(const vec4& a, const vec4& b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline vec3 normalize(const vec3& v) { return v * (1.0f / __builtin_sqrtf(dot(v, v))); }
inline vec4 normalize(const vec4& v) { return v * (1.0f / __builtin_sqrtf(dot(v, v))); }

// ---- images and invocation ids
struct image2D {
    vec4* texels = nullptr;  // row y at y * width
    int width = 0;
    int height = 0;
};
inline void imageStore(image2D& img, const ivec2& p, const vec4& v) {
    if (p.x >= 0 && p.y >= 0 && p.x < img.width && p.y < img.height)
        img.texels[static_cast<long>(p.y) * img.width + p.x] = v;
}

thread_local uvec3 gl_GlobalInvocationID;
uvec3 gl_NumWorkGroups;
