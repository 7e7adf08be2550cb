// Build shim: the GLSL vector and matrix types, built-ins and functions that
// the reference's particle shaders (Shaders/particle.vs.glsl, particle.fs.glsl)
// use, so that their source compiles as C++ (build_ref.sh includes each
// shader inside a struct, with `uniform`, `in`, `out` and `layout(...)`
// defined away and its uniform blocks as members).  Every operation is the
// plain IEEE float operation in GLSL's order of evaluation; the shaders are
// compiled with -fsingle-precision-constant -ffp-contract=off so that their
// literals are floats and nothing fuses.  Test infrastructure only.
#pragma once
#include <cmath>

namespace glsl {

struct vec2;
struct vec3;
struct vec4;

// .xy of a vector holding at least two floats: reads as a vec2, assigns both.
template <int kN>
struct Swizzle01 {
    float v[kN];
    inline operator vec2() const;
    inline Swizzle01& operator=(const vec2& o);
};

struct vec2 {
    union {
        struct {
            float x, y;
        };
        Swizzle01<2> xy;
    };
    vec2() : x(0.f), y(0.f) {}
    vec2(float a, float b) : x(a), y(b) {}
    vec2(const vec2& o) : x(o.x), y(o.y) {}
    vec2& operator=(const vec2& o) {
        x = o.x;
        y = o.y;
        return *this;
    }
};
template <int kN>
inline Swizzle01<kN>::operator vec2() const { return vec2(v[0], v[1]); }
template <int kN>
inline Swizzle01<kN>& Swizzle01<kN>::operator=(const vec2& o) {
    v[0] = o.x;
    v[1] = o.y;
    return *this;
}

struct vec3 {
    union {
        struct {
            float x, y, z;
        };
        Swizzle01<3> xy;
    };
    vec3() : x(0.f), y(0.f), z(0.f) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(const vec3& o) : x(o.x), y(o.y), z(o.z) {}
    explicit inline vec3(const vec4& o);
    vec3& operator=(const vec3& o) {
        x = o.x;
        y = o.y;
        z = o.z;
        return *this;
    }
    vec3& operator+=(const vec3& o) {
        x = x + o.x;
        y = y + o.y;
        z = z + o.z;
        return *this;
    }
};

struct vec4 {
    float x, y, z, w;

    vec4() = default;  // trivial, so that uniform blocks can hold it
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
};
inline vec3::vec3(const vec4& o) : x(o.x), y(o.y), z(o.z) {}

// column-major, m[c][r] as in GLSL
struct mat4 {
    vec4 c[4];
};

inline vec2 operator*(const vec2& a, const vec2& b) { return vec2(a.x * b.x, a.y * b.y); }
inline vec2 operator+(const vec2& a, const vec2& b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec4 operator+(const vec4& a, const vec4& b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator*(const vec4& a, const vec4& b) { return vec4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
inline vec4 operator*(const vec4& a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
// matrix * vector: sum over columns in order
inline vec4 operator*(const mat4& m, const vec4& v) {
    return vec4(((m.c[0].x * v.x + m.c[1].x * v.y) + m.c[2].x * v.z) + m.c[3].x * v.w,
                ((m.c[0].y * v.x + m.c[1].y * v.y) + m.c[2].y * v.z) + m.c[3].y * v.w,
                ((m.c[0].z * v.x + m.c[1].z * v.y) + m.c[2].z * v.z) + m.c[3].z * v.w,
                ((m.c[0].w * v.x + m.c[1].w * v.y) + m.c[2].w * v.z) + m.c[3].w * v.w);
}

inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(const vec3& a) { return std::sqrt(dot(a, a)); }
inline vec3 normalize(const vec3& a) { return a / length(a); }
inline float max(float a, float b) { return a < b ? b : a; }
inline float sqrt(float a) { return std::sqrt(a); }
inline float pow(float a, float b) { return std::pow(a, b); }

// the built-in variables of the two stages
struct Builtins {
    vec2 gl_PointCoord;
    float gl_PointSize = 0.f;
    vec4 gl_Position;
    bool discarded = false;
};

}  // namespace glsl
