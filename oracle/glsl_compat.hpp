// glsl_compat.hpp -- just enough of GLSL 1.20 as C++ to compile the reference's shaders unchanged
// (TEST INFRASTRUCTURE: used only to pin the CPU oracle against the reference's shader sources).
//
// The semantics GLSL leaves to the implementation are pinned exactly as the CPU oracle and the CUDA
// path pin them: single-precision IEEE arithmetic without contraction; dot(a,b) summed left to
// right; cross as the specification writes it; normalize(v) = v * (1/sqrt(dot(v,v)));
// reflect/refract as the specification writes them with dot(N,I) evaluated once; min/max =
// fminf/fmaxf; sign(0) = 0; fract(x) = x - floor(x); sin/cos/pow/exp from sppm_fpmath.h; textures
// sampled nearest with clamped coordinates (the reference sets GL_NEAREST + GL_CLAMP); the cube map
// face chosen by the major axis with ties broken x, then y, then z.
//
// GLSL's unsuffixed floating literals are single precision: the build appends the C suffix "f" to
// every floating literal of the shader text (oracle/build.py); nothing else of the source changes
// besides removing the "#version" line.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "sppm_fpmath.h"

namespace glsl {

struct vec2;
struct vec3;
struct vec4;

template <int... I>
struct swz;  // swizzle proxy over the storage of a vector

template <int N>
struct vec_of;
template <>
struct vec_of<2> {
    using type = vec2;
};
template <>
struct vec_of<3> {
    using type = vec3;
};
template <>
struct vec_of<4> {
    using type = vec4;
};

#define GLSL_SWZ_DECL                                                                          \
    static constexpr int n = sizeof...(I);                                                      \
    using V = typename vec_of<n>::type;                                                          \
    float f[4];                                                                                  \
    operator V() const;                                                                          \
    swz& operator=(const V& v);                                                                  \
    swz& operator=(const swz& o) { return *this = V(o); }                                        \
    template <int... J>                                                                          \
    swz& operator=(const swz<J...>& o) {                                                         \
        return *this = V(o);                                                                     \
    }

template <int... I>
struct swz {
    GLSL_SWZ_DECL
};

struct vec2 {
    union {
        struct {
            float x, y;
        };
        struct {
            float s, t;
        };
        struct {
            float r, g;
        };
        swz<0, 1> xy;
        swz<0, 1> st;
        swz<1, 0> yx;
        swz<0, 1, 0, 1> xyxy;
    };
    vec2() : x(0), y(0) {}
    explicit vec2(float a) : x(a), y(a) {}
    vec2(float a, float b) : x(a), y(b) {}
    vec2(const vec2& o) : x(o.x), y(o.y) {}
    vec2& operator=(const vec2& o) {
        x = o.x;
        y = o.y;
        return *this;
    }
    float& operator[](int i) { return i == 0 ? x : y; }
    float operator[](int i) const { return i == 0 ? x : y; }
};

struct vec3 {
    union {
        struct {
            float x, y, z;
        };
        struct {
            float r, g, b;
        };
        struct {
            float s, t, p;
        };
        swz<0, 1> xy;
        swz<0, 1, 2> xyz;
        swz<0, 1, 2> rgb;
        swz<0, 1> st;
    };
    vec3() : x(0), y(0), z(0) {}
    explicit vec3(float a) : x(a), y(a), z(a) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(const vec2& v, float c) : x(v.x), y(v.y), z(c) {}
    vec3(const vec3& o) : x(o.x), y(o.y), z(o.z) {}
    vec3& operator=(const vec3& o) {
        x = o.x;
        y = o.y;
        z = o.z;
        return *this;
    }
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

struct vec4 {
    union {
        struct {
            float x, y, z, w;
        };
        struct {
            float r, g, b, a;
        };
        struct {
            float s, t, p, q;
        };
        swz<0, 1> xy;
        swz<2, 3> zw;
        swz<3, 2> wz;
        swz<0, 1> st;
        swz<0, 1, 2> xyz;
        swz<0, 1, 2> rgb;
        swz<1, 3, 0> ywx;
        swz<0, 1, 0, 1> xyxy;
    };
    vec4() : x(0), y(0), z(0), w(0) {}
    explicit vec4(float v) : x(v), y(v), z(v), w(v) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec4(const vec2& v, float c, float d) : x(v.x), y(v.y), z(c), w(d) {}
    vec4(const vec2& u, const vec2& v) : x(u.x), y(u.y), z(v.x), w(v.y) {}
    vec4(const vec4& o) : x(o.x), y(o.y), z(o.z), w(o.w) {}
    vec4& operator=(const vec4& o) {
        x = o.x;
        y = o.y;
        z = o.z;
        w = o.w;
        return *this;
    }
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

template <int... I>
swz<I...>::operator typename swz<I...>::V() const {
    V v;
    const int idx[] = {I...};
    for (int k = 0; k < n; k++) v[k] = f[idx[k]];
    return v;
}
template <int... I>
swz<I...>& swz<I...>::operator=(const V& v) {
    const int idx[] = {I...};
    for (int k = 0; k < n; k++) f[idx[k]] = v[k];
    return *this;
}

// ---- component-wise arithmetic (single precision; the build disables contraction) -----------
#define GLSL_VEC_OPS(V, N)                                                                    \
    inline V operator+(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] + b[i]; return r; } \
    inline V operator-(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] - b[i]; return r; } \
    inline V operator*(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] * b[i]; return r; } \
    inline V operator/(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] / b[i]; return r; } \
    inline V operator+(const V& a, float b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] + b; return r; }      \
    inline V operator-(const V& a, float b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] - b; return r; }      \
    inline V operator*(const V& a, float b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] * b; return r; }      \
    inline V operator/(const V& a, float b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] / b; return r; }      \
    inline V operator+(float a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = a + b[i]; return r; }      \
    inline V operator-(float a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = a - b[i]; return r; }      \
    inline V operator*(float a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = a * b[i]; return r; }      \
    inline V operator/(float a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = a / b[i]; return r; }      \
    inline V operator-(const V& a) { V r; for (int i = 0; i < N; i++) r[i] = -a[i]; return r; }                  \
    inline V& operator+=(V& a, const V& b) { a = a + b; return a; }                                               \
    inline V& operator-=(V& a, const V& b) { a = a - b; return a; }                                               \
    inline V& operator*=(V& a, const V& b) { a = a * b; return a; }                                               \
    inline V& operator/=(V& a, const V& b) { a = a / b; return a; }                                               \
    inline V& operator*=(V& a, float b) { a = a * b; return a; }                                                  \
    inline V& operator/=(V& a, float b) { a = a / b; return a; }                                                  \
    inline V floor(const V& a) { V r; for (int i = 0; i < N; i++) r[i] = std::floor(a[i]); return r; }           \
    inline V fract(const V& a) { V r; for (int i = 0; i < N; i++) r[i] = a[i] - std::floor(a[i]); return r; }    \
    inline V abs(const V& a) { V r; for (int i = 0; i < N; i++) r[i] = std::fabs(a[i]); return r; }              \
    inline V sign(const V& a) { V r; for (int i = 0; i < N; i++) r[i] = a[i] > 0.0f ? 1.0f : (a[i] < 0.0f ? -1.0f : 0.0f); return r; } \
    inline V min(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = std::fmin(a[i], b[i]); return r; } \
    inline V max(const V& a, const V& b) { V r; for (int i = 0; i < N; i++) r[i] = std::fmax(a[i], b[i]); return r; } \
    inline V min(const V& a, float b) { V r; for (int i = 0; i < N; i++) r[i] = std::fmin(a[i], b); return r; }      \
    inline V max(const V& a, float b) { V r; for (int i = 0; i < N; i++) r[i] = std::fmax(a[i], b); return r; }      \
    inline V exp(const V& a) { V r; for (int i = 0; i < N; i++) r[i] = sppm_fexp(a[i]); return r; }              \
    inline V sqrt(const V& a) { V r; for (int i = 0; i < N; i++) r[i] = std::sqrt(a[i]); return r; }             \
    inline float dot(const V& a, const V& b) { float s = a[0] * b[0]; for (int i = 1; i < N; i++) s = s + a[i] * b[i]; return s; } \
    inline float length(const V& a) { return std::sqrt(dot(a, a)); }                                             \
    inline V normalize(const V& a) { return a * (1.0f / std::sqrt(dot(a, a))); }                                  \
    inline V reflect(const V& i, const V& n) { const float d = 2.0f * dot(n, i); return i - d * n; }             \
    inline V refract(const V& i, const V& n, float eta) {                                                         \
        const float d = dot(n, i);                                                                                \
        const float k = 1.0f - eta * eta * (1.0f - d * d);                                                        \
        if (k < 0.0f) return V(0.0f);                                                                             \
        return eta * i - (eta * d + std::sqrt(k)) * n;                                                            \
    }

GLSL_VEC_OPS(vec2, 2)
GLSL_VEC_OPS(vec3, 3)
GLSL_VEC_OPS(vec4, 4)

inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

inline float floor(float a) { return std::floor(a); }
inline float fract(float a) { return a - std::floor(a); }
inline float abs(float a) { return std::fabs(a); }
inline float sign(float a) { return a > 0.0f ? 1.0f : (a < 0.0f ? -1.0f : 0.0f); }
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline float sqrt(float a) { return std::sqrt(a); }
inline float sin(float a) { return sppm_fsin(a); }
inline float cos(float a) { return sppm_fcos(a); }
inline float pow(float a, float b) { return sppm_fpow(a, b); }
inline float exp(float a) { return sppm_fexp(a); }
inline float mod(float a, float b) { return a - b * std::floor(a / b); }
inline float length(float a) { return std::fabs(a); }

struct bvec4 {
    bool v[4];
};
struct bvec3 {
    bool v[3];
};
inline bvec4 greaterThanEqual(const vec4& a, const vec4& b) { return bvec4{{a.x >= b.x, a.y >= b.y, a.z >= b.z, a.w >= b.w}}; }
inline bvec3 greaterThan(const vec3& a, const vec3& b) { return bvec3{{a.x > b.x, a.y > b.y, a.z > b.z}}; }
inline bvec3 lessThan(const vec3& a, const vec3& b) { return bvec3{{a.x < b.x, a.y < b.y, a.z < b.z}}; }
inline bool all(const bvec4& b) { return b.v[0] && b.v[1] && b.v[2] && b.v[3]; }
inline bool all(const bvec3& b) { return b.v[0] && b.v[1] && b.v[2]; }

// ---- samplers ----------------------------------------------------------------------------------
struct sampler2D {
    const vec4* texels = nullptr;
    int w = 0, h = 0;
};
struct samplerCube {
    vec4 face[6];
};
struct sampler3D {
    int unused = 0;
};

// nearest texel, coordinates clamped to [0, 1] (GL_NEAREST, GL_CLAMP)
inline vec4 texture2D(const sampler2D& s, const vec2& uv) {
    float u = uv.x < 0.0f ? 0.0f : (uv.x > 1.0f ? 1.0f : uv.x);
    float v = uv.y < 0.0f ? 0.0f : (uv.y > 1.0f ? 1.0f : uv.y);
    int i = (int)std::floor(u * (float)s.w), j = (int)std::floor(v * (float)s.h);
    if (i > s.w - 1) i = s.w - 1;
    if (j > s.h - 1) j = s.h - 1;
    return s.texels[(size_t)j * s.w + i];
}
inline vec4 textureCube(const samplerCube& c, const vec3& d) {
    const float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    int f;
    if (ax >= ay && ax >= az) f = d.x < 0.0f ? 1 : 0;
    else if (ay >= az) f = d.y < 0.0f ? 3 : 2;
    else f = d.z < 0.0f ? 5 : 4;
    return c.face[f];
}
// the scenes used for the pin carry no textures: every texture3D call would read a material texture
vec4 texture3D(const sampler3D&, const vec3&);

}  // namespace glsl
