// glsl_subset.hpp — the subset of GLSL 4.60 compute-shader semantics that the reference's
// clustered-shading, bouncer, depth-pyramid and debug-view shaders use, as C++20 (TEST
// INFRASTRUCTURE ONLY).  oracle/ref_shaders.py rewrites those shaders mechanically into C++ against
// this header and builds them into oracle/_ref/, so the oracle can be compared with the reference's
// own shader source run on the CPU.
//
// What it models, and the choices made where GLSL leaves a choice to the implementation:
//  - vectors vecN / uvecN / ivecN (N = 2..4) and a column-major mat4; component access .x.y.z.w
//    (.r.g.b.a are rewritten to them), indexing, and swizzles as v.swz<i, j, ...>() (rvalue) and
//    v.set_swz<i, j>(value) (the rewrite of `v.xy = value;`).  int and uint vectors convert to float
//    vectors implicitly, as GLSL allows; the other direction is explicit.
//  - float -> uint/int conversion of a value outside the target's range (negative, NaN, too large)
//    is undefined in GLSL; here it saturates (NaN -> 0).
//  - arithmetic in single precision with every operation rounded on its own (the build uses
//    -ffp-contract=off); mat4 * vec4 = ((m0 x + m1 y) + m2 z) + m3 w; dot and length sum left to
//    right; normalize(v) = v / length(v); sqrt, division, log, tan, pow, exp2, acos from the C
//    library (GLSL bounds their error, a driver picks its own implementation).
//  - inverse(mat4) by cofactors in single precision.
//  - buffers: out-of-bounds reads return zero and out-of-bounds writes are dropped (Vulkan's robust
//    buffer access); each such access is counted in glsl::g_oob.
//  - sampler2D / usampler2D: NEAREST filtering with REPEAT addressing at normalised coordinates
//    (texel i = floor(u * size) wrapped into [0, size)), or at unnormalised coordinates with
//    CLAMP_TO_BORDER (the depth-pyramid copy's sampler); image2D / uimage2D with imageLoad /
//    imageStore / imageSize, out-of-bounds stores dropped.
//  - one 32-wide subgroup: subgroupBallot over 32 invocations that the driver runs in lockstep as
//    coroutines (each ballot suspends a lane until all 32 have voted); subgroupElect picks lane 0
//    (every call site here is in uniform control flow).
#pragma once

#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <type_traits>

namespace glsl {

typedef uint32_t uint;

inline std::atomic<uint64_t> g_oob{0};

// ---- scalar conversions -------------------------------------------------------------------------
inline uint to_uint(float f)
{
    if (!(f > 0.0f)) return 0u;  // negative, zero, NaN
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint)f;
}
inline int to_int(float f)
{
    if (f != f) return 0;
    if (f <= -2147483648.0f) return std::numeric_limits<int>::min();
    if (f >= 2147483648.0f) return std::numeric_limits<int>::max();
    return (int)f;
}
template <class T> inline uint glsl_uint(T v)
{
    if constexpr (std::is_floating_point_v<T>) return to_uint((float)v);
    else return (uint)v;
}
template <class T> inline int glsl_int(T v)
{
    if constexpr (std::is_floating_point_v<T>) return to_int((float)v);
    else return (int)v;
}
template <class T> inline float glsl_float(T v) { return (float)v; }
template <class T> inline bool glsl_bool(T v) { return v != T(0); }

template <class To, class From> inline To convert(From v)
{
    if constexpr (std::is_same_v<To, uint> && std::is_floating_point_v<From>) return to_uint((float)v);
    else if constexpr (std::is_same_v<To, int> && std::is_floating_point_v<From>) return to_int((float)v);
    else return (To)v;
}
// GLSL's implicit conversions: int -> uint, int/uint -> float
template <class To, class From>
inline constexpr bool implicit_v = std::is_same_v<To, From> || (std::is_same_v<To, float> && !std::is_same_v<From, float>) ||
                                   (std::is_same_v<To, uint> && std::is_same_v<From, int>);

template <class T> struct tvec2;
template <class T> struct tvec3;
template <class T> struct tvec4;

#define GLSL_VEC_COMMON(NAME, N)                                                                           \
    T& operator[](uint64_t i) { return (&x)[i]; }                                                          \
    const T& operator[](uint64_t i) const { return (&x)[i]; }                                              \
    template <int A, int B> tvec2<T> swz() const { return tvec2<T>((*this)[A], (*this)[B]); }              \
    template <int A, int B, int C> tvec3<T> swz() const { return tvec3<T>((*this)[A], (*this)[B], (*this)[C]); } \
    template <int A, int B, int C, int D> tvec4<T> swz() const                                            \
    {                                                                                                      \
        return tvec4<T>((*this)[A], (*this)[B], (*this)[C], (*this)[D]);                                   \
    }                                                                                                      \
    template <int A, int B> void set_swz(const tvec2<T>& v) { (*this)[A] = v.x; (*this)[B] = v.y; }        \
    template <int A, int B, int C> void set_swz(const tvec3<T>& v)                                        \
    {                                                                                                      \
        (*this)[A] = v.x; (*this)[B] = v.y; (*this)[C] = v.z;                                              \
    }                                                                                                      \
    friend NAME operator+(NAME a, const NAME& b) { for (int i = 0; i < N; ++i) a[i] = a[i] + b[i]; return a; } \
    friend NAME operator-(NAME a, const NAME& b) { for (int i = 0; i < N; ++i) a[i] = a[i] - b[i]; return a; } \
    friend NAME operator*(NAME a, const NAME& b) { for (int i = 0; i < N; ++i) a[i] = a[i] * b[i]; return a; } \
    friend NAME operator/(NAME a, const NAME& b) { for (int i = 0; i < N; ++i) a[i] = a[i] / b[i]; return a; } \
    friend NAME operator+(NAME a, T s) { for (int i = 0; i < N; ++i) a[i] = a[i] + s; return a; }          \
    friend NAME operator-(NAME a, T s) { for (int i = 0; i < N; ++i) a[i] = a[i] - s; return a; }          \
    friend NAME operator*(NAME a, T s) { for (int i = 0; i < N; ++i) a[i] = a[i] * s; return a; }          \
    friend NAME operator/(NAME a, T s) { for (int i = 0; i < N; ++i) a[i] = a[i] / s; return a; }          \
    friend NAME operator+(T s, NAME a) { for (int i = 0; i < N; ++i) a[i] = s + a[i]; return a; }          \
    friend NAME operator-(T s, NAME a) { for (int i = 0; i < N; ++i) a[i] = s - a[i]; return a; }          \
    friend NAME operator*(T s, NAME a) { for (int i = 0; i < N; ++i) a[i] = s * a[i]; return a; }          \
    friend NAME operator/(T s, NAME a) { for (int i = 0; i < N; ++i) a[i] = s / a[i]; return a; }          \
    friend NAME operator-(NAME a) { for (int i = 0; i < N; ++i) a[i] = -a[i]; return a; }                  \
    NAME& operator+=(const NAME& b) { return *this = *this + b; }                                          \
    NAME& operator-=(const NAME& b) { return *this = *this - b; }                                          \
    NAME& operator*=(const NAME& b) { return *this = *this * b; }                                          \
    NAME& operator/=(const NAME& b) { return *this = *this / b; }                                          \
    NAME& operator*=(T s) { return *this = *this * s; }                                                    \
    NAME& operator/=(T s) { return *this = *this / s; }                                                    \
    friend bool operator==(const NAME& a, const NAME& b)                                                   \
    {                                                                                                      \
        for (int i = 0; i < N; ++i)                                                                        \
            if (!(a[i] == b[i])) return false;                                                             \
        return true;                                                                                       \
    }                                                                                                      \
    friend bool operator!=(const NAME& a, const NAME& b) { return !(a == b); }

template <class T> struct tvec2 {
    T x, y;
    tvec2() : x(T(0)), y(T(0)) {}
    explicit tvec2(T s) : x(s), y(s) {}
    tvec2(T a, T b) : x(a), y(b) {}
    template <class U> explicit(!implicit_v<T, U>) tvec2(const tvec2<U>& o)
        : x(convert<T>(o.x)), y(convert<T>(o.y)) {}
    GLSL_VEC_COMMON(tvec2, 2)
};

template <class T> struct tvec3 {
    T x, y, z;
    tvec3() : x(T(0)), y(T(0)), z(T(0)) {}
    explicit tvec3(T s) : x(s), y(s), z(s) {}
    tvec3(T a, T b, T c) : x(a), y(b), z(c) {}
    tvec3(const tvec2<T>& v, T c) : x(v.x), y(v.y), z(c) {}
    template <class U> explicit(!implicit_v<T, U>) tvec3(const tvec3<U>& o)
        : x(convert<T>(o.x)), y(convert<T>(o.y)), z(convert<T>(o.z)) {}
    GLSL_VEC_COMMON(tvec3, 3)
};

template <class T> struct tvec4 {
    T x, y, z, w;
    tvec4() : x(T(0)), y(T(0)), z(T(0)), w(T(0)) {}
    explicit tvec4(T s) : x(s), y(s), z(s), w(s) {}
    tvec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    tvec4(const tvec2<T>& v, T c, T d) : x(v.x), y(v.y), z(c), w(d) {}
    tvec4(const tvec3<T>& v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
    template <class U> explicit(!implicit_v<T, U>) tvec4(const tvec4<U>& o)
        : x(convert<T>(o.x)), y(convert<T>(o.y)), z(convert<T>(o.z)), w(convert<T>(o.w)) {}
    GLSL_VEC_COMMON(tvec4, 4)
};
#undef GLSL_VEC_COMMON

typedef tvec2<float> vec2;
typedef tvec3<float> vec3;
typedef tvec4<float> vec4;
typedef tvec2<uint> uvec2;
typedef tvec3<uint> uvec3;
typedef tvec4<uint> uvec4;
typedef tvec2<int> ivec2;
typedef tvec3<int> ivec3;
typedef tvec4<int> ivec4;

// integer bit operations on uint vectors used by the shaders
inline uvec2 operator&(uvec2 a, uint m) { return uvec2(a.x & m, a.y & m); }

struct mat4 {
    vec4 c[4];
    mat4() {}
    explicit mat4(float d) { for (int i = 0; i < 4; ++i) c[i][i] = d; }
    vec4& operator[](uint64_t i) { return c[i]; }
    const vec4& operator[](uint64_t i) const { return c[i]; }
};
inline vec4 operator*(const mat4& m, const vec4& v)
{
    vec4 r;
    for (int i = 0; i < 4; ++i) r[i] = ((m.c[0][i] * v.x + m.c[1][i] * v.y) + m.c[2][i] * v.z) + m.c[3][i] * v.w;
    return r;
}
inline mat4 mat4_from(const float* m)  // column-major
{
    mat4 r;
    for (int k = 0; k < 16; ++k) r.c[k / 4][k % 4] = m[k];
    return r;
}

// inverse by cofactors, single precision
inline mat4 inverse(const mat4& M)
{
    float m[16], inv[16];
    for (int k = 0; k < 16; ++k) m[k] = M.c[k / 4][k % 4];
    inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
    inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
    inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
    inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
    inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
    inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
    inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
    inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
    inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
    inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
    inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
    inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
    inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
    inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
    inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
    inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
    const float det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
    mat4 r;
    for (int k = 0; k < 16; ++k) r.c[k / 4][k % 4] = inv[k] / det;
    return r;
}

// ---- built-in functions -------------------------------------------------------------------------
inline float floor(float v) { return std::floor(v); }
inline float sign(float v) { return v > 0.0f ? 1.0f : (v < 0.0f ? -1.0f : 0.0f); }
inline float min(float a, float b) { return b < a ? b : a; }  // GLSL min(x, y) = y < x ? y : x
inline float max(float a, float b) { return a < b ? b : a; }  // GLSL max(x, y) = x < y ? y : x
inline uint min(uint a, uint b) { return b < a ? b : a; }
inline uint max(uint a, uint b) { return a < b ? b : a; }
inline float clamp(float v, float lo, float hi) { return min(max(v, lo), hi); }
// scalar built-ins take any arithmetic argument (GLSL converts int and uint arguments to float)
template <class T> inline float log(T v) { return std::log((float)v); }
template <class T> inline float log2(T v) { return std::log2((float)v); }
template <class T> inline float exp2(T v) { return std::exp2((float)v); }
template <class T> inline float tan(T v) { return std::tan((float)v); }
template <class T> inline float acos(T v) { return std::acos((float)v); }
template <class A, class B> inline float pow(A a, B b) { return std::pow((float)a, (float)b); }
template <class T> inline float sqrt(T v) { return std::sqrt((float)v); }
inline float mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
template <class V> inline V vfloor(V v) { for (uint64_t i = 0; i < sizeof(V) / sizeof(float); ++i) v[i] = std::floor(v[i]); return v; }
inline vec2 floor(vec2 v) { return vfloor(v); }
inline vec3 floor(vec3 v) { return vfloor(v); }
inline vec4 floor(vec4 v) { return vfloor(v); }
inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline vec3 normalize(const vec3& v) { return v / length(v); }
inline vec3 min(vec3 a, const vec3& b) { for (int i = 0; i < 3; ++i) a[i] = min(a[i], b[i]); return a; }
inline vec3 max(vec3 a, const vec3& b) { for (int i = 0; i < 3; ++i) a[i] = max(a[i], b[i]); return a; }
inline vec3 max(vec3 a, float b) { for (int i = 0; i < 3; ++i) a[i] = max(a[i], b); return a; }
inline vec3 min(vec3 a, float b) { for (int i = 0; i < 3; ++i) a[i] = min(a[i], b); return a; }
inline vec3 mix(const vec3& a, const vec3& b, float t) { return a * (1.0f - t) + b * t; }
inline vec3 pow(vec3 a, const vec3& b) { for (int i = 0; i < 3; ++i) a[i] = std::pow(a[i], b[i]); return a; }
inline int findLSB(uint v) { return v == 0 ? -1 : __builtin_ctz(v); }
inline int bitCount(uint v) { return __builtin_popcount(v); }

// ---- buffers, samplers, images --------------------------------------------------------------------
template <class T> struct buffer {
    T* p = nullptr;
    uint64_t n = 0;
    T& operator[](uint64_t i) const
    {
        if (i < n) return p[i];
        g_oob.fetch_add(1, std::memory_order_relaxed);
        thread_local T dummy;
        std::memset(static_cast<void*>(&dummy), 0, sizeof(T));
        return dummy;
    }
    int length() const { return (int)n; }
};

struct sampler2D {
    const float* data = nullptr;  // row-major texels of `comps` floats
    int w = 0, h = 0, comps = 4;
    bool unnormalized = false;  // unnormalised coordinates with CLAMP_TO_BORDER (border = 0)
};
struct usampler2D {
    const uint* data = nullptr;
    int w = 0, h = 0, comps = 1;
};
inline int wrap(int i, int n) { i %= n; return i < 0 ? i + n : i; }
inline ivec2 nearest_repeat(const vec2& uv, int w, int h)
{
    return ivec2(wrap(to_int(std::floor(uv.x * (float)w)), w), wrap(to_int(std::floor(uv.y * (float)h)), h));
}
inline vec4 texel(const sampler2D& s, int x, int y)
{
    vec4 r(0.0f, 0.0f, 0.0f, 1.0f);
    const float* t = s.data + ((size_t)y * s.w + x) * s.comps;
    for (int c = 0; c < s.comps && c < 4; ++c) r[c] = t[c];
    return r;
}
inline vec4 texture(const sampler2D& s, const vec2& uv)
{
    if (s.unnormalized) {
        const int x = to_int(std::floor(uv.x)), y = to_int(std::floor(uv.y));
        if (x < 0 || y < 0 || x >= s.w || y >= s.h) return vec4(0.0f);
        return texel(s, x, y);
    }
    const ivec2 i = nearest_repeat(uv, s.w, s.h);
    return texel(s, i.x, i.y);
}
inline uvec4 texture(const usampler2D& s, const vec2& uv)
{
    const ivec2 i = nearest_repeat(uv, s.w, s.h);
    uvec4 r(0u, 0u, 0u, 1u);
    const uint* t = s.data + ((size_t)i.y * s.w + i.x) * s.comps;
    for (int c = 0; c < s.comps && c < 4; ++c) r[c] = t[c];
    return r;
}
inline ivec2 textureSize(const sampler2D& s, int) { return ivec2(s.w, s.h); }

struct image2D {
    float* data = nullptr;  // row-major, `comps` floats per texel
    int w = 0, h = 0, comps = 4;
};
struct uimage2D {
    uint* data = nullptr;
    int w = 0, h = 0, comps = 1;
};
inline ivec2 imageSize(const image2D& im) { return ivec2(im.w, im.h); }
inline ivec2 imageSize(const uimage2D& im) { return ivec2(im.w, im.h); }
inline bool inside(int x, int y, int w, int h) { return x >= 0 && y >= 0 && x < w && y < h; }
inline vec4 imageLoad(const image2D& im, const ivec2& p)
{
    vec4 r(0.0f, 0.0f, 0.0f, 1.0f);
    if (!inside(p.x, p.y, im.w, im.h)) return r;
    for (int c = 0; c < im.comps; ++c) r[c] = im.data[((size_t)p.y * im.w + p.x) * im.comps + c];
    return r;
}
inline uvec4 imageLoad(const uimage2D& im, const ivec2& p)
{
    uvec4 r(0u, 0u, 0u, 1u);
    if (!inside(p.x, p.y, im.w, im.h)) return r;
    r.x = im.data[(size_t)p.y * im.w + p.x];
    return r;
}
inline void imageStore(const image2D& im, const ivec2& p, const vec4& v)
{
    if (!inside(p.x, p.y, im.w, im.h)) return;  // dropped
    for (int c = 0; c < im.comps; ++c) im.data[((size_t)p.y * im.w + p.x) * im.comps + c] = v[c];
}
inline void imageStore(const uimage2D& im, const ivec2& p, const uvec4& v)
{
    if (!inside(p.x, p.y, im.w, im.h)) return;
    im.data[(size_t)p.y * im.w + p.x] = v.x;
}

// ---- built-in variables -----------------------------------------------------------------------
inline thread_local uvec3 gl_GlobalInvocationID, gl_WorkGroupID, gl_LocalInvocationID, gl_NumWorkGroups;
inline thread_local uvec3 gl_WorkGroupSize;
inline thread_local uint gl_LocalInvocationIndex = 0, gl_SubgroupInvocationID = 0, gl_SubgroupID = 0;
inline thread_local uint gl_SubgroupSize = 32, gl_NumSubgroups = 1;

// ---- one 32-wide subgroup -------------------------------------------------------------------------
// The driver runs the 32 invocations of a subgroup as coroutines on one host thread; a ballot stores
// the lane's vote and suspends it until every lane has voted (g_ballot, set by the driver).
inline thread_local uint (*g_ballot)(bool) = nullptr;

inline uvec4 subgroupBallot(bool b) { return uvec4(g_ballot(b), 0u, 0u, 0u); }
inline bool subgroupElect() { return gl_SubgroupInvocationID == 0; }
inline void subgroupMemoryBarrierBuffer() {}

}  // namespace glsl
