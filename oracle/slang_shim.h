// C++ stand-ins for the Slang/HLSL types and built-ins that pxlengine's shaders/fluid.slang and
// shaders/sim.slang use, so that the shaders' own source compiles with g++ and their compute
// kernels run on the CPU (test infrastructure only: oracle/ref_fluid.cpp and oracle/ref_sim.cpp,
// built by oracle/ref_build.py into oracle/_ref/).
//
// Semantics chosen for the built-ins (the SPIR-V the reference's slangc emits calls
// GLSL.std.450, whose results the Vulkan spec defines to these formulas or leaves open):
//   lerp(a, b, t)  = a * (1 - t) + b * t        (FMix definition)
//   normalize(v)   = v / sqrt(dot(v, v)),  dot = x*x + y*y + z*z in that order
//   max(a, b)      = a < b ? b : a,  min(a, b) = b < a ? b : a,  clamp(x, lo, hi) = min(max(x, lo), hi)
//   int(f)         = truncation toward zero; floor / ceil / sqrt are the C library's (correctly
//                    rounded, as SPIR-V's are exact for floor and ceil)
//   InterlockedAdd = an atomic add (relaxed): the invocations of a dispatch may run on several
//                    host threads; the add returns the value before it
//   GroupMemoryBarrierWithGroupSync = an OpenMP barrier: a workgroup's invocations run as one
//                    team of host threads; groupshared arrays are plain arrays shared by the team
//   saturate(v) = clamp(v, 0, 1) (NaN -> 0), cross = the usual determinant form, asuint = bit copy
// Unsuffixed floating literals are float (g++ -fsingle-precision-constant), as in Slang.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

typedef unsigned int uint;

template <class T> struct ident { typedef T type; };

struct bool3 {
    bool x, y, z;
};
inline bool any(bool3 b) { return b.x || b.y || b.z; }

template <class T>
struct vec3 {
    T x, y, z;
    vec3() = default;
    vec3(T s) : x(s), y(s), z(s) {}
    template <class A, class B, class C>
    vec3(A a, B b, C c) : x(T(a)), y(T(b)), z(T(c)) {}
    template <class U>
    explicit vec3(const vec3<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
    T& operator[](uint i) { return i == 0 ? x : (i == 1 ? y : z); }
    T operator[](uint i) const { return i == 0 ? x : (i == 1 ? y : z); }
    vec3& operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec3& operator-=(const vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
};
typedef vec3<float> float3;
typedef vec3<int> int3;
typedef vec3<uint> uint3;

#define SHIM_BINOP(OP)                                                                                  \
    template <class T> vec3<T> operator OP(const vec3<T>& a, const vec3<T>& b) {                        \
        return vec3<T>(a.x OP b.x, a.y OP b.y, a.z OP b.z);                                             \
    }                                                                                                   \
    template <class T> vec3<T> operator OP(const vec3<T>& a, typename ident<T>::type s) {               \
        return vec3<T>(a.x OP s, a.y OP s, a.z OP s);                                                   \
    }                                                                                                   \
    template <class T> vec3<T> operator OP(typename ident<T>::type s, const vec3<T>& a) {               \
        return vec3<T>(s OP a.x, s OP a.y, s OP a.z);                                                   \
    }
SHIM_BINOP(+)
SHIM_BINOP(-)
SHIM_BINOP(*)
SHIM_BINOP(/)
#undef SHIM_BINOP
template <class T> vec3<T> operator-(const vec3<T>& a) { return vec3<T>(-a.x, -a.y, -a.z); }

#define SHIM_CMP(OP)                                                                                    \
    template <class T> bool3 operator OP(const vec3<T>& a, const vec3<T>& b) {                          \
        return bool3{a.x OP b.x, a.y OP b.y, a.z OP b.z};                                               \
    }                                                                                                   \
    template <class T> bool3 operator OP(const vec3<T>& a, typename ident<T>::type s) {                 \
        return bool3{a.x OP s, a.y OP s, a.z OP s};                                                     \
    }
SHIM_CMP(<)
SHIM_CMP(>)
SHIM_CMP(==)
#undef SHIM_CMP

struct float4 {
    union {
        struct {
            float x, y, z, w;
        };
        struct {
            float r, g, b, a;
        };
        float3 xyz;
    };
    float4() = default;
    float4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    float4(const float3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    float& operator[](uint i) { return (&x)[i]; }
    float operator[](uint i) const { return (&x)[i]; }
};

inline float4 operator*(const float4& v, float s) { return float4(v.x * s, v.y * s, v.z * s, v.w * s); }
inline float4 operator+(const float4& v, float s) { return float4(v.x + s, v.y + s, v.z + s, v.w + s); }

struct uint4 {
    uint x, y, z, w;
    uint4() = default;
    template <class A, class B, class C, class D>
    uint4(A a, B b, C c, D d) : x(uint(a)), y(uint(b)), z(uint(c)), w(uint(d)) {}
    explicit uint4(const float4& v) : x(uint(v.x)), y(uint(v.y)), z(uint(v.z)), w(uint(v.w)) {}
};

struct int2 {
    int x, y;
    int2() = default;
    int2(int a, int b) : x(a), y(b) {}
};

inline float max(float a, float b) { return a < b ? b : a; }
inline float min(float a, float b) { return b < a ? b : a; }
template <class T> vec3<T> max(const vec3<T>& a, const vec3<T>& b) {
    return vec3<T>(a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y, a.z < b.z ? b.z : a.z);
}
template <class T> vec3<T> min(const vec3<T>& a, const vec3<T>& b) {
    return vec3<T>(b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y, b.z < a.z ? b.z : a.z);
}
template <class T> vec3<T> clamp(const vec3<T>& v, const vec3<T>& lo, const vec3<T>& hi) {
    return min(max(v, lo), hi);
}
inline float3 floor(const float3& v) { return float3(std::floor(v.x), std::floor(v.y), std::floor(v.z)); }
inline float3 ceil(const float3& v) { return float3(std::ceil(v.x), std::ceil(v.y), std::ceil(v.z)); }
inline float lerp(float a, float b, float t) { return a * (1.0f - t) + b * t; }
inline float3 lerp(const float3& a, const float3& b, float t) { return a * (1.0f - t) + b * t; }
inline float3 lerp(const float3& a, const float3& b, const float3& t) {
    return float3(lerp(a.x, b.x, t.x), lerp(a.y, b.y, t.y), lerp(a.z, b.z, t.z));
}
inline float dot(const float3& a, const float3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float3 normalize(const float3& v) { return v / std::sqrt(dot(v, v)); }
inline float3 cross(const float3& a, const float3& b) {
    return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float abs(float v) { return std::fabs(v); }
inline float saturate(float v) { return v > 0.0f ? (v < 1.0f ? v : 1.0f) : 0.0f; }
inline float4 saturate(const float4& v) { return float4(saturate(v.x), saturate(v.y), saturate(v.z), saturate(v.w)); }
inline uint asuint(float v) {
    uint u;
    std::memcpy(&u, &v, 4);
    return u;
}
inline uint4 asuint(const float4& v) { return uint4(asuint(v.x), asuint(v.y), asuint(v.z), asuint(v.w)); }
inline void GroupMemoryBarrierWithGroupSync() { _Pragma("omp barrier") }

template <class T> void InterlockedAdd(T& dst, T v) { __atomic_fetch_add(&dst, v, __ATOMIC_RELAXED); }
template <class T> void InterlockedAdd(T& dst, T v, T& original) { original = __atomic_fetch_add(&dst, v, __ATOMIC_RELAXED); }

template <class T>
struct RWStructuredBuffer {
    T* p = nullptr;
    T& operator[](uint i) const { return p[i]; }
};
template <class T>
using StructuredBuffer = RWStructuredBuffer<T>;
template <class T>
struct ConstantBuffer : T {};
