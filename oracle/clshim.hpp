// clshim.hpp — TEST INFRASTRUCTURE ONLY.
//
// A minimal OpenCL C environment in C++ so that the reference's kernel
// sources (assets/kernels/*.cl) compile unmodified apart from their vector
// literal syntax `(float3)(a, b, c)`, which build_ref.py rewrites to
// `make_float3(a, b, c)`.  Everything here lives in namespace clref and is
// included once, before the kernel sources, by the generated translation
// unit oracle/_ref/ref_kernels.cpp.
//
// Work-items run one after another on the host: ref_driver.inc sets the
// work-item ids in `clref::wi` before each call.  barrier() is a no-op, which
// is exact for every kernel ref_driver.inc runs (each work-item of histogram /
// reorder touches only its own local-memory column); scanhistograms and
// pastehistograms are not run through the shim.
//
// Built-ins have the meaning the oracle and the CUDA kernels give them:
// dot left to right, IEEE sqrt, fast_length = sqrt(dot), convert_int
// truncating (saturating, NaN -> 0), fmax/fmin for float max/min, and
// pow with exponent 2 or 3 taken exactly in double and rounded once.

#pragma once
#include "noise_sin.hpp"
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>

namespace clref {

typedef unsigned int uint;
typedef unsigned char uchar;

struct float2 {
    float x, y;
    float2() = default;
    float2(float s) { x = y = s; }
    float2(float a, float b) { x = a; y = b; }
};

struct float3 {
    union {
        struct { float x, y, z; };
        float2 xy;
    };
    float3() = default;
    float3(float s) { x = y = z = s; }
    float3(float a, float b, float c) { x = a; y = b; z = c; }
};

struct float4 {
    union {
        struct { float x, y, z, w; };
        float3 xyz;
        float2 xy;
    };
    float4() = default;
    float4(float s) { x = y = z = w = s; }
    float4(float a, float b, float c, float d) { x = a; y = b; z = c; w = d; }
};

struct int2 { int x, y; };
struct int3 { int x, y, z; };
struct int4 { int x, y, z, w; };
struct uint2 { uint x, y; };
struct uint4 { uint x, y, z, w; };

// ---- vector literals (the rewritten `(typeN)(...)` forms) ----
inline float2 make_float2(float a, float b) { return float2(a, b); }
inline float3 make_float3(float s) { return float3(s); }
inline float3 make_float3(float a, float b, float c) { return float3(a, b, c); }
inline float4 make_float4(float s) { return float4(s); }
inline float4 make_float4(float a, float b, float c, float d) { return float4(a, b, c, d); }
inline float4 make_float4(const float3& v, float w) { return float4(v.x, v.y, v.z, w); }
inline int2 make_int2(int a, int b) { return {a, b}; }
inline int3 make_int3(int a, int b, int c) { return {a, b, c}; }
inline uint2 make_uint2(uint a, uint b) { return {a, b}; }
inline uint4 make_uint4(uint a, uint b, uint c, uint d) { return {a, b, c, d}; }

// ---- arithmetic ----
#define CLSHIM_BINOP(OP)                                                                              \
    inline float3 operator OP(const float3& a, const float3& b) { return float3(a.x OP b.x, a.y OP b.y, a.z OP b.z); } \
    inline float3 operator OP(const float3& a, float s) { return float3(a.x OP s, a.y OP s, a.z OP s); }            \
    inline float3 operator OP(float s, const float3& a) { return float3(s OP a.x, s OP a.y, s OP a.z); }            \
    inline float4 operator OP(const float4& a, const float4& b) {                                     \
        return float4(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w); }                               \
    inline float4 operator OP(const float4& a, float s) { return float4(a.x OP s, a.y OP s, a.z OP s, a.w OP s); }  \
    inline float4 operator OP(float s, const float4& a) { return float4(s OP a.x, s OP a.y, s OP a.z, s OP a.w); }
CLSHIM_BINOP(+)
CLSHIM_BINOP(-)
CLSHIM_BINOP(*)
CLSHIM_BINOP(/)
#undef CLSHIM_BINOP

// Integer scalars with float vectors (e.g. `future * 5 / h`).
inline float3 operator*(const float3& a, int s) { return a * (float)s; }
inline float3 operator*(int s, const float3& a) { return (float)s * a; }
inline float3 operator*(const float3& a, double s) { return a * (float)s; }

inline float3& operator+=(float3& a, const float3& b) { a = a + b; return a; }
inline float3& operator-=(float3& a, const float3& b) { a = a - b; return a; }
inline float3& operator*=(float3& a, float s) { a = a * s; return a; }
inline float3& operator/=(float3& a, float s) { a = a / s; return a; }
inline float4& operator+=(float4& a, const float4& b) { a = a + b; return a; }
inline float3 operator-(const float3& a) { return float3(-a.x, -a.y, -a.z); }

inline int3 operator+(const int3& a, const int3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }

// ---- geometric / common built-ins ----
inline float dot(const float2& a, const float2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const float3& a, const float3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float3 cross(const float3& a, const float3& b) {
    return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float sqrt(float v) { return std::sqrt(v); }
inline float length(const float3& a) { return std::sqrt(dot(a, a)); }
inline float fast_length(const float3& a) { return std::sqrt(dot(a, a)); }
inline float3 normalize(const float3& a) { return a / length(a); }
inline float fabs(float v) { return std::fabs(v); }
// sin: the contract's portable definition (noise_sin.hpp)
inline float sin(float v) { return noise_sinf_ref(v); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline float min(float a, float b) { return std::fmin(a, b); }
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline float pow(float x, float y) {
    if (y == 2.0f) return (float)((double)x * (double)x);
    if (y == 3.0f) return (float)((double)x * (double)x * (double)x);
    return (float)std::pow((double)x, (double)y);
}
inline float fract(float x, float* ip) { float f = std::floor(x); *ip = f; return std::fmin(x - f, 0x1.fffffep-1f); }
inline float3 fract(const float3& x, float3* ip) {
    return float3(fract(x.x, &ip->x), fract(x.y, &ip->y), fract(x.z, &ip->z));
}
inline float smoothstep(float e0, float e1, float x) {
    float t = std::fmin(std::fmax((x - e0) / (e1 - e0), 0.0f), 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
inline float mix(float a, float b, float t) { return a + (b - a) * t; }
inline uint mul_hi(uint a, uint b) { return (uint)(((uint64_t)a * (uint64_t)b) >> 32); }

inline int convert_int(float v) {
    if (v != v) return 0;
    if (v >= 2147483647.0f) return 2147483647;
    if (v <= -2147483648.0f) return (-2147483647 - 1);
    return (int)v;
}
inline int3 convert_int3(const float3& v) { return {convert_int(v.x), convert_int(v.y), convert_int(v.z)}; }

// ---- images (a zero mask and a write-only texture) ----
struct ClImage { int width, height; int32_t* data; };
typedef ClImage* image2d_t;
typedef int sampler_t;
enum { CLK_NORMALIZED_COORDS_FALSE = 0, CLK_ADDRESS_CLAMP_TO_EDGE = 0, CLK_FILTER_NEAREST = 0 };
enum { CLK_LOCAL_MEM_FENCE = 1, CLK_GLOBAL_MEM_FENCE = 2 };
inline int4 read_imagei(image2d_t img, sampler_t, int2 c) {
    if (!img || !img->data) return {0, 0, 0, 0};
    int x = std::min(std::max(c.x, 0), img->width - 1), y = std::min(std::max(c.y, 0), img->height - 1);
    return {img->data[(size_t)y * img->width + x], 0, 0, 1};
}
inline uint4 read_imageui(image2d_t img, sampler_t s, int2 c) {
    int4 v = read_imagei(img, s, c);
    return {(uint)v.x, (uint)v.y, (uint)v.z, (uint)v.w};
}
inline void write_imageui(image2d_t, int2, uint4) {}
inline void write_imagef(image2d_t, int2, float4) {}
inline int get_image_width(image2d_t img) { return img ? img->width : 2048; }

// ---- work-item ids ----
// one per host thread: the driver runs work-items on several threads
struct WorkItem { uint gid, lid, grp, ngroups, lsize; };
extern thread_local WorkItem wi;
inline uint get_global_id(int) { return wi.gid; }
inline uint get_local_id(int) { return wi.lid; }
inline uint get_group_id(int) { return wi.grp; }
inline uint get_num_groups(int) { return wi.ngroups; }
inline uint get_local_size(int) { return wi.lsize; }
inline void barrier(int) {}

// ---- compile-time constants of Simulation.cpp:169-183, set per run ----
extern float g_poly6, g_gradSpiky;
extern int g_maxParticles, g_circles, g_perCircle, g_friendsBlock, g_gridBufSize;

}  // namespace clref

#define __kernel
#define __global
#define __local
#define __private
#define __constant const
#define __read_only
#define __write_only
#define __OPENCL_VERSION__ 120
#define cl_khr_global_int32_base_atomics 1
#define cl_khr_global_int32_extended_atomics 1
#define END_OF_CELL_LIST (-1)
#define LOG_SIZE 1024
#define POLY6_FACTOR g_poly6
#define GRAD_SPIKY_FACTOR g_gradSpiky
#define MAX_PARTICLES_COUNT g_maxParticles
#define MAX_FRIENDS_CIRCLES g_circles
#define MAX_FRIENDS_IN_CIRCLE g_perCircle
#define FRIENDS_BLOCK_SIZE g_friendsBlock
#define GRID_BUF_SIZE g_gridBufSize
