// OpenCL C -> host C++ shim for the reference-kernel CPU harness (test infrastructure only).
//
// The reference keeps its device code as OpenCL C text (src/kernel.cpp, assembled by
// src/kernel.hpp:7-18 get_opencl_c_code()). This header supplies the OpenCL C builtins and types that
// text uses, so the unmodified text compiles as C++ and runs over host threads. It replaces the
// OpenCL runtime only: the LBM arithmetic is the reference's own.
//
// Semantics follow the OpenCL C specification:
//  - vload_half / vstore_half_rte: exact widening, round-to-nearest-even narrowing (IEEE binary16);
//  - fma: fused multiply-add with one rounding (std::fma);
//  - dot(a,b) = a.x*b.x+a.y*b.y+a.z*b.z evaluated left to right, cross() the usual determinant
//    form; the harness is compiled with -ffp-contract=off, so no other multiply-add is fused;
//  - clamp(x,a,b) = min(max(x,a),b); sign(x) in {-1,0,+1} (NaN -> 0);
//  - work-item id: a thread-local global id set by the launching loop (one work-item at a time).
// Kernels that need work-group barriers (object_* reductions) compile but are never launched.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include "../half_ieee.h"

namespace ocl {
typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned int uint;
typedef unsigned long long ulong;
typedef unsigned short half; // only ever accessed through vload_half / vstore_half_rte

extern thread_local ulong global_id;

struct float3 {
	float x, y, z;
	float3() : x(0.0f), y(0.0f), z(0.0f) {}
	explicit float3(const float s) : x(s), y(s), z(s) {}
	float3(const float x, const float y, const float z) : x(x), y(y), z(z) {}
	float3& operator+=(const float3& o) { x += o.x; y += o.y; z += o.z; return *this; }
	float3& operator-=(const float3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
	float3& operator*=(const float s) { x *= s; y *= s; z *= s; return *this; }
};
static inline float3 operator+(const float3& a, const float3& b) { return float3(a.x+b.x, a.y+b.y, a.z+b.z); }
static inline float3 operator-(const float3& a, const float3& b) { return float3(a.x-b.x, a.y-b.y, a.z-b.z); }
static inline float3 operator-(const float3& a) { return float3(-a.x, -a.y, -a.z); }
static inline float3 operator*(const float3& a, const float3& b) { return float3(a.x*b.x, a.y*b.y, a.z*b.z); }
static inline float3 operator*(const float s, const float3& a) { return float3(s*a.x, s*a.y, s*a.z); }
static inline float3 operator*(const float3& a, const float s) { return float3(a.x*s, a.y*s, a.z*s); }
static inline float3 operator/(const float3& a, const float s) { return float3(a.x/s, a.y/s, a.z/s); }

struct uint3 {
	uint x, y, z;
	uint3() : x(0u), y(0u), z(0u) {}
	uint3(const uint x, const uint y, const uint z) : x(x), y(y), z(z) {}
};
struct int3 {
	int x, y, z;
	int3() : x(0), y(0), z(0) {}
	int3(const int x, const int y, const int z) : x(x), y(y), z(z) {}
};

static inline float dot(const float3& a, const float3& b) { return a.x*b.x+a.y*b.y+a.z*b.z; }
static inline float3 cross(const float3& a, const float3& b) { return float3(a.y*b.z-a.z*b.y, a.z*b.x-a.x*b.z, a.x*b.y-a.y*b.x); }
static inline float length(const float3& a) { return std::sqrt(dot(a, a)); }

static inline float fma(const float a, const float b, const float c) { return std::fma(a, b, c); }
static inline float fabs(const float x) { return std::fabs(x); }
static inline float fmod(const float x, const float y) { return std::fmod(x, y); }
static inline float acos(const float x) { return std::acos(x); }
static inline float sqrt(const float x) { return std::sqrt(x); }
static inline float sign(const float x) { return x>0.0f ? 1.0f : x<0.0f ? -1.0f : 0.0f; }
static inline float clamp(const float x, const float a, const float b) { return std::fmin(std::fmax(x, a), b); }
static inline int clamp(const int x, const int a, const int b) { return x<a ? a : x>b ? b : x; }
static inline uint clamp(const uint x, const uint a, const uint b) { return x<a ? a : x>b ? b : x; }
static inline uint min(const uint a, const uint b) { return a<b ? a : b; }
static inline int min(const int a, const int b) { return a<b ? a : b; }
static inline float min(const float a, const float b) { return std::fmin(a, b); }
static inline uint max(const uint a, const uint b) { return a>b ? a : b; }
static inline int max(const int a, const int b) { return a>b ? a : b; }
static inline float max(const float a, const float b) { return std::fmax(a, b); }

static inline float as_float(const uint x) { float f; std::memcpy(&f, &x, 4); return f; }
static inline uint as_uint(const float x) { uint u; std::memcpy(&u, &x, 4); return u; }
static inline int as_int(const float x) { int i; std::memcpy(&i, &x, 4); return i; }

static inline float vload_half(const ulong o, const half* p) { return half_bits_to_float(p[o]); }
static inline void vstore_half_rte(const float x, const ulong o, half* p) { p[o] = float_to_half_bits_rne(x); }

// work-group functions: present so the text compiles; the harness never launches the kernels using them
static inline uint get_local_id_stub() { return 0u; }
static inline void barrier_stub() {}
static inline uint atomic_add(volatile uint* p, const uint v) { const uint o = *p; *p = o+v; return o; }
static inline float atomic_xchg(volatile float* p, const float v) { const float o = *p; *p = v; return o; }
} // namespace ocl

#define kernel
#define global
#define local
#define get_global_id(i) (ocl::global_id)
#define get_local_id(i) (ocl::get_local_id_stub())
#define barrier(f) (ocl::barrier_stub())
#define CLK_LOCAL_MEM_FENCE 0
#define CLK_GLOBAL_MEM_FENCE 0
#define cl_workgroup_size 64u
