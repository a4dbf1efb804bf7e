// ref_shim.h -- an OpenCL C 1.1 work-item environment on the CPU under which
// the reference's own kernel source compiles as C++ and runs.  TEST
// INFRASTRUCTURE ONLY: the tests use it to run the reference's kernel text
// beside the oracle; the product never includes it.
//
// The reference (JuantAldea/trax) keeps its OpenCL C kernels as source text
// inside KERNEL_CLASS(...) macros in src/algorithms/*.h.  ref_extract.py
// copies that text, at build time and into oracle/_ref/ only, into a C++
// file that includes this header and wraps the kernels in namespace refk.
// This header supplies what the text needs from an OpenCL implementation:
//
//   * address-space qualifiers (__kernel, __global, __local) as empty macros;
//   * the scalar and vector types (uint, uchar, ulong, float2, float3, uint2)
//     with OpenCL's component-wise operators;
//   * the built-ins the kernels call, with the semantics the oracle and the
//     CUDA kernels fix for them (trax_math.h): atan2, acos, atan, asinh from
//     the shared polynomial implementations, correctly rounded sqrt and
//     division, sign(0) = 0, max(x, y) = x < y ? y : x, normalize(v) =
//     v / sqrt(dot(v, v)) with dot summed x, y, then z;
//   * float -> integer conversions of floor(...) results through the same
//     saturating definition as the oracle (f2u_sat / f2i_sat): floor returns
//     a value that converts to uint or int that way (and adds integers in
//     float first, as C does with floor(x) + 1);
//   * atomics as plain read-modify-writes (work-items run one at a time);
//   * get_global_id and the other work-item functions, set by the NDRange
//     runner in ref_driver.cpp, and barrier(), which switches to the next
//     work-item of the work-group (ucontext fibers) when the group has more
//     than one work-item.
#pragma once

#include <stddef.h>
#include <stdint.h>

#include "trax_math.h"

namespace refrt {

// The NDRange state of the work-item that is running.  One per host thread,
// so independent event groups can run on several threads.
struct ItemState {
  size_t gid[3];
  size_t lid[3];
  size_t grp[3];
  size_t gsz[3];
  size_t lsz[3];
  bool fibers;      // the work-group runs as fibers (barrier() switches)
  size_t group_items;
};
extern thread_local ItemState item;

void barrier_switch();  // ref_driver.cpp

}  // namespace refrt

namespace refk {

typedef unsigned int uint;
typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned long ulong;  // 64 bits on the LP64 targets this builds for
static_assert(sizeof(ulong) == 8, "OpenCL ulong is 64 bits");

#define __kernel
#define __global
#define __local
#define __constant const
#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2
#define M_PI_F TRAX_PI_F
#define PRINTF(a)

// ----------------------------------------------------------- work-items
inline size_t get_global_id(uint d) { return d < 3 ? refrt::item.gid[d] : 0; }
inline size_t get_local_id(uint d) { return d < 3 ? refrt::item.lid[d] : 0; }
inline size_t get_group_id(uint d) { return d < 3 ? refrt::item.grp[d] : 0; }
inline size_t get_global_size(uint d) { return d < 3 ? refrt::item.gsz[d] : 1; }
inline size_t get_local_size(uint d) { return d < 3 ? refrt::item.lsz[d] : 1; }
inline size_t get_num_groups(uint d) { return d < 3 ? refrt::item.gsz[d] / refrt::item.lsz[d] : 1; }

inline void barrier(int) {
  if (refrt::item.group_items > 1) refrt::barrier_switch();
}

template <class T>
inline void prefetch(const T*, size_t) {}

// ---------------------------------------------------------------- types
struct float2 {
  float x, y;
  float2() = default;
  float2(float a, float b) : x(a), y(b) {}
  explicit float2(float s) : x(s), y(s) {}
};
struct float3 {
  float x, y, z;
  float3() = default;
  float3(float a, float b, float c) : x(a), y(b), z(c) {}
  explicit float3(float s) : x(s), y(s), z(s) {}
};
struct float4 {
  float x, y, z, w;
  float4() = default;
  float4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  explicit float4(float s) : x(s), y(s), z(s), w(s) {}
};
struct uint2 {
  uint x, y;
  uint2() = default;
  uint2(uint a, uint b) : x(a), y(b) {}
  explicit uint2(uint s) : x(s), y(s) {}
};
struct uint4 {
  uint x, y, z, w;
  uint4() = default;
  uint4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
  explicit uint4(uint s) : x(s), y(s), z(s), w(s) {}
};
static_assert(sizeof(uint2) == 8, "uint2 buffers hold two 32-bit words");

inline float2 operator+(float2 a, float2 b) { return float2(a.x + b.x, a.y + b.y); }
inline float2 operator-(float2 a, float2 b) { return float2(a.x - b.x, a.y - b.y); }
inline float2 operator-(float2 a) { return float2(-a.x, -a.y); }
inline float2 operator*(float2 a, float s) { return float2(a.x * s, a.y * s); }
inline float2 operator*(float s, float2 a) { return float2(s * a.x, s * a.y); }
inline float2 operator/(float2 a, float s) { return float2(trax::div_(a.x, s), trax::div_(a.y, s)); }
inline float3 operator+(float3 a, float3 b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(float3 a, float3 b) { return float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator-(float3 a) { return float3(-a.x, -a.y, -a.z); }
inline float3 operator*(float3 a, float s) { return float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator*(float s, float3 a) { return float3(s * a.x, s * a.y, s * a.z); }
inline float3 operator/(float3 a, float s) {
  return float3(trax::div_(a.x, s), trax::div_(a.y, s), trax::div_(a.z, s));
}

// ------------------------------------------------------------- built-ins
inline float sqrt(float x) { return trax::sqrt_(x); }
inline float fabs(float x) { return trax::fabs_(x); }
inline float sign(float x) { return trax::cl_sign(x); }
inline float atan2(float y, float x) { return trax::atan2_(y, x); }
inline float acos(float x) { return trax::acos_(x); }
inline float atan(float x) { return trax::atan_(x); }
inline float asinh(float x) { return trax::asinh_(x); }

// floor(x): the kernels convert every floor result to an integer, directly
// or after adding an integer.  C leaves out-of-range and NaN conversions
// undefined and OpenCL leaves them to the implementation; this value
// converts with the saturating definition of the oracle and the CUDA kernels.
struct FloorValue {
  float v;
  operator uint() const { return trax::f2u_sat(v); }
  operator int() const { return trax::f2i_sat(v); }
};
inline FloorValue floor(float x) { return FloorValue{trax::floor_(x)}; }
inline FloorValue operator+(FloorValue a, int b) { return FloorValue{a.v + (float)b}; }

inline int max(int a, int b) { return a > b ? a : b; }
inline uint max(uint a, uint b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline uint min(uint a, uint b) { return a < b ? a : b; }
inline float max(float x, float y) { return trax::cl_max(x, y); }

inline float dot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
inline float dot(float3 a, float3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float3 cross(float3 a, float3 b) {
  return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(float2 v) { return trax::sqrt_(dot(v, v)); }
inline float length(float3 v) { return trax::sqrt_(dot(v, v)); }
inline float distance(float3 a, float3 b) { return length(a - b); }
inline float2 normalize(float2 v) { return v / length(v); }
inline float3 normalize(float3 v) { return v / length(v); }

// Atomics: work-items run one at a time, so a read-modify-write is atomic.
template <class V>
inline uint atomic_inc(volatile V* p) {
  V old = *p;
  *p = old + 1;
  return (uint)old;
}
template <class V, class A>
inline V atomic_add(volatile V* p, A v) {
  V old = *p;
  *p = old + (V)v;
  return old;
}
template <class V, class A>
inline V atomic_or(volatile V* p, A v) {
  V old = *p;
  *p = old | (V)v;
  return old;
}
template <class V, class A>
inline V atomic_max(volatile V* p, A v) {
  V old = *p;
  *p = old > (V)v ? old : (V)v;
  return old;
}

}  // namespace refk

// ---------------------------------------------------------------------------
// The accessors the reference's track evaluation (TripletBuilder.cpp, copied
// into ref_tracks.cpp) calls: HitCollection::getValue(HitId/GlobalX/Y/Z(), i)
// (HitCollection.h:23-62) and TrackletCollection::getValue(TrackletHit1/2/3(),
// t) (TrackletCollection.h:32-78), over plain arrays.
#include <algorithm>
#include <iostream>
#include <list>
#include <map>
#include <memory>
#include <utility>
#include <vector>

namespace reftr {
typedef unsigned int uint;
struct HitId {};
struct GlobalX {};
struct GlobalY {};
struct GlobalZ {};
struct TrackletHit1 {};
struct TrackletHit2 {};
struct TrackletHit3 {};

struct HitCollection {
  const uint32_t* hitId = nullptr;  // simulated track of each hit
  const float* x = nullptr;         // coordinates (printTrack only; may be null)
  const float* y = nullptr;
  const float* z = nullptr;
  uint getValue(HitId, uint i) const { return hitId[i]; }
  float getValue(GlobalX, uint i) const { return x ? x[i] : 0.0f; }
  float getValue(GlobalY, uint i) const { return y ? y[i] : 0.0f; }
  float getValue(GlobalZ, uint i) const { return z ? z[i] : 0.0f; }
};

struct TrackletCollection {
  const uint32_t* h1 = nullptr;
  const uint32_t* h2 = nullptr;
  const uint32_t* h3 = nullptr;
  uint getValue(TrackletHit1, uint t) const { return h1[t]; }
  uint getValue(TrackletHit2, uint t) const { return h2[t]; }
  uint getValue(TrackletHit3, uint t) const { return h3[t]; }
};
}  // namespace reftr
