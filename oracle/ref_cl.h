/*
 * ref_cl.h -- OpenCL C 1.1 built-ins for compiling the reference's own kernel
 * text as C++ on the host, plus a work-group emulator to launch it.
 *
 * TEST INFRASTRUCTURE ONLY (the reference-kernel side of the oracle).  The
 * reference keeps its device code as OpenCL C inside KERNEL_CLASS macro
 * arguments (src/algorithms/GridBuilder.h:48-427, PrefixSum.h:55-245,
 * PairGeneratorBeamspot.h:43-525, PairGeneratorSector.h:41-234,
 * TripletThetaPhiPredictor.h:46-497, TripletThetaPhiFilter.h:50-313).
 * oracle/ref_build.py lifts that text out of the reference tree into
 * oracle/_ref/ and compiles it against this header; ref_host.cpp restates the
 * host chain around it.  Nothing here is linked into the product.
 *
 * The built-ins the reference never defines itself come from the OpenCL
 * vendor runtime; here they take the meanings the parity contract fixes for
 * the CUDA kernels as well:
 *   - atan2 / acos / atan: the project math (trax_math.h);
 *   - sqrt, division: IEEE, correctly rounded; no contraction (the recipe
 *     builds with -ffp-contract=off);
 *   - sign(): 1, -1, +/-0 for +/-0, 0 for NaN; max/min on floats:
 *     "y if x < y, otherwise x";
 *   - normalize(v) = v / sqrt(dot(v, v)); cross() the textbook formula;
 *   - float-to-integer conversions of floor() results: trax_f2u / trax_f2i,
 *     a two's-complement target (floor() returns a value type whose integer
 *     conversions route through them);
 *   - work-items of a group run one at a time, in local-id order, switching
 *     only at barrier(); atomics are relaxed read-modify-writes.
 * With one worker, work-groups run one after another in group-id order (x
 * fastest), so every racy ordering in the reference resolves to the
 * sequential one.  With several workers (timing only) work-groups run in
 * parallel, as on an OpenCL CPU device, and the races are real again.
 */
#ifndef TRAX_REF_CL_H
#define TRAX_REF_CL_H

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>

#include "../trax_gb300/csrc/trax_math.h"

#define __kernel inline
#define __global
#define __local
#define __constant
#define __private
#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2
#define M_PI_F 3.14159274101257324219f
/* The reference's non-PROLIX oclDEFINES (KernelWrapper.hpp:24-27) and
 * PrefixSum's bank-offset macro (PrefixSum.cpp:4-6). */
#define PRINTF(a)
#define MEMORY_BANK_COUNT (16)
#define LOG2_MEMORY_BANK_COUNT (4)
#define MEMORY_BANK_OFFSET(index) ((index) >> LOG2_MEMORY_BANK_COUNT)

namespace refcl {

typedef uint32_t uint;
typedef uint64_t ulong;
typedef unsigned char uchar;

struct uint2 { uint x, y; };
struct float2 { float x, y; };
struct float3 { float x, y, z; };

inline float2 make_float2(float a, float b) { return float2{a, b}; }
inline float3 make_float3(float a, float b, float c) { return float3{a, b, c}; }
inline uint2 make_uint2(uint a, uint b) { return uint2{a, b}; }

inline float2 operator-(float2 a) { return float2{-a.x, -a.y}; }
inline float2 operator-(float2 a, float2 b) { return float2{a.x - b.x, a.y - b.y}; }
inline float3 operator-(float3 a) { return float3{-a.x, -a.y, -a.z}; }
inline float3 operator-(float3 a, float3 b) { return float3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float3 operator+(float3 a, float3 b) { return float3{a.x + b.x, a.y + b.y, a.z + b.z}; }

inline float3 cross(float3 a, float3 b)
{
    return float3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float3 normalize(float3 v)
{
    const float s = ::sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    return float3{v.x / s, v.y / s, v.z / s};
}
inline float2 normalize(float2 v)
{
    const float s = ::sqrtf(v.x * v.x + v.y * v.y);
    return float2{v.x / s, v.y / s};
}

inline float sqrt(float v) { return ::sqrtf(v); }
inline float fabs(float v) { return ::fabsf(v); }
inline float sign(float v) { return trax_signf(v); }
inline float atan2(float y, float x) { return trax_atan2f(y, x); }
inline float acos(float x) { return trax_acosf(x); }
inline float atan(float x) { return trax_atanf(x); }

/* floor() result: a float whose conversions to the integer types follow
 * trax_f2u / trax_f2i.  Arithmetic with an integer stays in float, as in
 * OpenCL C (floor(v) + 1 is a float). */
struct floor_value {
    float v;
    operator float() const { return v; }
    operator uint() const { return trax_f2u(v); }
    operator int() const { return trax_f2i(v); }
};
inline floor_value floor(float v) { return floor_value{::floorf(v)}; }
inline floor_value operator+(floor_value a, int b) { return floor_value{a.v + (float)b}; }
inline floor_value operator+(floor_value a, uint b) { return floor_value{a.v + (float)b}; }
inline floor_value operator-(floor_value a, int b) { return floor_value{a.v - (float)b}; }
inline floor_value operator-(floor_value a, uint b) { return floor_value{a.v - (float)b}; }

inline float max(float a, float b) { return trax_maxf(a, b); }
inline float min(float a, float b) { return trax_minf(a, b); }
inline int max(int a, int b) { return a < b ? b : a; }
inline int min(int a, int b) { return b < a ? b : a; }
inline uint max(uint a, uint b) { return a < b ? b : a; }
inline uint min(uint a, uint b) { return b < a ? b : a; }

template <class T> inline T atomic_inc(T *p) { return __atomic_fetch_add(p, (T)1, __ATOMIC_RELAXED); }
template <class T, class V> inline T atomic_add(T *p, V v)
{
    return __atomic_fetch_add(p, (T)v, __ATOMIC_RELAXED);
}
template <class T, class V> inline T atomic_or(T *p, V v)
{
    return __atomic_fetch_or(p, (T)v, __ATOMIC_RELAXED);
}
template <class T> inline void prefetch(const T *, size_t) {}

/* ---- NDRange and work-group emulation ----------------------------------- */
struct NDRange {
    size_t global[3];
    size_t local[3];
};

struct WorkItem {
    size_t gid[3], lid[3], grp[3];
};

extern const NDRange *g_range;
extern thread_local const WorkItem *g_item;

inline size_t get_global_id(uint d) { return g_item->gid[d]; }
inline size_t get_local_id(uint d) { return g_item->lid[d]; }
inline size_t get_group_id(uint d) { return g_item->grp[d]; }
inline size_t get_global_size(uint d) { return g_range->global[d]; }
inline size_t get_local_size(uint d) { return g_range->local[d]; }
inline size_t get_num_groups(uint d) { return g_range->global[d] / g_range->local[d]; }

/* Yields to the next work-item of the group; a no-op when the group has one
 * work-item or the kernel was launched without barriers. */
void barrier(int flags);

}  // namespace refcl

#endif
