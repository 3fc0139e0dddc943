// Host stand-ins for the CUDA intrinsics that the event headers use, so that the FP32_FIX event body
// (hydra_gb300/csrc/genbod_f32.cuh) compiles for the CPU and can be run against the FP64 body of
// the same events.  Test infrastructure only.
//
// Each stand-in is the IEEE operation the intrinsic names (x86-64 and AArch64 both evaluate float and
// double in their own precision; the build uses -ffp-contract=off, so no product is fused unless the
// source says fmaf).  The two hardware approximations of the float body, rcp.approx and
// rsqrt.approx, are replaced by 1/x and 1/sqrt(x) when the headers are copied (build.sh); they are
// about one ulp away from those, and each is followed by a Newton step in the body.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#define __shared__ static
#define __align__(x) alignas(x)

struct float2 { float x, y; };
inline float2 make_float2(float a, float b) { return {a, b}; }
struct ulonglong2 { unsigned long long x, y; };
inline ulonglong2 make_ulonglong2(unsigned long long a, unsigned long long b) { return {a, b}; }
struct dim3s { unsigned x = 0, y = 0, z = 0; };
static dim3s threadIdx, blockIdx, blockDim, gridDim;
inline void __syncthreads() {}
template <class T> inline T __ldg(const T* p) { return *p; }

inline float2 __ffma2_rn(float2 a, float2 b, float2 c) { return {std::fmaf(a.x, b.x, c.x), std::fmaf(a.y, b.y, c.y)}; }
inline float2 __fmul2_rn(float2 a, float2 b) { return {a.x * b.x, a.y * b.y}; }
inline float2 __fadd2_rn(float2 a, float2 b) { return {a.x + b.x, a.y + b.y}; }
inline float __uint2float_rn(uint32_t x) { return static_cast<float>(x); }
inline float __int2float_rn(int x) { return static_cast<float>(x); }
inline uint32_t __float_as_uint(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float __uint_as_float(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
inline float __int_as_float(int u) { float f; std::memcpy(&f, &u, 4); return f; }
inline double __hiloint2double(int hi, int lo)
{
    const uint64_t b = (static_cast<uint64_t>(static_cast<uint32_t>(hi)) << 32) | static_cast<uint32_t>(lo);
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}
inline long long __double_as_longlong(double d) { long long b; std::memcpy(&b, &d, 8); return b; }
inline int __clzll(long long x) { return x ? __builtin_clzll(static_cast<unsigned long long>(x)) : 64; }
inline unsigned long long __umul64hi(unsigned long long a, unsigned long long b)
{
    return static_cast<unsigned long long>((static_cast<unsigned __int128>(a) * b) >> 64);
}
inline double __dadd_rn(double a, double b) { return a + b; }
inline double __dsub_rn(double a, double b) { return a - b; }
inline double __dmul_rn(double a, double b) { return a * b; }
inline double __ddiv_rn(double a, double b) { return a / b; }
inline double __dsqrt_rn(double a) { return std::sqrt(a); }
inline double __ull2double_rn(unsigned long long x) { return static_cast<double>(x); }
inline float __fsqrt_rn(float x) { return std::sqrt(x); }
using std::fmaf;
using std::sqrt;
inline float rsqrtf(float x) { return 1.0f / std::sqrt(x); }
