// store.cuh -- output stores and the AverageOn merge.
#pragma once
#include <cstdint>
#include "../../include/hps.h"

namespace hps {

// One Vector4R = 32 bytes.  A warp writing 32 consecutive events covers 1 KiB
// contiguous per column, so each 256-bit store instruction is fully coalesced.
__device__ __forceinline__ void st_v4_f64(double* p, double a, double b, double c, double d)
{
    asm volatile("st.global.v4.f64 [%0], {%1, %2, %3, %4};" ::"l"(p), "d"(a), "d"(b), "d"(c), "d"(d)
                 : "memory");
}

__device__ __forceinline__ void st_v2_f64(double* p, double a, double b)
{
    asm volatile("st.global.v2.f64 [%0], {%1, %2};" ::"l"(p), "d"(a), "d"(b) : "memory");
}

__device__ __forceinline__ void store_vec4(double* col, uint64_t e, const double (&v)[4], bool vec32)
{
    double* q = col + 4 * e;
    if (vec32) {
        st_v4_f64(q, v[0], v[1], v[2], v[3]);
    } else {
        st_v2_f64(q, v[0], v[1]);
        st_v2_f64(q + 2, v[2], v[3]);
    }
}

// AddStatsPHSP (hydra/detail/functors/StatsPHSP.h:67-84), separately rounded in the
// reference's order.  Merging two empty partials (W = 0) keeps the left one instead of
// producing 0/0.
__device__ __forceinline__ hps_stats stats_merge(const hps_stats& x, const hps_stats& y)
{
    const double w = __dadd_rn(x.w, y.w);
    if (w == 0.0) return x;
    const double delta = __dsub_rn(y.mean, x.mean);
    const double delta2 = __dmul_rn(delta, delta);
    hps_stats r;
    r.w = w;
    r.mean = __ddiv_rn(__dadd_rn(__dmul_rn(x.mean, x.w), __dmul_rn(y.mean, y.w)), w);
    r.m2 = __dadd_rn(x.m2, y.m2);
    r.m2 = __dadd_rn(r.m2, __ddiv_rn(__dmul_rn(__dmul_rn(delta2, x.w), y.w), w));
    return r;
}

__device__ __forceinline__ hps_stats shfl_down_stats(const hps_stats& s, int offset)
{
    hps_stats o;
    o.mean = __shfl_down_sync(0xffffffffu, s.mean, offset);
    o.m2 = __shfl_down_sync(0xffffffffu, s.m2, offset);
    o.w = __shfl_down_sync(0xffffffffu, s.w, offset);
    return o;
}

// Fixed-shape warp tree: lane l merges lane l+off for off = 16, 8, 4, 2, 1.  Lane 0 holds
// the warp's result, which depends only on the 32 inputs and their lane order.
__device__ __forceinline__ hps_stats warp_reduce_stats(hps_stats s)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const hps_stats o = shfl_down_stats(s, off);
        s = stats_merge(s, o);
    }
    return s;
}

// Fixed-shape block tree for a block of NT threads (NT a multiple of 32, <= 1024).
// Result valid in thread 0.
template <int NT>
__device__ __forceinline__ hps_stats block_reduce_stats(hps_stats s)
{
    constexpr int NWARP = NT / 32;
    __shared__ hps_stats warp_part[NWARP];
    s = warp_reduce_stats(s);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_part[warp] = s;
    __syncthreads();
    if (warp == 0) {
        hps_stats t = (lane < NWARP) ? warp_part[lane] : hps_stats{0.0, 0.0, 0.0};
        t = warp_reduce_stats(t);
        s = t;
    }
    __syncthreads();
    return s;
}

}  // namespace hps
