// tiles_f32.cuh -- FP32_FIX work units shared by the single-channel kernels and the batched
// persistent kernel, so that a channel produces bit-identical results alone or in a batch.
//   store_chunk_f32:   NT consecutive events of a channel -> Decays columns, weight, flag
//   average_tile_f32:  one AverageOn tile (HPS_AVG_TILE events) -> its StatsPHSP (thread 0)
//   merge_partials:    the fixed-shape merge of a channel's tile partials
#pragma once
#include "common.h"
#include "store.cuh"

namespace hps {

struct Cols { double* p[HPS_MAX_DAUGHTERS]; };

constexpr int kTileThreads = 256;                      // CTA size of every FP32_FIX work unit
constexpr int kAvgPerThread = HPS_AVG_TILE / kTileThreads;
static_assert(kTileThreads * kAvgPerThread == HPS_AVG_TILE, "tile shape");
constexpr int kFinalThreads = 1024;

// Events [cb, cb + NT) of the call (event index first + e); all NT threads call together.
template <int N, int ENGINE>
__device__ __forceinline__ void store_chunk_f32(const DevChannel& chd, const DevChannelF& ch, const Cols& cols,
                                                double* __restrict__ weights, uint8_t* __restrict__ flags,
                                                uint64_t ukey, uint64_t first, uint64_t n, uint64_t cb,
                                                bool vec32, void* smem)
{
    uint64_t w[3 * N - 4];
    cta_event_words<N, ENGINE, kTileThreads>(chd.key, first + cb, smem, w);
    const uint64_t e = cb + threadIdx.x;
    if (e < n) {
        float p[N][4];
        const f32::EventWeight ew = f32::event_from_words<N, ENGINE>(chd, ch, w, p);
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const double v[4] = {f32::widen_pos(p[k][0]), f32::widen(p[k][1]), f32::widen(p[k][2]),
                                 f32::widen(p[k][3])};
            store_vec4(cols.p[k], e, v, vec32);
        }
        if (weights) weights[e] = ew.weight;
        if (flags) flags[e] = f32::accept(ew, squares3_word(ukey, first + e)) ? 1 : 0;
    }
}

__device__ __forceinline__ void ff_add(float& sh, float& sl, float xh, float xl)
{
    const float s = sh + xh;
    const float bb = s - sh;
    float e = (sh - (s - bb)) + (xh - bb);
    e += sl + xl;
    const float t = s + e;
    sl = e - (t - s);
    sh = t;
}

// AverageOn tile t: thread j takes events t*4096 + j + 256k, k = 0..15, and accumulates their
// prod(pdk) P (the weight without the common factor max_weight) as float-float sums
// W' = sum P, S1' = sum P (f - K), S2' = sum P (f - K)^2 with K its first functor value -- the
// StatsPHSP of those events in closed form once scaled by max_weight in double; the fixed
// warp/CTA tree then merges the per-thread StatsPHSP.  Result valid in thread 0.
template <int N, int ENGINE>
__device__ __forceinline__ hps_stats average_tile_f32(const DevChannel& chd, const DevChannelF& ch,
                                                      const DevFunctor& fn, uint64_t first, uint64_t n,
                                                      uint64_t t, void* smem)
{
    float swh = 0.0f, swl = 0.0f, s1h = 0.0f, s1l = 0.0f, s2h = 0.0f, s2l = 0.0f;
    float K = 0.0f;
    const uint64_t base = t * HPS_AVG_TILE;
    for (int k = 0; k < kAvgPerThread; ++k) {
        const uint64_t cb = base + (uint64_t)k * kTileThreads;
        if (cb >= n) break;                                              // CTA-uniform
        uint64_t w[3 * N - 4];
        cta_event_words<N, ENGINE, kTileThreads>(chd.key, first + cb, smem, w);
        const uint64_t e = cb + threadIdx.x;
        if (e < n) {
            float p[N][4];
            const f32::EventWeight ew = f32::event_from_words<N, ENGINE>(chd, ch, w, p);
            const float f = f32::functor<N>(fn, p);
            if (k == 0) K = f;
            const float d = f - K;
            // P*d and P*d^2 as float-float products
            const float h1 = ew.prod_hi * d;
            const float l1 = fmaf(ew.prod_lo, d, fmaf(ew.prod_hi, d, -h1));
            const float h2 = h1 * d;
            const float l2 = fmaf(l1, d, fmaf(h1, d, -h2));
            ff_add(swh, swl, ew.prod_hi, ew.prod_lo);
            ff_add(s1h, s1l, h1, l1);
            ff_add(s2h, s2l, h2, l2);
        }
    }
    hps_stats acc{0.0, 0.0, 0.0};
    const double W = chd.max_weight * (f32::widen(swh) + f32::widen(swl));
    if (W != 0.0) {
        const double S1 = chd.max_weight * (f32::widen(s1h) + f32::widen(s1l));
        const double S2 = chd.max_weight * (f32::widen(s2h) + f32::widen(s2l));
        const double q = S1 / W;
        acc.w = W;
        acc.mean = f32::widen(K) + q;
        acc.m2 = fma(-S1, q, S2);
    }
    return block_reduce_stats<kTileThreads>(acc);
}

// Thread j of a kFinalThreads CTA folds partials j, j+1024, ... in order, then the fixed CTA
// tree.  Result valid in thread 0.
__device__ __forceinline__ hps_stats merge_partials(const hps_stats* __restrict__ partials, uint64_t ntiles)
{
    hps_stats acc{0.0, 0.0, 0.0};
    for (uint64_t t = threadIdx.x; t < ntiles; t += kFinalThreads) acc = stats_merge(acc, partials[t]);
    return block_reduce_stats<kFinalThreads>(acc);
}

}  // namespace hps
