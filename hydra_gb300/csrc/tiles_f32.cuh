// tiles_f32.cuh -- FP32_FIX work units shared by the single-channel kernels and the batched
// persistent kernel, so that a channel produces bit-identical results alone or in a batch.
//   store_chunk_f32:   NT consecutive events of a channel -> Decays columns, weight, flag
//   average_tile_f32:  one AverageOn tile (HPS_AVG_TILE events) -> its shifted weighted sums
//   merge_sums:        the fixed-shape sum of a call's tile sums -> its StatsPHSP
//   merge_partials:    the fixed-shape StatsPHSP merge of the FP64 form's tile partials
#pragma once
#include "common.h"
#include "store.cuh"

namespace hps {

struct Cols { double* p[HPS_MAX_DAUGHTERS]; };

constexpr int kTileThreads = 256;                      // CTA size of every FP32_FIX work unit
constexpr int kAvgPerThread = HPS_AVG_TILE / kTileThreads;
static_assert(kTileThreads * kAvgPerThread == HPS_AVG_TILE, "tile shape");
constexpr int kFinalThreads = 1024;

// Shared memory of a CTA whose work units exchange the words of two chunks at a time.
template <int N, int ENGINE> struct PairedSmem {
    static constexpr int BYTES = WordShare<N, ENGINE, 2 * kTileThreads>::BYTES2;
};

// Where a storing work unit puts event e of the call: Decays columns, weight, unweight flag.
struct StoreOut {
    Cols cols;
    double* weights;      // may be NULL
    uint8_t* flags;       // may be NULL
    uint64_t ukey;        // splitmix64 of the unweight seed
    int vec32;            // all columns 32-byte aligned
};

template <int N>
__device__ __forceinline__ void store_event_f32(const float (&p)[N][4], const f32::EventWeight& ew,
                                                const Cols& cols, double* __restrict__ weights,
                                                uint8_t* __restrict__ flags, uint64_t ukey, uint64_t first,
                                                uint64_t e, bool vec32)
{
    // the alignment test is uniform: one branch around all N stores, not one per store
    if (vec32) {
#pragma unroll
        for (int k = 0; k < N; ++k)
            st_v4_f64(cols.p[k] + 4 * e, f32::widen_pos(p[k][0]), f32::widen_nz(p[k][1]), f32::widen_nz(p[k][2]),
                      f32::widen_nz(p[k][3]));
    } else {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            st_v2_f64(cols.p[k] + 4 * e, f32::widen_pos(p[k][0]), f32::widen_nz(p[k][1]));
            st_v2_f64(cols.p[k] + 4 * e + 2, f32::widen_nz(p[k][2]), f32::widen_nz(p[k][3]));
        }
    }
    if (weights) weights[e] = ew.weight;
    if (flags) flags[e] = f32::accept(ew, squares3_word(ukey, first + e)) ? 1 : 0;
}

// Events [cb, cb + NT) of the call (event index first + e); all NT threads call together, with
// the word-buffer parity alternating between consecutive calls (cta_event_words).
template <int N, int ENGINE, int NT = kTileThreads>
__device__ __forceinline__ void store_chunk_f32(const DevChannel& chd, const DevChannelF& ch, const Cols& cols,
                                                double* __restrict__ weights, uint8_t* __restrict__ flags,
                                                uint64_t ukey, uint64_t first, uint64_t n, uint64_t cb,
                                                bool vec32, void* smem, int parity)
{
    uint64_t w[3 * N - 4];
    cta_event_words<N, ENGINE, NT>(chd.key, first + cb, smem, w, parity);
    const uint64_t e = cb + threadIdx.x;
    if (e < n) {
        float p[N][4];
        const f32::EventWeight ew = f32::event_from_words<N, ENGINE>(chd, ch, w, p);
        store_event_f32<N>(p, ew, cols, weights, flags, ukey, first, e, vec32);
    }
}

// Events [cb, cb + 2 NT): thread t computes events cb + t and cb + NT + t from one word exchange
// (both are computed whatever n is; only events below n are stored).
template <int N, int ENGINE, int NT>
__device__ __forceinline__ void store_pair_f32(const DevChannel& chd, const DevChannelF& ch, const Cols& cols,
                                               double* __restrict__ weights, uint8_t* __restrict__ flags,
                                               uint64_t ukey, uint64_t first, uint64_t n, uint64_t cb,
                                               bool vec32, void* smem, int parity)
{
    uint64_t wa[3 * N - 4], wb[3 * N - 4];
    cta_event_words_pair<N, ENGINE, NT>(chd.key, first + cb, smem, wa, wb, parity);
    const uint64_t ea = cb + threadIdx.x, eb = ea + NT;
    float pa[N][4], pb[N][4];
    const f32::EventWeight wta = f32::event_from_words<N, ENGINE>(chd, ch, wa, pa);
    const f32::EventWeight wtb = f32::event_from_words<N, ENGINE>(chd, ch, wb, pb);
    if (ea < n) store_event_f32<N>(pa, wta, cols, weights, flags, ukey, first, ea, vec32);
    if (eb < n) store_event_f32<N>(pb, wtb, cols, weights, flags, ukey, first, eb, vec32);
}

// Events [cb, cb + 2 NT) with one word exchange, computed one after the other (thread t: event
// cb + t, then cb + NT + t), so the registers are those of one event.
template <int N, int ENGINE, int NT>
__device__ __forceinline__ void store_pair_seq_f32(const DevChannel& chd, const DevChannelF& ch, const Cols& cols,
                                                   double* __restrict__ weights, uint8_t* __restrict__ flags,
                                                   uint64_t ukey, uint64_t first, uint64_t n, uint64_t cb,
                                                   bool vec32, void* smem, int parity)
{
    const bool shared = cta_words_pair_fill<N, ENGINE, NT>(chd.key, first + cb, smem, parity);
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
        const uint64_t e = cb + (uint64_t)h * NT + threadIdx.x;
        uint64_t w[3 * N - 4];
        if (shared) cta_words_pair_read<N, ENGINE, NT>(smem, parity, h, w);
        else event_words<N, ENGINE>(chd.key, first + e, w);
        if (e < n) {
            float p[N][4];
            const f32::EventWeight ew = f32::event_from_words<N, ENGINE>(chd, ch, w, p);
            store_event_f32<N>(p, ew, cols, weights, flags, ukey, first, e, vec32);
        }
    }
}

// Two threads per event: events [cb, cb + kTileThreads / 2) of the call; threads t and
// t + kTileThreads / 2 (different warps) both compute event cb + t's stage quantities and weight,
// and each computes and stores the daughter pairs of its half (f32::owns_pair); the first half
// stores the weight and the flag.  The same values as store_chunk_f32, bit for bit.
template <int N, int ENGINE, int HALF>
__device__ __forceinline__ void store_half_f32(const DevChannel& chd, const DevChannelF& ch, const Cols& cols,
                                               double* __restrict__ weights, uint8_t* __restrict__ flags,
                                               uint64_t ukey, uint64_t first, uint64_t e, bool vec32,
                                               uint64_t (&w)[3 * N - 4])
{
    constexpr int kForm = N >= f32::kPreciseN ? f32::kFormFull
                          : (N >= f32::kHardMinN && (ENGINE & kPreciseForm) != 0) ? f32::kFormBoosts
                                                                                   : f32::kFormPlain;
    float p[N][4];
    const f32::EventWeight ew = f32::event_body<N, ENGINE, kForm, HALF>(chd, ch, w, p);
#pragma unroll
    for (int k = 0; k < N; ++k) {
        if (!f32::owns_pair<HALF>(k >> 1)) continue;
        const double v[4] = {f32::widen_pos(p[k][0]), f32::widen_nz(p[k][1]), f32::widen_nz(p[k][2]),
                             f32::widen_nz(p[k][3])};
        store_vec4(cols.p[k], e, v, vec32);
    }
    if constexpr (HALF == 0) {
        if (weights) weights[e] = ew.weight;
        if (flags) flags[e] = f32::accept(ew, squares3_word(ukey, first + e)) ? 1 : 0;
    }
}

template <int N, int ENGINE>
__device__ __forceinline__ void store_chunk_split_f32(const DevChannel& chd, const DevChannelF& ch, const Cols& cols,
                                                      double* __restrict__ weights, uint8_t* __restrict__ flags,
                                                      uint64_t ukey, uint64_t first, uint64_t n, uint64_t cb,
                                                      bool vec32, void* smem, int parity)
{
    constexpr int NE = kTileThreads / 2;
    uint64_t w[3 * N - 4];
    cta_event_words_split<N, ENGINE, NE>(chd.key, first + cb, smem, w, parity);
    const uint64_t e = cb + (threadIdx.x % NE);
    if (e < n) {
        if (threadIdx.x < NE) store_half_f32<N, ENGINE, 0>(chd, ch, cols, weights, flags, ukey, first, e, vec32, w);
        else store_half_f32<N, ENGINE, 1>(chd, ch, cols, weights, flags, ukey, first, e, vec32, w);
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

// Weighted sums of one AverageOn tile relative to a shift K0 common to the whole call:
// W = sum w, S1 = sum w (f - K0), S2 = sum w (f - K0)^2.  Tiles combine by addition, and
// {K0 + S1/W, S2 - S1^2/W, W} is the call's StatsPHSP (StatsPHSP.h:38-86) in closed form.
// Stored in the 24-byte partial slot of a tile.
struct hps_sums {
    double s1, s2, w;
};
static_assert(sizeof(hps_sums) == sizeof(hps_stats), "partials hold either form");

__device__ __forceinline__ hps_sums shfl_down_sums(const hps_sums& s, int offset)
{
    return hps_sums{__shfl_down_sync(0xffffffffu, s.s1, offset), __shfl_down_sync(0xffffffffu, s.s2, offset),
                    __shfl_down_sync(0xffffffffu, s.w, offset)};
}

// Fixed-shape CTA tree of additions (NT a multiple of 32, <= 1024); result valid in thread 0.
template <int NT>
__device__ __forceinline__ hps_sums block_reduce_sums(hps_sums s)
{
    constexpr int NWARP = NT / 32;
    __shared__ hps_sums warp_part[NWARP];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const hps_sums o = shfl_down_sums(s, off);
        s.s1 += o.s1; s.s2 += o.s2; s.w += o.w;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_part[warp] = s;
    __syncthreads();
    if (warp == 0) {
        hps_sums t = (lane < NWARP) ? warp_part[lane] : hps_sums{0.0, 0.0, 0.0};
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const hps_sums o = shfl_down_sums(t, off);
            t.s1 += o.s1; t.s2 += o.s2; t.w += o.w;
        }
        s = t;
    }
    __syncthreads();
    return s;
}

// The shift K0: the functor value of the call's first event.  One thread computes it once per
// call (k_shift_f32 / k_batch_shift) into the first 4 bytes of the call's hps_stats output, which
// the tile and merge kernels read before the merge overwrites it with the result.
template <int N, int ENGINE>
__device__ __forceinline__ float call_shift(const DevChannel& chd, const DevChannelF& ch, const DevFunctor& fn,
                                            uint64_t first)
{
    uint64_t w[3 * N - 4];
    event_words<N, ENGINE>(chd.key, first, w);
    float p[N][4];
    f32::event_from_words<N, ENGINE>(chd, ch, w, p);
    return f32::functor<N>(fn, p);
}

// AverageOn tile t: thread j takes events t*4096 + j + 256k, k = 0..15, and accumulates their
// prod(pdk) P (the weight without the common factor max_weight) as float-float sums
// sum P, sum P (f - K0), sum P (f - K0)^2, converted to double and scaled by max_weight; the
// fixed CTA tree adds the per-thread sums.  Result valid in thread 0.  With STORE, every event is
// also stored (Generate and AverageOn of the same events in one pass): the sums are those of the
// plain tile, bit for bit, and the stored events those of store_chunk_f32.
// With MOTHERS (AverageMothers), event e is boosted by mothers[e] (a Vector4R column) and the
// functor sees (mother, daughter 0, ..., daughter N-1).
template <int N>
__device__ __forceinline__ void load_mother(const double* __restrict__ mothers, uint64_t e, double (&mo)[4])
{
    const double2 a = __ldg(reinterpret_cast<const double2*>(mothers + 4 * e));
    const double2 b = __ldg(reinterpret_cast<const double2*>(mothers + 4 * e) + 1);
    mo[0] = a.x; mo[1] = a.y; mo[2] = b.x; mo[3] = b.y;
}

template <int N>
__device__ __forceinline__ float mother_functor_f32(const DevFunctor& fn, const f32::MotherFrame& f,
                                                    const float (&p)[N][4])
{
    float pm[N + 1][4];
    pm[0][0] = f.e; pm[0][1] = f.px; pm[0][2] = f.py; pm[0][3] = f.pz;
#pragma unroll
    for (int k = 0; k < N; ++k)
#pragma unroll
        for (int c = 0; c < 4; ++c) pm[k + 1][c] = p[k][c];
    return f32::functor<N + 1>(fn, pm);
}

template <int N, int ENGINE, bool STORE = false, bool MOTHERS = false, bool PAIRED = false>
__device__ __forceinline__ hps_sums average_tile_f32(const DevChannel& chd, const DevChannelF& ch,
                                                     const DevFunctor& fn, uint64_t first, uint64_t n,
                                                     uint64_t t, float K0, void* smem,
                                                     const StoreOut* so = nullptr,
                                                     const double* __restrict__ mothers = nullptr)
{
    static_assert(!(STORE && MOTHERS), "a storing tile keeps the events in the decay's rest frame");
    float swh = 0.0f, swl = 0.0f, s1h = 0.0f, s1l = 0.0f, s2h = 0.0f, s2l = 0.0f;
    const uint64_t base = t * HPS_AVG_TILE;
    // one event of the tile from its words: functor, weight, and the shifted sums
    auto add_event = [&](uint64_t e, uint64_t (&w)[3 * N - 4]) {
            float p[N][4];
            const f32::EventWeight ew = f32::event_from_words<N, ENGINE>(chd, ch, w, p);
            if constexpr (STORE)
                store_event_f32<N>(p, ew, so->cols, so->weights, so->flags, so->ukey, first, e, so->vec32 != 0);
            float d;
            if constexpr (MOTHERS) {
                double mo[4];
                load_mother<N>(mothers, e, mo);
                const f32::MotherFrame mf = f32::mother_frame(mo);
                f32::boost_to_mother<N>(p, ch.m2, mf);
                d = mother_functor_f32<N>(fn, mf, p) - K0;
            } else {
                d = f32::functor<N>(fn, p) - K0;
            }
            // P*d and P*d^2 as float-float products
            const float h1 = ew.prod_hi * d;
            const float l1 = fmaf(ew.prod_lo, d, fmaf(ew.prod_hi, d, -h1));
            const float h2 = h1 * d;
            const float l2 = fmaf(l1, d, fmaf(h1, d, -h2));
            ff_add(swh, swl, ew.prod_hi, ew.prod_lo);
            ff_add(s1h, s1l, h1, l1);
            ff_add(s2h, s2l, h2, l2);
    };
    if constexpr (PAIRED) {
        // chunks in pairs: one word exchange for two chunks, a thread's two events in turn (the same
        // events in the same order as one chunk at a time, so the same sums bit for bit)
        static_assert(kAvgPerThread % 2 == 0, "chunks in pairs");
        for (int kp = 0; kp < kAvgPerThread / 2; ++kp) {
            const uint64_t cb = base + (uint64_t)(2 * kp) * kTileThreads;
            if (cb >= n) break;                                          // CTA-uniform
            const bool shared = cta_words_pair_fill<N, ENGINE, kTileThreads>(chd.key, first + cb, smem, kp);
#pragma unroll 1
            for (int h = 0; h < 2; ++h) {
                const uint64_t e = cb + (uint64_t)h * kTileThreads + threadIdx.x;
                uint64_t w[3 * N - 4];
                if (shared) cta_words_pair_read<N, ENGINE, kTileThreads>(smem, kp, h, w);
                else event_words<N, ENGINE>(chd.key, first + e, w);
                if (e < n) add_event(e, w);
            }
        }
    } else {
        for (int k = 0; k < kAvgPerThread; ++k) {
            const uint64_t cb = base + (uint64_t)k * kTileThreads;
            if (cb >= n) break;                                          // CTA-uniform
            uint64_t w[3 * N - 4];
            cta_event_words<N, ENGINE, kTileThreads>(chd.key, first + cb, smem, w, k);
            const uint64_t e = cb + threadIdx.x;
            if (e < n) add_event(e, w);
        }
    }
    hps_sums acc;
    acc.w = chd.max_weight * (f32::widen(swh) + f32::widen(swl));
    acc.s1 = chd.max_weight * (f32::widen(s1h) + f32::widen(s1l));
    acc.s2 = chd.max_weight * (f32::widen(s2h) + f32::widen(s2l));
    return block_reduce_sums<kTileThreads>(acc);
}

// Thread j of a kFinalThreads CTA adds tile sums j, j+1024, ... in order, the fixed CTA tree adds
// the threads' sums, and the call's StatsPHSP is formed from them.  Result valid in thread 0.
template <int N, int ENGINE>
__device__ __forceinline__ hps_stats merge_sums(const DevChannel& chd, const DevChannelF& ch, const DevFunctor& fn,
                                                uint64_t first, const hps_stats* __restrict__ partials,
                                                uint64_t ntiles, float K0)
{
    const hps_sums* tiles = reinterpret_cast<const hps_sums*>(partials);
    hps_sums acc{0.0, 0.0, 0.0};
    for (uint64_t t = threadIdx.x; t < ntiles; t += kFinalThreads) {
        const hps_sums v = tiles[t];
        acc.s1 += v.s1; acc.s2 += v.s2; acc.w += v.w;
    }
    const hps_sums tot = block_reduce_sums<kFinalThreads>(acc);
    hps_stats r{0.0, 0.0, 0.0};
    if (tot.w != 0.0) {
        const double q = tot.s1 / tot.w;
        r.w = tot.w;
        r.mean = f32::widen(K0) + q;
        r.m2 = fma(-tot.s1, q, tot.s2);
    }
    return r;
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
