/*
 * hps_user_kernels.cuh -- the phase-space kernels with a user functor compiled in.
 *
 * A functor that is not one of the C ABI's menu entries (hydra::hps_fn::One / Mass2 / BW2) cannot
 * cross into libhps.so, so hydra::PhaseSpace::AverageOn / Evaluate and hydra::Decays::Unweight /
 * GetEventWeights instantiate these templates in the caller's own translation unit, which must be
 * compiled by nvcc for sm_103a.  The functor is called in device code as the reference calls it
 * (hydra/detail/functors/AverageMother.h:272-292, EvalMother.h:285-307): on a hydra::tuple of the
 * event's N daughters, as Vector4R; with (mother, daughters...) in the per-event-mother form; on
 * the Decays' own column types in PhaseSpaceReweight.  The events are the library's: the same
 * streams and, in the FP64 form, the same separately rounded operations as the reference
 * (hydra_gb300/csrc/genbod.cuh); in the FP32_FIX form the float kinematics of genbod_f32.cuh,
 * widened to double before the functor sees them.  The AverageOn reduction is the fixed tile tree
 * of hps_average_on: tiles of HPS_AVG_TILE events folded with AddStatsPHSP (StatsPHSP.h:67-84)
 * lane by lane and then across the CTA, the tile partials merged in one CTA in a fixed order, so
 * the result does not depend on the launch shape.  Kernels defined here are templates, so that
 * every translation unit may instantiate them.
 */
#ifndef HYDRA_HPS_USER_KERNELS_CUH_
#define HYDRA_HPS_USER_KERNELS_CUH_

#if !defined(__CUDACC__)
#error "hps_user_kernels.cuh holds device code: compile this translation unit with nvcc"
#endif

#include <cuda_runtime.h>

#include <cstdint>
#include <tuple>
#include <type_traits>
#include <utility>

#include "../../../hydra_gb300/csrc/genbod.cuh"
#include "../../../hydra_gb300/csrc/genbod_f32.cuh"
#include "../../../hydra_gb300/csrc/store.cuh"
#include "../../../hydra_gb300/csrc/tiles_f32.cuh"

namespace hydra {
namespace detail {
namespace user {

constexpr int kThreads = 256;                          // CTA of the tile kernels
constexpr int kPerThread = HPS_AVG_TILE / kThreads;    // events per thread and tile
constexpr int kFinal = 1024;                           // CTA of the merges

static_assert(kThreads * kPerThread == HPS_AVG_TILE, "tile shape");

// The event as the reference's functors receive it: a tuple of N Vector4R.
template <typename V, size_t N, size_t... I>
__host__ __device__ inline auto as_tuple(const double (&p)[N][4], std::index_sequence<I...>)
{
    return hydra::tuple<decltype((void)I, V())...>(V(p[I][0], p[I][1], p[I][2], p[I][3])...);
}

template <typename V, size_t N>
__host__ __device__ inline auto event_tuple(const double (&p)[N][4])
{
    return as_tuple<V>(p, std::make_index_sequence<N>{});
}

// The event as a tuple of given element types (each constructible from a Vector4R V): the
// Decays' own column types, which PhaseSpaceReweight hands its functor (Decays.inl:383).
template <typename Tup, typename V, size_t N, size_t... I>
__host__ __device__ inline Tup as_typed_tuple(const double (&p)[N][4], std::index_sequence<I...>)
{
    return Tup(typename std::tuple_element<I, Tup>::type(V(p[I][0], p[I][1], p[I][2], p[I][3]))...);
}

// (mother, daughters...) for the per-event-mother form.
template <typename V, size_t N, size_t... I>
__host__ __device__ inline auto as_tuple_m(const double (&mo)[4], const double (&p)[N][4], std::index_sequence<I...>)
{
    return hydra::tuple<V, decltype((void)I, V())...>(V(mo[0], mo[1], mo[2], mo[3]),
                                                       V(p[I][0], p[I][1], p[I][2], p[I][3])...);
}

// One event in the requested form: FP64 (the reference's arithmetic) or FP32_FIX (float
// kinematics; ENGINE may carry hps::kPreciseForm).  p in double either way; returns the
// generation-time weight.
template <int N, int ENGINE, int PREC>
__device__ __forceinline__ double event(const hps::DevChannel& ch, const hps::DevChannelF& chf, uint64_t evt,
                                        double (&p)[N][4])
{
    if constexpr (PREC == HPS_PREC_FP64) {
        return hps::f64::event<N, hps::engine_of(ENGINE)>(ch, evt, p);
    } else {
        uint64_t w[3 * N - 4];
        hps::event_words<N, hps::engine_of(ENGINE)>(ch.key, evt, w);
        float q[N][4];
        const hps::f32::EventWeight ew = hps::f32::event_from_words<N, ENGINE>(ch, chf, w, q);
#pragma unroll
        for (int k = 0; k < N; ++k) {
            p[k][0] = hps::f32::widen_pos(q[k][0]);
#pragma unroll
            for (int c = 1; c < 4; ++c) p[k][c] = hps::f32::widen(q[k][c]);
        }
        return ew.weight;
    }
}

// AverageOn (AverageMother): tile t folds events t*HPS_AVG_TILE + j + 256 k of the call, thread j
// in order, then the CTA tree; partials[t] gets the tile's StatsPHSP.
template <int N, int ENGINE, int PREC, typename V, typename F>
__global__ void __launch_bounds__(kThreads)
k_average_tiles(hps::DevChannel ch, hps::DevChannelF chf, F f, uint64_t first, uint64_t n, uint64_t ntiles,
                hps_stats* __restrict__ partials)
{
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        hps_stats acc{0.0, 0.0, 0.0};
        const uint64_t base = t * HPS_AVG_TILE + threadIdx.x;
        for (int k = 0; k < kPerThread; ++k) {
            const uint64_t e = base + (uint64_t)k * kThreads;
            if (e < n) {
                double p[N][4];
                hps_stats y;
                y.w = event<N, ENGINE, PREC>(ch, chf, first + e, p);
                y.mean = static_cast<double>(f(event_tuple<V>(p)));
                y.m2 = 0.0;
                acc = hps::stats_merge(acc, y);
            }
        }
        const hps_stats r = hps::block_reduce_stats<kThreads>(acc);
        if (threadIdx.x == 0) partials[t] = r;
    }
}

// One event of the per-event-mother form (AverageMothers.h:134-285): generated at the channel's
// ECM and boosted into the frame of its mother mo.  FP64: the reference's arithmetic; FP32_FIX:
// the float event of genbod_f32.cuh with the light-cone boost into the mother's frame, widened.
template <int N, int ENGINE, int PREC>
__device__ __forceinline__ double event_mother(const hps::DevChannel& ch, const hps::DevChannelF& chf, uint64_t evt,
                                               const double (&mo)[4], double (&p)[N][4])
{
    if constexpr (PREC == HPS_PREC_FP64) {
        return hps::f64::event_mother<N, hps::engine_of(ENGINE)>(ch, evt, mo, p);
    } else {
        uint64_t w[3 * N - 4];
        hps::event_words<N, hps::engine_of(ENGINE)>(ch.key, evt, w);
        float q[N][4];
        const hps::f32::EventWeight ew = hps::f32::event_from_words<N, ENGINE>(ch, chf, w, q);
        hps::f32::boost_to_mother<N>(q, chf.m2, hps::f32::mother_frame(mo));
#pragma unroll
        for (int k = 0; k < N; ++k) {
            p[k][0] = hps::f32::widen_pos(q[k][0]);
#pragma unroll
            for (int c = 1; c < 4; ++c) p[k][c] = hps::f32::widen(q[k][c]);
        }
        return ew.weight;
    }
}

// AverageOn in the FP32_FIX form: the tile fold of hps_average_on's FP32_FIX kernels
// (tiles_f32.cuh average_tile_f32) with the user's functor.  The CTA shares the random words of
// each chunk of kThreads events (about one Philox block per event instead of ceil((3N-4)/2)); each
// thread keeps float-float sums of P, P d and P d^2, P = prod(pdk) of the event and d = f - K0, K0
// the functor's value at the call's first event (k_user_shift_f32, read from *k0); the tile's sums,
// scaled by the maximum weight, go to partials as hps_sums, and k_average_final_sums forms
// (K0 + S1/W, S2 - S1^2/W, W).  The functor sees the widened four-vectors, as in k_average_tiles.
// The functor's value at one FP32_FIX event, rounded to float.  With MOTHERS the event is first
// boosted into the frame of its mother mo and the functor sees (mother, daughters...).
template <int N, int ENGINE, bool MOTHERS, typename V, typename F>
__device__ __forceinline__ float user_value_f32(const hps::DevChannelF& chf, const F& f, float (&q)[N][4],
                                                const double* __restrict__ mothers, uint64_t e)
{
    double mo[4] = {0.0, 0.0, 0.0, 0.0};
    if constexpr (MOTHERS) {
        for (int c = 0; c < 4; ++c) mo[c] = mothers[4 * e + c];
        hps::f32::boost_to_mother<N>(q, chf.m2, hps::f32::mother_frame(mo));
    }
    double p[N][4];
#pragma unroll
    for (int k = 0; k < N; ++k) {
        p[k][0] = hps::f32::widen_pos(q[k][0]);
#pragma unroll
        for (int c = 1; c < 4; ++c) p[k][c] = hps::f32::widen(q[k][c]);
    }
    if constexpr (MOTHERS)
        return static_cast<float>(static_cast<double>(f(as_tuple_m<V>(mo, p, std::make_index_sequence<N>{}))));
    else
        return static_cast<float>(static_cast<double>(f(event_tuple<V>(p))));
}

template <int N, int ENGINE, bool MOTHERS, typename V, typename F>
__global__ void __launch_bounds__(kThreads)
k_average_tiles_f32(hps::DevChannel ch, hps::DevChannelF chf, F f, uint64_t first, uint64_t n, uint64_t ntiles,
                    const float* __restrict__ k0, hps_stats* __restrict__ partials,
                    const double* __restrict__ mothers = nullptr)
{
    static_assert(kThreads == hps::kTileThreads, "the word exchange is sized for the tile's CTA");
    __shared__ __align__(16) unsigned char smem[hps::WordShare<N, ENGINE, kThreads>::BYTES2];
    const float K0 = *k0;
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        float swh = 0.0f, swl = 0.0f, s1h = 0.0f, s1l = 0.0f, s2h = 0.0f, s2l = 0.0f;
        const uint64_t base = t * HPS_AVG_TILE;
        for (int k = 0; k < kPerThread; ++k) {
            const uint64_t cb = base + (uint64_t)k * kThreads;
            if (cb >= n) break;                                          // CTA-uniform
            uint64_t w[3 * N - 4];
            hps::cta_event_words<N, ENGINE, kThreads>(ch.key, first + cb, smem, w, k);
            const uint64_t e = cb + threadIdx.x;
            if (e < n) {
                float q[N][4];
                const hps::f32::EventWeight ew = hps::f32::event_from_words<N, ENGINE>(ch, chf, w, q);
                const float d = user_value_f32<N, ENGINE, MOTHERS, V>(chf, f, q, mothers, e) - K0;
                const float h1 = ew.prod_hi * d;
                const float l1 = fmaf(ew.prod_lo, d, fmaf(ew.prod_hi, d, -h1));
                const float h2 = h1 * d;
                const float l2 = fmaf(l1, d, fmaf(h1, d, -h2));
                hps::ff_add(swh, swl, ew.prod_hi, ew.prod_lo);
                hps::ff_add(s1h, s1l, h1, l1);
                hps::ff_add(s2h, s2l, h2, l2);
            }
        }
        hps::hps_sums acc;
        acc.w = ch.max_weight * (hps::f32::widen(swh) + hps::f32::widen(swl));
        acc.s1 = ch.max_weight * (hps::f32::widen(s1h) + hps::f32::widen(s1l));
        acc.s2 = ch.max_weight * (hps::f32::widen(s2h) + hps::f32::widen(s2l));
        const hps::hps_sums r = hps::block_reduce_sums<kThreads>(acc);
        if (threadIdx.x == 0) reinterpret_cast<hps::hps_sums*>(partials)[t] = r;
        __syncthreads();          // the next tile's word exchange reuses the buffers
    }
}

// The FP32_FIX tiles' sums in a fixed order (thread j adds tiles j, j + kFinal, ...; the fixed CTA
// tree adds the threads' sums) and the call's StatsPHSP from them.
template <int = 0>
__global__ void __launch_bounds__(kFinal)
k_average_final_sums(const hps_stats* __restrict__ partials, uint64_t ntiles, const float* __restrict__ k0,
                     hps_stats* __restrict__ out)
{
    const float K0 = *k0;
    const hps::hps_sums* tiles = reinterpret_cast<const hps::hps_sums*>(partials);
    hps::hps_sums acc{0.0, 0.0, 0.0};
    for (uint64_t t = threadIdx.x; t < ntiles; t += kFinal) {
        const hps::hps_sums v = tiles[t];
        acc.s1 += v.s1; acc.s2 += v.s2; acc.w += v.w;
    }
    const hps::hps_sums tot = hps::block_reduce_sums<kFinal>(acc);
    if (threadIdx.x == 0) {
        hps_stats r{0.0, 0.0, 0.0};
        if (tot.w != 0.0) {
            const double q = tot.s1 / tot.w;
            r.w = tot.w;
            r.mean = hps::f32::widen(K0) + q;
            r.m2 = fma(-tot.s1, q, tot.s2);
        }
        *out = r;
    }
}

// The functor's value at one event in the FP32_FIX form (the shift K0 of the call's first event,
// with its mother mothers[0] in the per-event-mother form).
template <int N, int ENGINE, bool MOTHERS, typename V, typename F>
__global__ void k_user_shift_f32(hps::DevChannel ch, hps::DevChannelF chf, F f, uint64_t first, float* __restrict__ k0,
                                 const double* __restrict__ mothers = nullptr)
{
    if (threadIdx.x != 0) return;
    uint64_t w[3 * N - 4];
    hps::event_words<N, hps::engine_of(ENGINE)>(ch.key, first, w);
    float q[N][4];
    hps::f32::event_from_words<N, ENGINE>(ch, chf, w, q);
    *k0 = user_value_f32<N, ENGINE, MOTHERS, V>(chf, f, q, mothers, 0);
}

// AverageOn(mothers, functor) (AverageMothers): event e boosted by mothers[e]; the functor sees
// (mother, daughters...).
template <int N, int ENGINE, int PREC, typename V, typename F>
__global__ void __launch_bounds__(kThreads)
k_average_mothers_tiles(hps::DevChannel ch, hps::DevChannelF chf, F f, const double* __restrict__ mothers,
                        uint64_t first, uint64_t n, uint64_t ntiles, hps_stats* __restrict__ partials)
{
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        hps_stats acc{0.0, 0.0, 0.0};
        const uint64_t base = t * HPS_AVG_TILE + threadIdx.x;
        for (int k = 0; k < kPerThread; ++k) {
            const uint64_t e = base + (uint64_t)k * kThreads;
            if (e < n) {
                double mo[4];
                for (int c = 0; c < 4; ++c) mo[c] = mothers[4 * e + c];
                double p[N][4];
                hps_stats y;
                y.w = event_mother<N, ENGINE, PREC>(ch, chf, first + e, mo, p);
                y.mean = static_cast<double>(f(as_tuple_m<V>(mo, p, std::make_index_sequence<N>{})));
                y.m2 = 0.0;
                acc = hps::stats_merge(acc, y);
            }
        }
        const hps_stats r = hps::block_reduce_stats<kThreads>(acc);
        if (threadIdx.x == 0) partials[t] = r;
    }
}

// Thread j folds partials j, j + 1024, ... in order, then the fixed CTA tree.
template <int = 0>
__global__ void __launch_bounds__(kFinal)
k_average_final(const hps_stats* __restrict__ partials, uint64_t ntiles, hps_stats* __restrict__ out)
{
    hps_stats acc{0.0, 0.0, 0.0};
    for (uint64_t t = threadIdx.x; t < ntiles; t += kFinal) acc = hps::stats_merge(acc, partials[t]);
    const hps_stats r = hps::block_reduce_stats<kFinal>(acc);
    if (threadIdx.x == 0) *out = r;
}

// Evaluate (EvalMother): column 0 the generation-time weight, column k + 1 functor k.
template <int K> struct OutColumns { double* p[K + 1]; };

template <size_t I, typename V, size_t N, typename Fs>
__device__ __forceinline__ void eval_each(const Fs& fs, const double (&p)[N][4], double* const* out, uint64_t e)
{
    if constexpr (I < std::tuple_size<Fs>::value) {
        out[I + 1][e] = static_cast<double>(std::get<I>(fs)(event_tuple<V>(p)));
        eval_each<I + 1, V>(fs, p, out, e);
    }
}

template <int N, int ENGINE, int PREC, typename V, typename Fs, int K>
__global__ void __launch_bounds__(kThreads)
k_evaluate(hps::DevChannel ch, hps::DevChannelF chf, Fs fs, OutColumns<K> out, uint64_t first, uint64_t n)
{
    if constexpr (PREC == HPS_PREC_FP64) {
        for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
             e += (uint64_t)gridDim.x * blockDim.x) {
            double p[N][4];
            const double w = event<N, ENGINE, PREC>(ch, chf, first + e, p);
            out.p[0][e] = w;
            eval_each<0, V>(fs, p, out.p, e);
        }
    } else {
        // chunks of kThreads consecutive events whose random words the CTA shares (about one Philox
        // block per event instead of ceil((3N - 4) / 2))
        static_assert(kThreads == hps::kTileThreads, "the word exchange is sized for the tile's CTA");
        __shared__ __align__(16) unsigned char smem[hps::WordShare<N, ENGINE, kThreads>::BYTES2];
        const uint64_t step = (uint64_t)gridDim.x * kThreads;
        int parity = 0;
        for (uint64_t cb = (uint64_t)blockIdx.x * kThreads; cb < n; cb += step, parity ^= 1) {
            uint64_t w[3 * N - 4];
            hps::cta_event_words<N, ENGINE, kThreads>(ch.key, first + cb, smem, w, parity);
            const uint64_t e = cb + threadIdx.x;
            if (e < n) {
                float q[N][4];
                const hps::f32::EventWeight ew = hps::f32::event_from_words<N, ENGINE>(ch, chf, w, q);
                double p[N][4];
#pragma unroll
                for (int k = 0; k < N; ++k) {
                    p[k][0] = hps::f32::widen_pos(q[k][0]);
#pragma unroll
                    for (int c = 1; c < 4; ++c) p[k][c] = hps::f32::widen(q[k][c]);
                }
                out.p[0][e] = ew.weight;
                eval_each<0, V>(fs, p, out.p, e);
            }
        }
    }
}

// Evaluate(mothers, result, functors...) (EvalMothers.h:143-305): the stream hash((int)evt, seed)
// per event, ECM and maximum weight from the event's own mother, the daughters boosted into its
// frame; column 0 the weight, column k + 1 functor k on (mother, daughters...).
template <size_t I, typename V, size_t N, typename Fs>
__device__ __forceinline__ void eval_each_m(const Fs& fs, const double (&mo)[4], const double (&p)[N][4],
                                            double* const* out, uint64_t e)
{
    if constexpr (I < std::tuple_size<Fs>::value) {
        out[I + 1][e] = static_cast<double>(std::get<I>(fs)(as_tuple_m<V>(mo, p, std::make_index_sequence<N>{})));
        eval_each_m<I + 1, V>(fs, mo, p, out, e);
    }
}

template <int N, int ENGINE, int PREC, typename V, typename Fs, int K>
__global__ void __launch_bounds__(kThreads)
k_evaluate_mothers(hps::DevChannel ch, hps::DevChannelF chf, uint64_t seed, const double* __restrict__ mothers,
                   Fs fs, OutColumns<K> out, uint64_t first, uint64_t n)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
        double mo[4];
        for (int c = 0; c < 4; ++c) mo[c] = mothers[4 * e + c];
        double p[N][4];
        double w;
        if constexpr (PREC == HPS_PREC_FP64) {
            w = hps::f64::event_evalmothers<N, hps::engine_of(ENGINE)>(ch, first + e, seed, mo, p);
        } else {
            float q[N][4];
            hps::f32::MotherFrame mf;
            w = hps::f32::event_evalmothers<N, ENGINE>(ch, chf, first + e, seed, mo, q, mf).weight;
#pragma unroll
            for (int k = 0; k < N; ++k) {
                p[k][0] = hps::f32::widen_pos(q[k][0]);
#pragma unroll
                for (int c = 1; c < 4; ++c) p[k][c] = hps::f32::widen(q[k][c]);
            }
        }
        out.p[0][e] = w;
        eval_each_m<0, V>(fs, mo, p, out.p, e);
    }
}

// PhaseSpaceReweight (Decays.inl:372-386) on stored events: PhaseSpaceWeight recomputed from the
// four-vectors (Decays.inl:215-231) times the functor; each CTA's largest value into block_max.
template <int N> struct InColumns { const double* p[N]; };

template <int N, typename V, typename Tup, typename F>
__global__ void __launch_bounds__(kThreads)
k_reweight(InColumns<N> cols, hps::DevChannel ch, F f, uint64_t n, double* __restrict__ out,
           double* __restrict__ block_max)
{
    __shared__ double smax[kThreads];
    double m = -1.0 / 0.0;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
        double p[N][4];
#pragma unroll
        for (int k = 0; k < N; ++k)
#pragma unroll
            for (int c = 0; c < 4; ++c) p[k][c] = cols.p[k][4 * e + c];
        const double w = hps::f64::recomputed_weight<N>(ch.masses, ch.max_weight, p) *
                         static_cast<double>(f(as_typed_tuple<Tup, V>(p, std::make_index_sequence<N>{})));
        out[e] = w;
        m = w > m ? w : m;
    }
    smax[threadIdx.x] = m;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s && smax[threadIdx.x + s] > smax[threadIdx.x]) smax[threadIdx.x] = smax[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) block_max[blockIdx.x] = smax[0];
}

template <int = 0>
__global__ void __launch_bounds__(kFinal)
k_max_final(const double* __restrict__ block_max, unsigned nblocks, double* __restrict__ out)
{
    __shared__ double smax[kFinal];
    double m = -1.0 / 0.0;
    for (unsigned b = threadIdx.x; b < nblocks; b += kFinal) m = block_max[b] > m ? block_max[b] : m;
    smax[threadIdx.x] = m;
    __syncthreads();
    for (int s = kFinal / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s && smax[threadIdx.x + s] > smax[threadIdx.x]) smax[threadIdx.x] = smax[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = smax[0];
}

inline unsigned grid_for(uint64_t items, unsigned threads, unsigned cap = 152u * 32u)
{
    const uint64_t need = (items + threads - 1) / threads;
    return static_cast<unsigned>(need == 0 ? 1 : (need < cap ? need : cap));
}

// Host: the kernel-side channel constants of a launch.
struct LaunchChannel {
    hps::DevChannel ch;
    hps::DevChannelF chf;
    int engine;
};

inline LaunchChannel launch_channel(const hps_channel& c)
{
    LaunchChannel lc;
    hps::make_channel(c, lc.ch);
    hps::f32::make_channel_f(c, lc.chf);
    lc.engine = c.engine == HPS_ENGINE_PHILOX ? hps::kPhilox : hps::kSquares3;
    return lc;
}

// Calls body(std::integral_constant<int, ENGINE>) with the channel's engine, plus
// hps::kPreciseForm where the FP32_FIX form of this N takes the float-float boosts for it.
template <int N, typename Body>
inline void with_engine(const LaunchChannel& lc, int precision, Body&& body)
{
    const bool ff = precision == HPS_PREC_FP32_FIX && N >= hps::f32::kHardMinN && N < hps::f32::kPreciseN &&
                    lc.chf.precise != 0;
    if (lc.engine == hps::kPhilox) {
        if (ff) body(std::integral_constant<int, hps::kPhilox | hps::kPreciseForm>{});
        else body(std::integral_constant<int, hps::kPhilox>{});
    } else {
        if (ff) body(std::integral_constant<int, hps::kSquares3 | hps::kPreciseForm>{});
        else body(std::integral_constant<int, hps::kSquares3>{});
    }
}

}  // namespace user
}  // namespace detail
}  // namespace hydra

#endif  // HYDRA_HPS_USER_KERNELS_CUH_
