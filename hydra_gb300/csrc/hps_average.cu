// hps_average.cu -- storage-free AverageOn.
//
// Replaces hydra::detail::launch_reducer -> thrust::transform_reduce(counting, AverageMother,
// StatsPHSP(), AddStatsPHSP()) (hydra/detail/launch_decayers.inl:94-106, PhaseSpace.inl:255-273).
// Each event is generated and weighted in registers, mapped to StatsPHSP{f, w, 0}
// (AverageMother.h:272-292) and merged with AddStatsPHSP.  The merge tree is fixed by the
// event count alone:
//   tile t = events [t*4096, (t+1)*4096); thread j of the 256-thread CTA folds events
//   t*4096 + j + 256*k, k = 0..15, in order; a fixed warp/CTA tree merges the 256 folds;
//   the tile partials are merged by one CTA in a fixed tree.
// Which CTA runs which tile does not matter, so the result is bit-identical for every grid.
#include "common.h"
#include "store.cuh"
#include "tiles_f32.cuh"

namespace hps {

constexpr int kAvgThreads = kTileThreads;

// The AverageOn tiles exchange the random words of two chunks at a time for N = 3..5 (the same
// sums bit for bit, half the barriers): at 2^24 events N = 3 0.306 ms against 0.309, N = 5 0.575
// against 0.577, and the one-pass Generate + AverageOn at N = 5 0.694 against 0.705; at N = 2
// 0.191 against 0.188, N = 6 0.760 against 0.735, N = 10 2.127 against 2.080.
__host__ __device__ constexpr bool avg_paired(int N) { return N >= 3 && N <= 5; }

// Resident CTAs per SM the register allocation of the FP32_FIX tile kernels must allow (second
// argument of __launch_bounds__; 0 leaves the choice to the compiler).  AverageOn at 2^24 events,
// ms for N = 3, 5, 9, 10 (registers in brackets):
//   compiler  0.270 0.484 1.940 2.309  (48, 60, 128, 128)
//   1 CTA     0.280 0.524 2.251 2.599  (72..252)
//   2 CTAs    0.280 0.524 1.958 2.372  (<= 128)
//   3 CTAs    0.276 0.507 1.996 2.404  (<= 80)
// (With the functor's parameters converted to float on the device for each event, N = 10 had
// taken 2.278 ms with 2 CTAs against 2.335 with the compiler's choice.)
// With the current body, N = 2..6 (ms): compiler 0.180 0.271 0.368 0.488 0.788; 5 CTAs (48
// registers) 0.186 0.288 0.379 0.492 0.822; 6 CTAs (40 registers, spilling at N = 5, 6) 0.191 0.286
// 0.382 0.514 0.843.
__host__ __device__ constexpr int avg_min_ctas(int) { return 0; }

template <int N, int ENGINE>
__global__ void __launch_bounds__(kAvgThreads)
k_average_tiles_f64(DevChannel ch, DevFunctor fn, uint64_t first, uint64_t n, uint64_t ntiles,
                    hps_stats* __restrict__ partials)
{
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        hps_stats acc{0.0, 0.0, 0.0};
        const uint64_t base = t * HPS_AVG_TILE + threadIdx.x;
        for (int k = 0; k < kAvgPerThread; ++k) {
            const uint64_t e = base + (uint64_t)k * kAvgThreads;
            if (e < n) {
                double p[N][4];
                hps_stats y;
                y.w = f64::event<N, ENGINE>(ch, first + e, p);
                y.mean = functor_f64<N>(fn, p);
                y.m2 = 0.0;
                acc = stats_merge(acc, y);
            }
        }
        const hps_stats r = block_reduce_stats<kAvgThreads>(acc);
        if (threadIdx.x == 0) partials[t] = r;
    }
}

// Generate + AverageOn of the same events in one pass, FP64 form: the tile fold above with every
// event also stored as k_generate_f64 stores it (four-vectors, weight, FlagDaugthers flag).
template <int N, int ENGINE>
__global__ void __launch_bounds__(kAvgThreads)
k_generate_average_f64(DevChannel ch, DevFunctor fn, uint64_t first, uint64_t n, uint64_t ntiles,
                       hps_stats* __restrict__ partials, StoreOut so)
{
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        hps_stats acc{0.0, 0.0, 0.0};
        const uint64_t base = t * HPS_AVG_TILE + threadIdx.x;
        for (int k = 0; k < kAvgPerThread; ++k) {
            const uint64_t e = base + (uint64_t)k * kAvgThreads;
            if (e < n) {
                double p[N][4];
                hps_stats y;
                y.w = f64::event<N, ENGINE>(ch, first + e, p);
#pragma unroll
                for (int d = 0; d < N; ++d) store_vec4(so.cols.p[d], e, p[d], so.vec32 != 0);
                if (so.weights) so.weights[e] = y.w;
                if (so.flags) {
                    const double wr = f64::recomputed_weight<N>(ch.masses, ch.max_weight, p);
                    const double u = static_cast<double>(squares3_word(so.ukey, first + e)) * 0x1p-32;
                    so.flags[e] = (f64::dvd(wr, ch.max_weight) > u) ? 1 : 0;
                }
                y.mean = functor_f64<N>(fn, p);
                y.m2 = 0.0;
                acc = stats_merge(acc, y);
            }
        }
        const hps_stats r = block_reduce_stats<kAvgThreads>(acc);
        if (threadIdx.x == 0) partials[t] = r;
    }
}

// FP32_FIX form: average_tile_f32 (tiles_f32.cuh) per tile, CTA-shared random words.
template <int N, int ENGINE>
__global__ void __launch_bounds__(kAvgThreads, avg_min_ctas(N))
k_average_tiles_f32fix(DevChannel chd, DevChannelF ch, DevFunctor fn, uint64_t first, uint64_t n,
                       uint64_t ntiles, hps_stats* __restrict__ partials, const float* __restrict__ k0)
{
    __shared__ __align__(16) unsigned char smem[PairedSmem<N, ENGINE>::BYTES];
    const float K0 = *k0;
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const hps_sums r =
            average_tile_f32<N, ENGINE, false, false, avg_paired(N)>(chd, ch, fn, first, n, t, K0, smem);
        if (threadIdx.x == 0) reinterpret_cast<hps_sums*>(partials)[t] = r;
    }
}

template <int N, int ENGINE>
__global__ void __launch_bounds__(kAvgThreads, avg_min_ctas(N))
k_generate_average_f32fix(DevChannel chd, DevChannelF ch, DevFunctor fn, uint64_t first, uint64_t n,
                          uint64_t ntiles, hps_stats* __restrict__ partials, const float* __restrict__ k0,
                          StoreOut so)
{
    __shared__ __align__(16) unsigned char smem[PairedSmem<N, ENGINE>::BYTES];
    const float K0 = *k0;
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const hps_sums r =
            average_tile_f32<N, ENGINE, true, false, avg_paired(N)>(chd, ch, fn, first, n, t, K0, smem, &so);
        if (threadIdx.x == 0) reinterpret_cast<hps_sums*>(partials)[t] = r;
    }
}

// K0 of the call into the first 4 bytes of *out (read by the tile and final kernels).
template <int N, int ENGINE>
__global__ void k_shift_f32(DevChannel chd, DevChannelF ch, DevFunctor fn, uint64_t first, float* __restrict__ k0)
{
    if (threadIdx.x == 0) *k0 = call_shift<N, ENGINE>(chd, ch, fn, first);
}

template <int N, int ENGINE>
__global__ void __launch_bounds__(kFinalThreads)
k_average_final_f32fix(DevChannel chd, DevChannelF ch, DevFunctor fn, uint64_t first,
                       const hps_stats* __restrict__ partials, uint64_t ntiles, hps_stats* __restrict__ out)
{
    // every thread reads K0 from *out before the block reduction's barriers; thread 0 writes *out after them
    const float K0 = ntiles ? *reinterpret_cast<const float*>(out) : 0.0f;
    const hps_stats r = merge_sums<N, ENGINE>(chd, ch, fn, first, partials, ntiles, K0);
    if (threadIdx.x == 0) *out = r;
}

// One CTA: thread j folds partials j, j+1024, ... in order, then the fixed CTA tree.
__global__ void __launch_bounds__(kFinalThreads)
k_average_final(const hps_stats* __restrict__ partials, uint64_t ntiles, hps_stats* __restrict__ out)
{
    const hps_stats r = merge_partials(partials, ntiles);
    if (threadIdx.x == 0) *out = r;
}

// Host-side validation shared by every AverageOn entry point; touches no device state.
hps_status average_args(const hps_channel* channel, const hps_functor* functor, int32_t precision,
                        DevChannel* ch, DevFunctor* fn)
{
    hps_status st = to_device_channel(channel, ch);
    if (st != HPS_OK) return st;
    st = to_device_functor(functor, channel->n_daughters, fn);
    if (st != HPS_OK) return st;
    if (precision != HPS_PREC_FP64 && precision != HPS_PREC_FP32_FIX)
        return set_error(HPS_ERR_BAD_ARG, "unknown precision %d", precision);
    return HPS_OK;
}

hps_status launch_average(const hps_channel* channel, const DevChannel& ch, const DevFunctor& fn,
                          uint64_t first_evt, uint64_t n, hps_stats* out, hps_stats* partials,
                          int32_t precision, cudaStream_t stream, const StoreOut* so)
{
    const uint64_t ntiles = (n + HPS_AVG_TILE - 1) / HPS_AVG_TILE;
    if (ntiles > 0) {
        const unsigned grid = static_cast<unsigned>(ntiles < 152u * 16u ? ntiles : 152u * 16u);
        if (precision == HPS_PREC_FP32_FIX) {
            DevChannelF chf;
            to_device_channel_f(channel, &chf);
            float* k0 = reinterpret_cast<float*>(out);
#define HPS_BODY(NN, EE)                                                                          \
            k_shift_f32<NN, EE><<<1, 32, 0, stream>>>(ch, chf, fn, first_evt, k0);                  \
            if (so)                                                                                \
                k_generate_average_f32fix<NN, EE><<<grid, kAvgThreads, 0, stream>>>(               \
                    ch, chf, fn, first_evt, n, ntiles, partials, k0, *so);                         \
            else                                                                                   \
                k_average_tiles_f32fix<NN, EE><<<grid, kAvgThreads, 0, stream>>>(ch, chf, fn, first_evt, n, \
                                                                                  ntiles, partials, k0);
            HPS_DISPATCH_F32(channel->n_daughters, channel->engine, chf.precise, HPS_BODY)
#undef HPS_BODY
        } else {
#define HPS_BODY(NN, EE)                                                                          \
            if (so)                                                                                \
                k_generate_average_f64<NN, EE><<<grid, kAvgThreads, 0, stream>>>(ch, fn, first_evt, n, \
                                                                                  ntiles, partials, *so); \
            else                                                                                   \
                k_average_tiles_f64<NN, EE><<<grid, kAvgThreads, 0, stream>>>(ch, fn, first_evt, n, ntiles, \
                                                                               partials);
            HPS_DISPATCH_N_ENGINE(channel->n_daughters, channel->engine, HPS_BODY)
#undef HPS_BODY
        }
    }
    if (precision == HPS_PREC_FP32_FIX) {
        DevChannelF chf;
        to_device_channel_f(channel, &chf);
#define HPS_BODY(NN, EE)                                                                                   \
        k_average_final_f32fix<NN, EE><<<1, kFinalThreads, 0, stream>>>(ch, chf, fn, first_evt, partials, ntiles, out);
        HPS_DISPATCH_F32(channel->n_daughters, channel->engine, chf.precise, HPS_BODY)
#undef HPS_BODY
    } else {
        k_average_final<<<1, kFinalThreads, 0, stream>>>(partials, ntiles, out);
    }
    return cuda_status(cudaGetLastError(), "hps_average_on launch");
}

}  // namespace hps

using namespace hps;

extern "C" {

size_t hps_average_on_workspace_size(uint64_t n)
{
    const uint64_t ntiles = (n + HPS_AVG_TILE - 1) / HPS_AVG_TILE;
    return static_cast<size_t>((ntiles == 0 ? 1 : ntiles) * sizeof(hps_stats));
}

hps_status hps_average_on(const hps_channel* channel, uint64_t first_evt, uint64_t n, const hps_functor* functor,
                          hps_stats* out, void* workspace, size_t workspace_bytes, int32_t precision, void* stream)
{
    HPS_ENTRY();
    DevChannel ch;
    DevFunctor fn;
    hps_status st = average_args(channel, functor, precision, &ch, &fn);
    if (st != HPS_OK) return st;
    if (!out) return set_error(HPS_ERR_BAD_ARG, "out is NULL");
    if (!range_ok(first_evt, n)) return set_error(HPS_ERR_BAD_ARG, "event range wraps 2^64");
    if (!aligned(out, 8)) return set_error(HPS_ERR_BAD_ARG, "out not 8-byte aligned");
    const size_t need = hps_average_on_workspace_size(n);
    cudaStream_t s = as_stream(stream);
    if (workspace) {
        if (workspace_bytes < need)
            return set_error(HPS_ERR_BAD_ARG, "workspace of %zu bytes, %zu needed", workspace_bytes, need);
        if (!aligned(workspace, 8)) return set_error(HPS_ERR_BAD_ARG, "workspace not 8-byte aligned");
        return launch_average(channel, ch, fn, first_evt, n, out, static_cast<hps_stats*>(workspace), precision, s);
    }
    void* scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&scratch, need, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(HPS_ERR_OOM, "cudaMallocAsync(%zu): %s", need, cudaGetErrorString(e));
    }
    st = launch_average(channel, ch, fn, first_evt, n, out, static_cast<hps_stats*>(scratch), precision, s);
    e = cudaFreeAsync(scratch, s);
    if (st == HPS_OK && e != cudaSuccess) return cuda_status(e, "cudaFreeAsync");
    return st;
}

hps_status hps_generate_average(const hps_channel* channel, uint64_t first_evt, uint64_t n, double* const* cols,
                                double* weights, uint8_t* flags, uint64_t unweight_seed, const hps_functor* functor,
                                hps_stats* out, void* workspace, size_t workspace_bytes, int32_t precision,
                                void* stream)
{
    HPS_ENTRY();
    DevChannel ch;
    DevFunctor fn;
    hps_status st = average_args(channel, functor, precision, &ch, &fn);
    if (st != HPS_OK) return st;
    if (!out || !aligned(out, 8)) return set_error(HPS_ERR_BAD_ARG, "out NULL or not 8-byte aligned");
    if (!range_ok(first_evt, n)) return set_error(HPS_ERR_BAD_ARG, "event range wraps 2^64");
    StoreOut so{};
    const int N = channel->n_daughters;
    if (n) {
        if (!cols) return set_error(HPS_ERR_BAD_ARG, "cols is NULL");
        bool all32 = true;
        for (int k = 0; k < N; ++k) {
            if (!cols[k]) return set_error(HPS_ERR_BAD_ARG, "column %d is NULL", k);
            if (!aligned(cols[k], 16)) return set_error(HPS_ERR_BAD_ARG, "column %d not 16-byte aligned", k);
            all32 = all32 && aligned(cols[k], 32);
            so.cols.p[k] = cols[k];
        }
        so.vec32 = all32 ? 1 : 0;
    }
    if (weights && !aligned(weights, 8)) return set_error(HPS_ERR_BAD_ARG, "weights not 8-byte aligned");
    so.weights = weights;
    so.flags = flags;
    so.ukey = splitmix64(unweight_seed);
    const size_t need = hps_average_on_workspace_size(n);
    cudaStream_t s = as_stream(stream);
    if (workspace) {
        if (workspace_bytes < need)
            return set_error(HPS_ERR_BAD_ARG, "workspace of %zu bytes, %zu needed", workspace_bytes, need);
        if (!aligned(workspace, 8)) return set_error(HPS_ERR_BAD_ARG, "workspace not 8-byte aligned");
        return launch_average(channel, ch, fn, first_evt, n, out, static_cast<hps_stats*>(workspace), precision, s,
                              &so);
    }
    void* scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&scratch, need, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(HPS_ERR_OOM, "cudaMallocAsync(%zu): %s", need, cudaGetErrorString(e));
    }
    st = launch_average(channel, ch, fn, first_evt, n, out, static_cast<hps_stats*>(scratch), precision, s, &so);
    e = cudaFreeAsync(scratch, s);
    if (st == HPS_OK && e != cudaSuccess) return cuda_status(e, "cudaFreeAsync");
    return st;
}

}  // extern "C"
