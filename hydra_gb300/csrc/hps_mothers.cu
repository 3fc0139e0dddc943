// hps_mothers.cu -- the per-event-mother forms of Generate, AverageOn and Evaluate (FP64 and FP32_FIX).
//
// PhaseSpace::Generate(mothers, daughters), AverageOn(begin, end, functor) and
// Evaluate(mothers, result, functors) (hydra/detail/PhaseSpace.inl:276-309, 331-444) use the
// functors DecayMothers, AverageMothers and EvalMothers (hydra/detail/functors/*Mothers.h):
// each event is boosted by its own mother four-vector, read from a column of Vector4R (for
// instance a daughter column of an earlier Decays, as in a decay chain).  AverageMothers and
// EvalMothers hand the functor (mother, daughter 0, ..., daughter N-1), so functor indices here
// count the mother as particle 0.  EvalMothers draws a different stream per event (engine seeded
// with hash(evt, seed), no discard) and takes ECM and the maximum weight from the mother's mass.
#include "common.h"
#include "store.cuh"
#include "tiles_f32.cuh"

namespace hps {

struct MCols { double* p[HPS_MAX_DAUGHTERS]; };
constexpr int kMaxMotherFunctors = 8;
struct MFunctors { DevFunctor f[kMaxMotherFunctors]; };
struct MOut { double* p[kMaxMotherFunctors]; };

// (mother, daughters...) as the *Mothers functors see them.
template <int N>
__device__ __forceinline__ double functor_with_mother(const DevFunctor& fn, const double (&mo)[4],
                                                      const double (&p)[N][4])
{
    double pm[N + 1][4];
#pragma unroll
    for (int c = 0; c < 4; ++c) pm[0][c] = mo[c];
#pragma unroll
    for (int k = 0; k < N; ++k)
#pragma unroll
        for (int c = 0; c < 4; ++c) pm[k + 1][c] = p[k][c];
    return functor_f64<N + 1>(fn, pm);
}

template <int N, int ENGINE>
__global__ void __launch_bounds__(256)
k_generate_mothers_f64(DevChannel ch, const double* __restrict__ mothers, MCols cols, double* __restrict__ weights,
                       uint64_t first, uint64_t n, int vec32)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
         e += (uint64_t)gridDim.x * blockDim.x) {
        double mo[4];
        load_mother<N>(mothers, e, mo);
        double p[N][4];
        const double wt = f64::event_mother<N, ENGINE>(ch, first + e, mo, p);
#pragma unroll
        for (int k = 0; k < N; ++k) store_vec4(cols.p[k], e, p[k], vec32 != 0);
        if (weights) weights[e] = wt;
    }
}

template <int N, int ENGINE>
__global__ void __launch_bounds__(256)
k_evaluate_mothers_f64(DevChannel ch, uint64_t seed, const double* __restrict__ mothers, MFunctors fs, int nf,
                       double* __restrict__ weights, MOut out, uint64_t first, uint64_t n)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
         e += (uint64_t)gridDim.x * blockDim.x) {
        double mo[4];
        load_mother<N>(mothers, e, mo);
        double p[N][4];
        const double wt = f64::event_evalmothers<N, ENGINE>(ch, first + e, seed, mo, p);
        if (weights) weights[e] = wt;
        for (int k = 0; k < nf; ++k) out.p[k][e] = functor_with_mother<N>(fs.f[k], mo, p);
    }
}

// FP32_FIX EvalMothers (f32::event_evalmothers per event).
template <int N, int ENGINE>
__global__ void __launch_bounds__(256)
k_evaluate_mothers_f32fix(DevChannel ch, DevChannelF chf, uint64_t seed, const double* __restrict__ mothers,
                          MFunctors fs, int nf, double* __restrict__ weights, MOut out, uint64_t first, uint64_t n)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
         e += (uint64_t)gridDim.x * blockDim.x) {
        double mo[4];
        load_mother<N>(mothers, e, mo);
        float p[N][4];
        f32::MotherFrame mf;
        const f32::EventWeight ew = f32::event_evalmothers<N, ENGINE>(ch, chf, first + e, seed, mo, p, mf);
        if (weights) weights[e] = ew.weight;
        for (int k = 0; k < nf; ++k) out.p[k][e] = f32::widen(mother_functor_f32<N>(fs.f[k], mf, p));
    }
}

// AverageMothers: the tile / fold / tree structure of k_average_tiles_f64.
constexpr int kMThreads = 256;
constexpr int kMPerThread = HPS_AVG_TILE / kMThreads;

template <int N, int ENGINE>
__global__ void __launch_bounds__(kMThreads)
k_average_mothers_tiles_f64(DevChannel ch, const double* __restrict__ mothers, DevFunctor fn, uint64_t first,
                            uint64_t n, uint64_t ntiles, hps_stats* __restrict__ partials)
{
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        hps_stats acc{0.0, 0.0, 0.0};
        const uint64_t base = t * HPS_AVG_TILE + threadIdx.x;
        for (int k = 0; k < kMPerThread; ++k) {
            const uint64_t e = base + (uint64_t)k * kMThreads;
            if (e < n) {
                double mo[4];
                load_mother<N>(mothers, e, mo);
                double p[N][4];
                hps_stats y;
                y.w = f64::event_mother<N, ENGINE>(ch, first + e, mo, p);
                y.mean = functor_with_mother<N>(fn, mo, p);
                y.m2 = 0.0;
                acc = stats_merge(acc, y);
            }
        }
        const hps_stats r = block_reduce_stats<kMThreads>(acc);
        if (threadIdx.x == 0) partials[t] = r;
    }
}

__global__ void __launch_bounds__(1024)
k_average_mothers_final(const hps_stats* __restrict__ partials, uint64_t ntiles, hps_stats* __restrict__ out)
{
    hps_stats acc{0.0, 0.0, 0.0};
    for (uint64_t t = threadIdx.x; t < ntiles; t += 1024) acc = stats_merge(acc, partials[t]);
    const hps_stats r = block_reduce_stats<1024>(acc);
    if (threadIdx.x == 0) *out = r;
}

// FP32_FIX DecayMothers: the store path of k_generate_f32fix (CTA-shared words: the stream is the
// DecayMother one) with each event boosted by its own mother (f32::boost_to_mother).
template <int N, int ENGINE>
__global__ void __launch_bounds__(kTileThreads)
k_generate_mothers_f32fix(DevChannel chd, DevChannelF ch, const double* __restrict__ mothers, Cols cols,
                          double* __restrict__ weights, uint64_t first, uint64_t n, int vec32)
{
    __shared__ __align__(16) unsigned char smem[WordShare<N, ENGINE, kTileThreads>::BYTES2];
    const uint64_t step = (uint64_t)gridDim.x * kTileThreads;
    int parity = 0;
    for (uint64_t cb = (uint64_t)blockIdx.x * kTileThreads; cb < n; cb += step, parity ^= 1) {
        uint64_t w[3 * N - 4];
        cta_event_words<N, ENGINE, kTileThreads>(chd.key, first + cb, smem, w, parity);
        const uint64_t e = cb + threadIdx.x;
        if (e < n) {
            double mo[4];
            load_mother<N>(mothers, e, mo);
            float p[N][4];
            const f32::EventWeight ew = f32::event_from_words<N, ENGINE>(chd, ch, w, p);
            f32::boost_to_mother<N>(p, ch.m2, f32::mother_frame(mo));
            store_event_f32<N>(p, ew, cols, weights, nullptr, 0, first, e, vec32 != 0);
        }
    }
}

// FP32_FIX AverageMothers: the tiles of k_average_tiles_f32fix with mothers; K0 from event `first`.
template <int N, int ENGINE>
__global__ void k_shift_mothers_f32(DevChannel chd, DevChannelF ch, DevFunctor fn, uint64_t first,
                                    const double* __restrict__ mothers, float* __restrict__ k0)
{
    if (threadIdx.x != 0) return;
    uint64_t w[3 * N - 4];
    event_words<N, ENGINE>(chd.key, first, w);
    float p[N][4];
    f32::event_from_words<N, ENGINE>(chd, ch, w, p);
    double mo[4];
    load_mother<N>(mothers, 0, mo);
    const f32::MotherFrame mf = f32::mother_frame(mo);
    f32::boost_to_mother<N>(p, ch.m2, mf);
    *k0 = mother_functor_f32<N>(fn, mf, p);
}

template <int N, int ENGINE>
__global__ void __launch_bounds__(kTileThreads)
k_average_mothers_tiles_f32fix(DevChannel chd, DevChannelF ch, DevFunctor fn, uint64_t first, uint64_t n,
                               uint64_t ntiles, hps_stats* __restrict__ partials, const float* __restrict__ k0,
                               const double* __restrict__ mothers)
{
    __shared__ __align__(16) unsigned char smem[WordShare<N, ENGINE, kTileThreads>::BYTES2];
    const float K0 = *k0;
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const hps_sums r = average_tile_f32<N, ENGINE, false, true>(chd, ch, fn, first, n, t, K0, smem, nullptr,
                                                                   mothers);
        if (threadIdx.x == 0) reinterpret_cast<hps_sums*>(partials)[t] = r;
    }
}

template <int N, int ENGINE>
__global__ void __launch_bounds__(kFinalThreads)
k_average_mothers_final_f32fix(DevChannel chd, DevChannelF ch, DevFunctor fn, uint64_t first,
                               const hps_stats* __restrict__ partials, uint64_t ntiles, hps_stats* __restrict__ out)
{
    // every thread reads K0 from *out before the block reduction's barriers; thread 0 writes *out after them
    const float K0 = ntiles ? *reinterpret_cast<const float*>(out) : 0.0f;
    const hps_stats r = merge_sums<N, ENGINE>(chd, ch, fn, first, partials, ntiles, K0);
    if (threadIdx.x == 0) *out = r;
}

static hps_status mother_args(const hps_channel* channel, uint64_t first, uint64_t n, const double* mothers,
                              int32_t precision, DevChannel* ch, bool fp32_ok)
{
    hps_status st = to_device_channel(channel, ch);
    if (st != HPS_OK) return st;
    ch->boost_active = 0;              // the mothers' own boosts replace the channel's
    if (precision != HPS_PREC_FP64 && !(fp32_ok && precision == HPS_PREC_FP32_FIX)) {
        if (precision == HPS_PREC_FP32_FIX)
            return set_error(HPS_ERR_UNSUPPORTED, "EvalMothers is built for HPS_PREC_FP64 only");
        return set_error(HPS_ERR_BAD_ARG, "unknown precision %d", precision);
    }
    if (!range_ok(first, n)) return set_error(HPS_ERR_BAD_ARG, "event range wraps 2^64");
    if (n && !mothers) return set_error(HPS_ERR_BAD_ARG, "mothers is NULL");
    if (!aligned(mothers, 16)) return set_error(HPS_ERR_BAD_ARG, "mothers not 16-byte aligned");
    return HPS_OK;
}

// Functor indices run over (mother, daughters): 0..N.
static hps_status mother_functor(const hps_functor* f, int n_daughters, DevFunctor* out)
{
    return to_device_functor(f, n_daughters + 1, out);
}

}  // namespace hps

using namespace hps;

extern "C" {

hps_status hps_generate_mothers(const hps_channel* channel, uint64_t first_evt, uint64_t n, const double* mothers,
                                double* const* cols, double* weights, int32_t precision, void* stream)
{
    HPS_ENTRY();
    DevChannel ch;
    hps_status st = mother_args(channel, first_evt, n, mothers, precision, &ch, true);
    if (st != HPS_OK || n == 0) return st;
    if (!cols) return set_error(HPS_ERR_BAD_ARG, "cols is NULL");
    const int N = channel->n_daughters;
    MCols cc{};
    bool all32 = true;
    for (int k = 0; k < N; ++k) {
        if (!cols[k] || !aligned(cols[k], 16)) return set_error(HPS_ERR_BAD_ARG, "column %d NULL or misaligned", k);
        all32 = all32 && aligned(cols[k], 32);
        cc.p[k] = cols[k];
    }
    const unsigned grid = grid_for(n, 256);
    if (precision == HPS_PREC_FP32_FIX) {
        DevChannelF chf;
        to_device_channel_f(channel, &chf);
        Cols c32{};
        for (int k = 0; k < N; ++k) c32.p[k] = cc.p[k];
#define HPS_BODY(NN, EE)                                                                                 \
        k_generate_mothers_f32fix<NN, EE><<<grid, kTileThreads, 0, as_stream(stream)>>>(ch, chf, mothers, c32, \
                                                                                     weights, first_evt, n, all32 ? 1 : 0);
        HPS_DISPATCH_F32(N, channel->engine, chf.precise, HPS_BODY)
#undef HPS_BODY
        return cuda_status(cudaGetLastError(), "hps_generate_mothers launch");
    }
#define HPS_BODY(NN, EE)                                                                                 \
    k_generate_mothers_f64<NN, EE><<<grid, 256, 0, as_stream(stream)>>>(ch, mothers, cc, weights, first_evt, n, \
                                                                         all32 ? 1 : 0);
    HPS_DISPATCH_N_ENGINE(N, channel->engine, HPS_BODY)
#undef HPS_BODY
    return cuda_status(cudaGetLastError(), "hps_generate_mothers launch");
}

hps_status hps_evaluate_mothers(const hps_channel* channel, uint64_t first_evt, uint64_t n, const double* mothers,
                                const hps_functor* functors, int32_t n_functors, double* weights, double* const* out,
                                int32_t precision, void* stream)
{
    HPS_ENTRY();
    DevChannel ch;
    hps_status st = mother_args(channel, first_evt, n, mothers, precision, &ch, true);
    if (st != HPS_OK) return st;
    if (n_functors < 0 || n_functors > kMaxMotherFunctors)
        return set_error(HPS_ERR_BAD_ARG, "n_functors %d outside 0..%d", n_functors, kMaxMotherFunctors);
    if (n == 0) return HPS_OK;
    const int N = channel->n_daughters;
    MFunctors fs{};
    MOut oc{};
    for (int k = 0; k < n_functors; ++k) {
        if ((st = mother_functor(functors + k, N, &fs.f[k])) != HPS_OK) return st;
        if (!out || !out[k]) return set_error(HPS_ERR_BAD_ARG, "output column %d is NULL", k);
        oc.p[k] = out[k];
    }
    const unsigned grid = grid_for(n, 256);
    if (precision == HPS_PREC_FP32_FIX) {
        DevChannelF chf;
        to_device_channel_f(channel, &chf);
#define HPS_BODY(NN, EE)                                                                                    \
        k_evaluate_mothers_f32fix<NN, EE><<<grid, 256, 0, as_stream(stream)>>>(ch, chf, channel->seed, mothers, fs, \
                                                                               n_functors, weights, oc, first_evt, n);
        HPS_DISPATCH_F32(N, channel->engine, chf.precise, HPS_BODY)
#undef HPS_BODY
        return cuda_status(cudaGetLastError(), "hps_evaluate_mothers launch");
    }
#define HPS_BODY(NN, EE)                                                                                    \
    k_evaluate_mothers_f64<NN, EE><<<grid, 256, 0, as_stream(stream)>>>(ch, channel->seed, mothers, fs, n_functors, \
                                                                         weights, oc, first_evt, n);
    HPS_DISPATCH_N_ENGINE(N, channel->engine, HPS_BODY)
#undef HPS_BODY
    return cuda_status(cudaGetLastError(), "hps_evaluate_mothers launch");
}

hps_status hps_average_on_mothers(const hps_channel* channel, uint64_t first_evt, uint64_t n, const double* mothers,
                                  const hps_functor* functor, hps_stats* out, void* workspace, size_t workspace_bytes,
                                  int32_t precision, void* stream)
{
    HPS_ENTRY();
    DevChannel ch;
    hps_status st = mother_args(channel, first_evt, n, mothers, precision, &ch, true);
    if (st != HPS_OK) return st;
    DevFunctor fn;
    if ((st = mother_functor(functor, channel->n_daughters, &fn)) != HPS_OK) return st;
    if (!out || !aligned(out, 8)) return set_error(HPS_ERR_BAD_ARG, "out NULL or misaligned");
    const size_t need = hps_average_on_workspace_size(n);
    cudaStream_t s = as_stream(stream);
    void* scratch = workspace;
    bool owned = false;
    if (workspace) {
        if (workspace_bytes < need)
            return set_error(HPS_ERR_BAD_ARG, "workspace of %zu bytes, %zu needed", workspace_bytes, need);
    } else {
        cudaError_t e = cudaMallocAsync(&scratch, need, s);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_error(HPS_ERR_OOM, "cudaMallocAsync(%zu): %s", need, cudaGetErrorString(e));
        }
        owned = true;
    }
    hps_stats* partials = static_cast<hps_stats*>(scratch);
    const uint64_t ntiles = (n + HPS_AVG_TILE - 1) / HPS_AVG_TILE;
    const unsigned grid = static_cast<unsigned>(ntiles < 152u * 16u ? (ntiles ? ntiles : 1) : 152u * 16u);
    if (precision == HPS_PREC_FP32_FIX) {
        DevChannelF chf;
        to_device_channel_f(channel, &chf);
        float* k0 = reinterpret_cast<float*>(out);
#define HPS_BODY(NN, EE)                                                                                        \
        if (ntiles) {                                                                                           \
            k_shift_mothers_f32<NN, EE><<<1, 32, 0, s>>>(ch, chf, fn, first_evt, mothers, k0);                  \
            k_average_mothers_tiles_f32fix<NN, EE><<<grid, kTileThreads, 0, s>>>(ch, chf, fn, first_evt, n, ntiles, \
                                                                                 partials, k0, mothers);        \
        }                                                                                                       \
        k_average_mothers_final_f32fix<NN, EE><<<1, kFinalThreads, 0, s>>>(ch, chf, fn, first_evt, partials, ntiles, out);
        HPS_DISPATCH_F32(channel->n_daughters, channel->engine, chf.precise, HPS_BODY)
#undef HPS_BODY
    } else {
        if (ntiles) {
#define HPS_BODY(NN, EE)                                                                                        \
            k_average_mothers_tiles_f64<NN, EE><<<grid, kMThreads, 0, s>>>(ch, mothers, fn, first_evt, n, ntiles, partials);
            HPS_DISPATCH_N_ENGINE(channel->n_daughters, channel->engine, HPS_BODY)
#undef HPS_BODY
        }
        k_average_mothers_final<<<1, 1024, 0, s>>>(partials, ntiles, out);
    }
    st = cuda_status(cudaGetLastError(), "hps_average_on_mothers launch");
    if (owned) {
        cudaError_t e = cudaFreeAsync(scratch, s);
        if (st == HPS_OK && e != cudaSuccess) st = cuda_status(e, "cudaFreeAsync");
    }
    return st;
}

}  // extern "C"
