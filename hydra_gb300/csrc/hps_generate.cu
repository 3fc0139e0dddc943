// hps_generate.cu -- Generate (store path) and Evaluate entry points.
//
// Generate replaces hydra::detail::launch_decayer -> thrust::tabulate(Decays, DecayMother)
// (hydra/detail/launch_decayers.inl:133-149); Evaluate replaces launch_evaluator ->
// thrust::tabulate(multivector, EvalMother) (launch_decayers.inl:66-72).  One thread owns
// one event; events of a warp are consecutive, so every column store of a warp is one
// contiguous 1 KiB span.
#include <mutex>

#include "common.h"
#include "store.cuh"
#include "tiles_f32.cuh"

namespace hps {

template <int N, int ENGINE>
__global__ void __launch_bounds__(256)
k_generate_f64(DevChannel ch, Cols cols, double* __restrict__ weights, uint8_t* __restrict__ flags,
               uint64_t ukey, uint64_t first, uint64_t n, int vec32)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
         e += (uint64_t)gridDim.x * blockDim.x) {
        double p[N][4];
        const double wt = f64::event<N, ENGINE>(ch, first + e, p);
#pragma unroll
        for (int k = 0; k < N; ++k) store_vec4(cols.p[k], e, p[k], vec32 != 0);
        if (weights) weights[e] = wt;
        if (flags) {
            // FlagDaugthers (hydra/detail/Decays.inl:77-89) on the event just stored.
            const double wr = f64::recomputed_weight<N>(ch.masses, ch.max_weight, p);
            const double u = static_cast<double>(squares3_word(ukey, first + e)) * 0x1p-32;
            flags[e] = (f64::dvd(wr, ch.max_weight) > u) ? 1 : 0;
        }
    }
}

// FP32_FIX store path: kinematics in float (light-cone boosts, exact-octant angles), weight
// finished in double, four-vectors widened to double for the Decays columns.  Each CTA takes two
// chunks of gen_threads(N) consecutive events per iteration and shares their random words
// (cta_event_words_pair, cta_words_pair_fill).  The unweight flag tests prod(pdk) -- weight /
// max_weight, the quantity FlagDaugthers tests -- against u using the generation-time weight.
constexpr int kGenThreads = kTileThreads;

// CTA size of the store kernel and the resident CTAs per SM its register allocation must allow
// (the second argument of __launch_bounds__: registers are capped at 65536 / (threads x CTAs); 0
// leaves the choice to the compiler).  Smaller CTAs wait less at the per-chunk barrier of the
// shared random words, at the cost of (B - 1) / NT more Philox blocks per event; from N = 7 the
// event body is long enough that 256 threads pay, and at N = 7..9 a register cap beats the
// compiler's choice.  Measured at 2^24 events (ms; registers in brackets):
//   N                  2      3      4      5      6      7      8      9      10
//   128, compiler  0.169  0.287  0.396  0.506  0.794  1.438  1.770  2.223  2.838  (47..110)
//   128, 6 CTAs    0.167  0.293  0.400  0.533  0.808  1.489  1.807  2.212  2.727  (<= 80)
//   256, compiler  0.174  0.295  0.396  0.530  0.814  1.476  1.836  2.127  2.400  (47..110)
//   256, 2 CTAs    0.174  0.318  0.493  0.555  0.914  1.522  1.929  2.208  2.482  (<= 128)
//   256, 3 CTAs    0.174  0.326  0.433  0.561  0.832  1.423  1.705  2.015  2.511  (<= 80)
//   256, 4 CTAs    0.176  0.301  0.397  0.531  0.836  1.408  1.767  2.127  2.686  (<= 64)
// At N = 10 the order turns at the 2^26 events of the ten-pion workload: 10.08 ms with 2 CTAs,
// 10.39 with 3 and 10.66 with the compiler's 110 registers, so N = 10 takes 2 CTAs.
// With the current event body, N = 2..6 at 2^24 events (ms): the compiler's 44..64 registers
// 0.165 0.276 0.382 0.487 0.773; 10 CTAs (48 registers) 0.165 0.277 0.385 0.496 0.782; 12 CTAs
// (40 registers, spilling at N = 3, 4, 6) 0.166 0.277 0.399 0.499 0.827.  More resident warps do
// not pay for the tighter schedule, so N <= 6 keeps the compiler's choice.
__host__ __device__ constexpr int gen_threads(int N) { return N <= 6 ? 128 : kGenThreads; }
__host__ __device__ constexpr int gen_min_ctas(int N) { return N <= 6 ? 0 : N == 7 ? 4 : N == 10 ? 2 : 3; }

// Two events per thread and iteration (store_pair_f32: one word exchange for two chunks, and two
// independent event bodies for the scheduler to interleave) pays where an event is short: at 2^24
// events N = 2 0.174 ms against 0.186, N = 3 0.320 against 0.328, N = 4 0.463 against 0.469; at
// N = 5 and 6 the doubled registers (76 and 91) cost more than it saves (0.671 against 0.618,
// 0.900 against 0.797).
// From N = 5 on, the two events of an iteration are computed one after the other from the same
// word exchange (store_pair_seq_f32: the registers of one event, one barrier per two chunks):
// N = 5 0.613 ms against 0.618, N = 7 1.284 against 1.298, N = 10 2.254 against 2.326.  N = 8
// and 9 keep one exchange per chunk (store_chunk_f32; N = 8: 1.562 against 1.570).
enum : int { kGenChunk = 0, kGenPair = 1, kGenPairSeq = 2 };
__host__ __device__ constexpr int gen_form(int N)
{
    return N <= 4 ? kGenPair : (N == 8 || N == 9) ? kGenChunk : kGenPairSeq;
}

// Events a CTA takes per iteration: two chunks of gen_threads(N) events, or one.
__host__ __device__ constexpr int gen_events_per_iteration(int N)
{
    return gen_form(N) == kGenChunk ? gen_threads(N) : 2 * gen_threads(N);
}

// Grid cap of the store kernel (CTAs loop over chunks beyond it).  At 2^24 events, N = 5: 152 x 128
// CTAs 0.618 ms, x 64 0.621, x 256 0.622, x 512 0.628, one CTA per chunk 0.640, one resident wave
// (152 x 10) 0.667.
constexpr unsigned kGenMaxCtas = 152u * 128u;

template <int N, int ENGINE>
__global__ void __launch_bounds__(gen_threads(N), gen_min_ctas(N))
k_generate_f32fix(DevChannel chd, DevChannelF ch, Cols cols, double* __restrict__ weights,
                  uint8_t* __restrict__ flags, uint64_t ukey, uint64_t first, uint64_t n, int vec32)
{
    constexpr int NT = gen_threads(N);
    __shared__ __align__(16) unsigned char smem[WordShare<N, ENGINE, 2 * NT>::BYTES2];
    const uint64_t step = (uint64_t)gridDim.x * gen_events_per_iteration(N);
    int parity = 0;
    for (uint64_t cb = (uint64_t)blockIdx.x * gen_events_per_iteration(N); cb < n; cb += step, parity ^= 1) {
        if constexpr (gen_form(N) == kGenPair)
            store_pair_f32<N, ENGINE, NT>(chd, ch, cols, weights, flags, ukey, first, n, cb, vec32 != 0, smem,
                                          parity);
        else if constexpr (gen_form(N) == kGenPairSeq)
            store_pair_seq_f32<N, ENGINE, NT>(chd, ch, cols, weights, flags, ukey, first, n, cb, vec32 != 0, smem,
                                              parity);
        else
            store_chunk_f32<N, ENGINE, NT>(chd, ch, cols, weights, flags, ukey, first, n, cb, vec32 != 0, smem,
                                           parity);
    }
}

constexpr int kMaxFunctors = 8;
struct Functors { DevFunctor f[kMaxFunctors]; };
struct OutCols { double* p[kMaxFunctors]; };

template <int N, int ENGINE>
__global__ void __launch_bounds__(256)
k_evaluate_f64(DevChannel ch, Functors fs, int nf, double* __restrict__ weights, OutCols out,
               uint64_t first, uint64_t n)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
         e += (uint64_t)gridDim.x * blockDim.x) {
        double p[N][4];
        const double wt = f64::event<N, ENGINE>(ch, first + e, p);
        if (weights) weights[e] = wt;
        for (int k = 0; k < nf; ++k) out.p[k][e] = functor_f64<N>(fs.f[k], p);
    }
}

template <int N, int ENGINE>
__global__ void __launch_bounds__(kGenThreads)
k_evaluate_f32fix(DevChannel chd, DevChannelF ch, Functors fs, int nf, double* __restrict__ weights,
                  OutCols out, uint64_t first, uint64_t n)
{
    __shared__ __align__(16) unsigned char smem[WordShare<N, ENGINE, kGenThreads>::BYTES2];
    const uint64_t step = (uint64_t)gridDim.x * kGenThreads;
    int parity = 0;
    for (uint64_t cb = (uint64_t)blockIdx.x * kGenThreads; cb < n; cb += step, parity ^= 1) {
        uint64_t w[3 * N - 4];
        cta_event_words<N, ENGINE, kGenThreads>(chd.key, first + cb, smem, w, parity);
        const uint64_t e = cb + threadIdx.x;
        if (e < n) {
            float p[N][4];
            const f32::EventWeight ew = f32::event_from_words<N, ENGINE>(chd, ch, w, p);
            if (weights) weights[e] = ew.weight;
            for (int k = 0; k < nf; ++k) out.p[k][e] = f32::widen(f32::functor<N>(fs.f[k], p));
        }
    }
}

}  // namespace hps

using namespace hps;

extern "C" {

hps_status hps_generate(const hps_channel* channel, uint64_t first_evt, uint64_t n, double* const* cols,
                        double* weights, uint8_t* flags, uint64_t unweight_seed, int32_t precision,
                        void* stream)
{
    HPS_ENTRY();
    DevChannel ch;
    hps_status st = to_device_channel(channel, &ch);
    if (st != HPS_OK) return st;
    if (precision != HPS_PREC_FP64 && precision != HPS_PREC_FP32_FIX)
        return set_error(HPS_ERR_BAD_ARG, "unknown precision %d", precision);
    if (!range_ok(first_evt, n)) return set_error(HPS_ERR_BAD_ARG, "event range wraps 2^64");
    if (n == 0) return HPS_OK;
    if (!cols) return set_error(HPS_ERR_BAD_ARG, "cols is NULL");
    const int N = channel->n_daughters;
    Cols cc{};
    bool all32 = true;
    for (int k = 0; k < N; ++k) {
        if (!cols[k]) return set_error(HPS_ERR_BAD_ARG, "column %d is NULL", k);
        if (!aligned(cols[k], 16)) return set_error(HPS_ERR_BAD_ARG, "column %d not 16-byte aligned", k);
        all32 = all32 && aligned(cols[k], 32);
        cc.p[k] = cols[k];
    }
    if (weights && !aligned(weights, 8)) return set_error(HPS_ERR_BAD_ARG, "weights not 8-byte aligned");
    const uint64_t ukey = splitmix64(unweight_seed);
    const unsigned grid = grid_for(n, 256);
    const int vec32 = all32 ? 1 : 0;
    if (precision == HPS_PREC_FP32_FIX) {
        DevChannelF chf;
        to_device_channel_f(channel, &chf);
#define HPS_BODY(NN, EE)                                                                         \
        k_generate_f32fix<NN, EE><<<grid_for(n, gen_events_per_iteration(NN), kGenMaxCtas), gen_threads(NN), 0, as_stream(stream)>>>(ch, chf, cc, weights, flags, ukey, \
                                                                        first_evt, n, vec32);
        HPS_DISPATCH_F32(N, channel->engine, chf.precise, HPS_BODY)
#undef HPS_BODY
    } else {
#define HPS_BODY(NN, EE)                                                                  \
        k_generate_f64<NN, EE><<<grid, 256, 0, as_stream(stream)>>>(ch, cc, weights, flags, ukey, \
                                                                     first_evt, n, vec32);
        HPS_DISPATCH_N_ENGINE(N, channel->engine, HPS_BODY)
#undef HPS_BODY
    }
    return cuda_status(cudaGetLastError(), "hps_generate launch");
}

hps_status hps_evaluate(const hps_channel* channel, uint64_t first_evt, uint64_t n, const hps_functor* functors,
                        int32_t n_functors, double* weights, double* const* out, int32_t precision, void* stream)
{
    HPS_ENTRY();
    DevChannel ch;
    hps_status st = to_device_channel(channel, &ch);
    if (st != HPS_OK) return st;
    if (precision != HPS_PREC_FP64 && precision != HPS_PREC_FP32_FIX)
        return set_error(HPS_ERR_BAD_ARG, "unknown precision %d", precision);
    if (n_functors < 0 || n_functors > kMaxFunctors)
        return set_error(HPS_ERR_BAD_ARG, "n_functors %d outside 0..%d", n_functors, kMaxFunctors);
    if (!range_ok(first_evt, n)) return set_error(HPS_ERR_BAD_ARG, "event range wraps 2^64");
    if (n == 0) return HPS_OK;
    const int N = channel->n_daughters;
    Functors fs{};
    OutCols oc{};
    for (int k = 0; k < n_functors; ++k) {
        st = to_device_functor(functors + k, N, &fs.f[k]);
        if (st != HPS_OK) return st;
        if (!out || !out[k]) return set_error(HPS_ERR_BAD_ARG, "output column %d is NULL", k);
        oc.p[k] = out[k];
    }
    const unsigned grid = grid_for(n, 256);
    if (precision == HPS_PREC_FP32_FIX) {
        DevChannelF chf;
        to_device_channel_f(channel, &chf);
#define HPS_BODY(NN, EE)                                                                           \
        k_evaluate_f32fix<NN, EE><<<grid, kGenThreads, 0, as_stream(stream)>>>(ch, chf, fs, n_functors, weights, \
                                                                        oc, first_evt, n);
        HPS_DISPATCH_F32(N, channel->engine, chf.precise, HPS_BODY)
#undef HPS_BODY
    } else {
#define HPS_BODY(NN, EE)                                                                          \
        k_evaluate_f64<NN, EE><<<grid, 256, 0, as_stream(stream)>>>(ch, fs, n_functors, weights, oc, \
                                                                     first_evt, n);
        HPS_DISPATCH_N_ENGINE(N, channel->engine, HPS_BODY)
#undef HPS_BODY
    }
    return cuda_status(cudaGetLastError(), "hps_evaluate launch");
}

}  // extern "C"

namespace hps {

// Per-device copy stream of the host-output pipeline, created on first use.  Events are
// per call, so concurrent calls from several host threads do not share state.
struct HostPipe {
    cudaStream_t copy = nullptr;
    cudaEvent_t gen_done[2] = {nullptr, nullptr};
    cudaEvent_t copy_done[2] = {nullptr, nullptr};
    ~HostPipe()
    {
        for (int b = 0; b < 2; ++b) {
            if (gen_done[b]) cudaEventDestroy(gen_done[b]);
            if (copy_done[b]) cudaEventDestroy(copy_done[b]);
        }
    }
};

static hps_status copy_stream(cudaStream_t* out)
{
    static std::mutex mu;
    static cudaStream_t streams[64];
    static bool ready[64] = {false};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64) return set_error(HPS_ERR_UNSUPPORTED, "device ordinal %d", dev);
    std::lock_guard<std::mutex> lock(mu);
    if (!ready[dev]) {
        if ((e = cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking)) != cudaSuccess)
            return cuda_status(e, "cudaStreamCreate");
        ready[dev] = true;
    }
    *out = streams[dev];
    return HPS_OK;
}

}  // namespace hps

namespace hps {

// Device addresses of pinned, device-mapped host buffers; false if any buffer is not one.
static bool map_host_outputs(int N, double* const* host_cols, double* host_weights, uint8_t* host_flags,
                             double** dcols, double** dw, uint8_t** df)
{
    bool mapped = true;
    auto map = [&](void* h, void** d) {
        *d = nullptr;
        if (!h || !mapped) return;
        if (cudaHostGetDevicePointer(d, h, 0) != cudaSuccess) {
            cudaGetLastError();
            mapped = false;
        }
    };
    for (int k = 0; k < N; ++k) map(host_cols[k], reinterpret_cast<void**>(&dcols[k]));
    map(host_weights, reinterpret_cast<void**>(dw));
    map(host_flags, reinterpret_cast<void**>(df));
    return mapped;
}

}  // namespace hps

extern "C" hps_status hps_generate_host(const hps_channel* channel, uint64_t first_evt, uint64_t n,
                                        double* const* host_cols, double* host_weights, uint8_t* host_flags,
                                        uint64_t unweight_seed, int32_t precision, uint64_t chunk_events,
                                        void* stream)
{
    HPS_ENTRY();
    DevChannel ch;
    hps_status st = to_device_channel(channel, &ch);
    if (st != HPS_OK) return st;
    if (!range_ok(first_evt, n)) return set_error(HPS_ERR_BAD_ARG, "event range wraps 2^64");
    if (n == 0) return HPS_OK;
    const int N = channel->n_daughters;
    if (!host_cols) return set_error(HPS_ERR_BAD_ARG, "host_cols is NULL");
    for (int k = 0; k < N; ++k)
        if (!host_cols[k]) return set_error(HPS_ERR_BAD_ARG, "host column %d is NULL", k);
    if (chunk_events == 0) {
        // Direct mode: when every host buffer is pinned, device-mapped memory, the kernel writes
        // the Decays straight into it across the CPU-GPU link -- no staging copy, no copy engine.
        double* dcols[HPS_MAX_DAUGHTERS];
        double* dw = nullptr;
        uint8_t* df = nullptr;
        if (map_host_outputs(N, host_cols, host_weights, host_flags, dcols, &dw, &df)) {
            st = hps_generate(channel, first_evt, n, dcols, dw, df, unweight_seed, precision, stream);
            if (st != HPS_OK) return st;
            return cuda_status(cudaStreamSynchronize(as_stream(stream)), "cudaStreamSynchronize");
        }
    }
    const uint64_t chunk = chunk_events ? chunk_events : (uint64_t(1) << 20);
    // staging: N columns of 32 B/event (32-byte aligned), then weights, then flags
    const size_t col_bytes = (size_t)chunk * 32;
    const size_t buf_bytes = (col_bytes * N + (size_t)chunk * 8 + (size_t)chunk + 255) / 256 * 256;
    HostPipe pipeobj;
    HostPipe* pipe = &pipeobj;
    if ((st = copy_stream(&pipe->copy)) != HPS_OK) return st;
    for (int b = 0; b < 2; ++b) {
        cudaError_t ee;
        if ((ee = cudaEventCreateWithFlags(&pipe->gen_done[b], cudaEventDisableTiming)) != cudaSuccess ||
            (ee = cudaEventCreateWithFlags(&pipe->copy_done[b], cudaEventDisableTiming)) != cudaSuccess)
            return cuda_status(ee, "cudaEventCreate");
    }
    cudaStream_t s = as_stream(stream);
    void* staging = nullptr;
    cudaError_t e = cudaMallocAsync(&staging, 2 * buf_bytes, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(HPS_ERR_OOM, "staging cudaMallocAsync(%zu): %s", 2 * buf_bytes, cudaGetErrorString(e));
    }
    const uint64_t nchunks = (n + chunk - 1) / chunk;
    for (uint64_t c = 0; c < nchunks && st == HPS_OK; ++c) {
        const int b = static_cast<int>(c & 1);
        const uint64_t off = c * chunk;
        const uint64_t m = (n - off < chunk) ? (n - off) : chunk;
        char* base = static_cast<char*>(staging) + b * buf_bytes;
        double* dcols[HPS_MAX_DAUGHTERS];
        for (int k = 0; k < N; ++k) dcols[k] = reinterpret_cast<double*>(base + k * col_bytes);
        double* dw = host_weights ? reinterpret_cast<double*>(base + N * col_bytes) : nullptr;
        uint8_t* df = host_flags ? reinterpret_cast<uint8_t*>(base + N * col_bytes + chunk * 8) : nullptr;
        if (c >= 2 && (e = cudaStreamWaitEvent(s, pipe->copy_done[b], 0)) != cudaSuccess) {
            st = cuda_status(e, "cudaStreamWaitEvent");
            break;
        }
        st = hps_generate(channel, first_evt + off, m, dcols, dw, df, unweight_seed, precision, stream);
        if (st != HPS_OK) break;
        if ((e = cudaEventRecord(pipe->gen_done[b], s)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(pipe->copy, pipe->gen_done[b], 0)) != cudaSuccess) {
            st = cuda_status(e, "pipeline event");
            break;
        }
        for (int k = 0; k < N && e == cudaSuccess; ++k)
            e = cudaMemcpyAsync(host_cols[k] + 4 * off, dcols[k], m * 32, cudaMemcpyDeviceToHost, pipe->copy);
        if (e == cudaSuccess && dw)
            e = cudaMemcpyAsync(host_weights + off, dw, m * 8, cudaMemcpyDeviceToHost, pipe->copy);
        if (e == cudaSuccess && df)
            e = cudaMemcpyAsync(host_flags + off, df, m, cudaMemcpyDeviceToHost, pipe->copy);
        if (e == cudaSuccess) e = cudaEventRecord(pipe->copy_done[b], pipe->copy);
        if (e != cudaSuccess) st = cuda_status(e, "device-to-host copy");
    }
    // the staging buffers may be released only after the last copies read them
    for (int b = 0; b < 2 && b < (int)nchunks; ++b) cudaStreamWaitEvent(s, pipe->copy_done[b], 0);
    e = cudaFreeAsync(staging, s);
    if (st == HPS_OK && e != cudaSuccess) st = cuda_status(e, "cudaFreeAsync");
    e = cudaStreamSynchronize(s);
    if (st == HPS_OK && e != cudaSuccess) st = cuda_status(e, "cudaStreamSynchronize");
    return st;
}

extern "C" hps_status hps_generate_average_host(const hps_channel* channel, uint64_t first_evt, uint64_t n,
                                                double* const* host_cols, double* host_weights, uint8_t* host_flags,
                                                uint64_t unweight_seed, const hps_functor* functor, hps_stats* out,
                                                int32_t precision, void* stream)
{
    HPS_ENTRY();
    DevChannel ch;
    hps_status st = to_device_channel(channel, &ch);
    if (st != HPS_OK) return st;
    if (!host_cols && n) return set_error(HPS_ERR_BAD_ARG, "host_cols is NULL");
    const int N = channel->n_daughters;
    for (int k = 0; k < N && n; ++k)
        if (!host_cols[k]) return set_error(HPS_ERR_BAD_ARG, "host column %d is NULL", k);
    double* dcols[HPS_MAX_DAUGHTERS] = {};
    double* dw = nullptr;
    uint8_t* df = nullptr;
    if (n && map_host_outputs(N, host_cols, host_weights, host_flags, dcols, &dw, &df)) {
        // one pass: the kernel writes the Decays across the link and reduces AverageOn meanwhile
        st = hps_generate_average(channel, first_evt, n, dcols, dw, df, unweight_seed, functor, out, nullptr, 0,
                                  precision, stream);
    } else {
        st = hps_generate_host(channel, first_evt, n, host_cols, host_weights, host_flags, unweight_seed, precision, 0,
                               stream);
        if (st == HPS_OK)
            st = hps_average_on(channel, first_evt, n, functor, out, nullptr, 0, precision, stream);
    }
    if (st != HPS_OK) return st;
    return cuda_status(cudaStreamSynchronize(as_stream(stream)), "cudaStreamSynchronize");
}
