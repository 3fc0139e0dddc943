// hps_consumers.cu -- what the reference does with a stored sample right after Generate:
// PhaseSpaceReweight and the max-weight search of Decays::Unweight(functor, weight, seed)
// (hydra/detail/Decays.inl:258-411, 458-511), hit-or-miss flags from a weight column, and the
// two-dimensional DenseHistogram of Dalitz variables (hydra/detail/DenseHistogram.inl:45-103,
// hydra/detail/functors/GetGlobalBin.h:120-138), over stored events or fused into generation.
#include <cstring>

#include "common.h"
#include "store.cuh"
#include "tiles_f32.cuh"

namespace hps {

// Doubles as unsigned keys in the same order: flip the sign bit of non-negatives, all bits of
// negatives.  atomicMax over keys is then max over doubles, whatever order the CTAs finish in.
__device__ __forceinline__ uint64_t order_key(double x)
{
    const uint64_t b = static_cast<uint64_t>(__double_as_longlong(x));
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__device__ __forceinline__ double key_value(uint64_t k)
{
    const uint64_t b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double(static_cast<long long>(b));
}

template <int N>
__global__ void __launch_bounds__(256)
k_reweight(ConstCols cols, DevChannel ch, DevFunctor fn, uint64_t n, double* __restrict__ out,
           unsigned long long* __restrict__ max_key)
{
    uint64_t best = 0;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
         e += (uint64_t)gridDim.x * blockDim.x) {
        double p[N][4];
        load_event<N>(cols, e, p);
        // PhaseSpaceReweight::Evaluate (Decays.inl:372-386): w * functor(p...)
        const double v = f64::mul(f64::recomputed_weight<N>(ch.masses, ch.max_weight, p), functor_f64<N>(fn, p));
        if (out) out[e] = v;
        const uint64_t k = order_key(v);
        best = k > best ? k : best;
    }
    if (max_key) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const uint64_t other = __shfl_xor_sync(0xffffffffu, best, o);
            best = other > best ? other : best;
        }
        if ((threadIdx.x & 31) == 0 && best) atomicMax(max_key, static_cast<unsigned long long>(best));
    }
}

__global__ void k_key_to_double(unsigned long long* slot)
{
    *reinterpret_cast<double*>(slot) = key_value(*slot);
}

__global__ void __launch_bounds__(256)
k_weight_flags(const double* __restrict__ w, uint64_t n, double max_weight, const double* __restrict__ max_dev,
               uint64_t ukey, uint64_t first, uint8_t* __restrict__ flags)
{
    const double W = max_dev ? *max_dev : max_weight;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const double u = static_cast<double>(squares3_word(ukey, first + e)) * 0x1p-32;
        flags[e] = (f64::dvd(w[e], W) > u) ? 1 : 0;
    }
}

// ----------------------------------------------------------------------- Dalitz histogram --

struct DevHist {
    int a0, a1, b0, b1;
    uint64_t g0, g1;
    double lo0, lo1, delta0, delta1;
    uint64_t nbins;          // g0 * g1 + 2
    // the FP32_FIX form: lower edges, grid / (upper - lower) and the grid sizes as floats
    float lo0f, lo1f, sc0f, sc1f, g0f, g1f;
};

// GetGlobalBin::operator() for two dimensions, each step in the reference's order:
// X = (x - lower) * grid / delta.
__device__ __forceinline__ uint64_t global_bin(const DevHist& h, double x0, double x1)
{
    const double X0 = f64::dvd(f64::mul(f64::sub(x0, h.lo0), static_cast<double>(h.g0)), h.delta0);
    const double X1 = f64::dvd(f64::mul(f64::sub(x1, h.lo1), static_cast<double>(h.g1)), h.delta1);
    const uint64_t nb = h.g0 * h.g1;
    if (X0 < 0.0 && X1 < 0.0) return nb;
    if (X0 > static_cast<double>(h.g0) && X1 > static_cast<double>(h.g1)) return nb + 1;
    if (!(X0 >= 0.0 && X0 < static_cast<double>(h.g0) && X1 >= 0.0 && X1 < static_cast<double>(h.g1)))
        return nb + 1;
    return static_cast<uint64_t>(X0) * h.g1 + static_cast<uint64_t>(X1);
}

template <int N>
__device__ __forceinline__ void dalitz_xy(const DevHist& h, const double (&p)[N][4], double& x0, double& x1)
{
    double s[4], t[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) { s[c] = 0.0; t[c] = 0.0; }
#pragma unroll
    for (int k = 0; k < N; ++k) {
        if (k == h.a0) {
#pragma unroll
            for (int c = 0; c < 4; ++c) s[c] = p[k][c];
        }
        if (k == h.b0) {
#pragma unroll
            for (int c = 0; c < 4; ++c) t[c] = p[k][c];
        }
    }
#pragma unroll
    for (int k = 0; k < N; ++k) {
        if (k == h.a1) {
#pragma unroll
            for (int c = 0; c < 4; ++c) s[c] = f64::add(s[c], p[k][c]);
        }
        if (k == h.b1) {
#pragma unroll
            for (int c = 0; c < 4; ++c) t[c] = f64::add(t[c], p[k][c]);
        }
    }
    x0 = f64::mass2(s);
    x1 = f64::mass2(t);
}

// The FP32_FIX form of both: the pair masses squared of the float four-vectors (as the FP32_FIX
// functor forms them) and the bin from X = (x - lower) * (grid / (upper - lower)) in float, the
// same under/overflow rules.  An event whose Dalitz variable lies within the float form's error of
// a bin edge may fall in the neighbouring bin.
template <int N>
__device__ __forceinline__ void dalitz_xy_f32(const DevHist& h, const float (&p)[N][4], float& x0, float& x1)
{
    float s[4] = {0.0f, 0.0f, 0.0f, 0.0f}, t[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const float ws = (k == h.a0 ? 1.0f : 0.0f) + (k == h.a1 ? 1.0f : 0.0f);
        const float wt = (k == h.b0 ? 1.0f : 0.0f) + (k == h.b1 ? 1.0f : 0.0f);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            s[c] = fmaf(ws, p[k][c], s[c]);
            t[c] = fmaf(wt, p[k][c], t[c]);
        }
    }
    x0 = fmaf(s[0], s[0], -fmaf(s[1], s[1], fmaf(s[2], s[2], s[3] * s[3])));
    x1 = fmaf(t[0], t[0], -fmaf(t[1], t[1], fmaf(t[2], t[2], t[3] * t[3])));
}

__device__ __forceinline__ uint64_t global_bin_f32(const DevHist& h, float x0, float x1)
{
    const float X0 = (x0 - h.lo0f) * h.sc0f, X1 = (x1 - h.lo1f) * h.sc1f;
    const uint64_t nb = h.g0 * h.g1;
    if (X0 < 0.0f && X1 < 0.0f) return nb;
    if (X0 > h.g0f && X1 > h.g1f) return nb + 1;
    if (!(X0 >= 0.0f && X0 < h.g0f && X1 >= 0.0f && X1 < h.g1f)) return nb + 1;
    return static_cast<uint64_t>(X0) * h.g1 + static_cast<uint64_t>(X1);
}

// Up to kSmemBins bins each CTA keeps a private copy in shared memory and adds its non-zero
// bins to the output once; larger grids add straight into the output.
constexpr int kHistThreads = 256;
constexpr uint64_t kSmemBins = 12288;      // 96 KB of doubles

struct HistSink {
    double* smem;
    double* global;
    __device__ __forceinline__ void add(uint64_t bin, double w) const
    {
        if (smem) atomicAdd(smem + bin, w);
        else atomicAdd(global + bin, w);
    }
};

__device__ __forceinline__ HistSink hist_begin(const DevHist& h, double* bins, bool use_smem)
{
    extern __shared__ double hist_smem[];
    if (use_smem) {
        for (uint64_t b = threadIdx.x; b < h.nbins; b += blockDim.x) hist_smem[b] = 0.0;
        __syncthreads();
        return HistSink{hist_smem, bins};
    }
    return HistSink{nullptr, bins};
}

__device__ __forceinline__ void hist_end(const DevHist& h, const HistSink& s)
{
    if (!s.smem) return;
    __syncthreads();
    for (uint64_t b = threadIdx.x; b < h.nbins; b += blockDim.x) {
        const double v = s.smem[b];
        if (v != 0.0) atomicAdd(s.global + b, v);
    }
}

template <int N>
__global__ void __launch_bounds__(kHistThreads)
k_dalitz_stored(ConstCols cols, DevChannel ch, const double* __restrict__ weights, int mode, DevHist h, uint64_t n,
                double* __restrict__ bins, int use_smem)
{
    const HistSink sink = hist_begin(h, bins, use_smem != 0);
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
         e += (uint64_t)gridDim.x * blockDim.x) {
        double p[N][4];
        load_event<N>(cols, e, p);
        double x0, x1;
        dalitz_xy<N>(h, p, x0, x1);
        double w = 1.0;
        if (mode == HPS_HIST_COLUMN) w = weights[e];
        else if (mode == HPS_HIST_PHSP_WEIGHT) w = f64::recomputed_weight<N>(ch.masses, ch.max_weight, p);
        sink.add(global_bin(h, x0, x1), w);
    }
    hist_end(h, sink);
}

template <int N, int ENGINE>
__global__ void __launch_bounds__(kHistThreads)
k_dalitz_generate(DevChannel ch, int mode, DevHist h, uint64_t first, uint64_t n, double* __restrict__ bins,
                  int use_smem)
{
    const HistSink sink = hist_begin(h, bins, use_smem != 0);
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
         e += (uint64_t)gridDim.x * blockDim.x) {
        double p[N][4];
        const double wt = f64::event<N, ENGINE>(ch, first + e, p);
        double x0, x1;
        dalitz_xy<N>(h, p, x0, x1);
        sink.add(global_bin(h, x0, x1), mode == HPS_HIST_PHSP_WEIGHT ? wt : 1.0);
    }
    hist_end(h, sink);
}

// FP32_FIX fused form: chunks of kTileThreads consecutive events with their random words shared by
// the CTA (cta_event_words), the float event body, binned where it is made.  From N = 9 the body
// is held to 128 registers (two CTAs per SM; the compiler's choice, 136, leaves one).
template <int N, int ENGINE>
__global__ void __launch_bounds__(kTileThreads, N >= 9 ? 2 : 0)
k_dalitz_generate_f32(DevChannel chd, DevChannelF ch, int mode, DevHist h, uint64_t first, uint64_t n,
                      double* __restrict__ bins, int use_smem)
{
    __shared__ __align__(16) unsigned char words[WordShare<N, ENGINE, kTileThreads>::BYTES2];
    const HistSink sink = hist_begin(h, bins, use_smem != 0);
    const uint64_t step = (uint64_t)gridDim.x * kTileThreads;
    int parity = 0;
    for (uint64_t cb = (uint64_t)blockIdx.x * kTileThreads; cb < n; cb += step, parity ^= 1) {
        uint64_t w[3 * N - 4];
        cta_event_words<N, ENGINE, kTileThreads>(chd.key, first + cb, words, w, parity);
        const uint64_t e = cb + threadIdx.x;
        if (e < n) {
            float p[N][4];
            const f32::EventWeight ew = f32::event_from_words<N, ENGINE>(chd, ch, w, p);
            float x0, x1;
            dalitz_xy_f32<N>(h, p, x0, x1);
            sink.add(global_bin_f32(h, x0, x1), mode == HPS_HIST_PHSP_WEIGHT ? ew.weight : 1.0);
        }
    }
    hist_end(h, sink);
}

static hps_status hist_args(const hps_hist2d* hist, int32_t n_daughters, int32_t weight_mode, DevHist* h)
{
    if (!hist) return set_error(HPS_ERR_BAD_ARG, "hist is NULL");
    const int32_t idx[4] = {hist->pair_a[0], hist->pair_a[1], hist->pair_b[0], hist->pair_b[1]};
    for (int k = 0; k < 4; ++k)
        if (idx[k] < 0 || idx[k] >= n_daughters)
            return set_error(HPS_ERR_BAD_ARG, "daughter index %d outside 0..%d", idx[k], n_daughters - 1);
    if (idx[0] == idx[1] || idx[2] == idx[3])
        return set_error(HPS_ERR_BAD_ARG, "a pair names the same daughter twice");
    if (hist->grid[0] == 0 || hist->grid[1] == 0 || hist->grid[0] > (1u << 20) || hist->grid[1] > (1u << 20))
        return set_error(HPS_ERR_BAD_ARG, "grid must be 1..2^20 bins per axis");
    for (int d = 0; d < 2; ++d)
        if (!(hist->upper[d] > hist->lower[d]))
            return set_error(HPS_ERR_BAD_ARG, "upper[%d] must exceed lower[%d]", d, d);
    if (weight_mode < HPS_HIST_UNIT || weight_mode > HPS_HIST_PHSP_WEIGHT)
        return set_error(HPS_ERR_BAD_ARG, "unknown weight mode %d", weight_mode);
    h->a0 = idx[0]; h->a1 = idx[1]; h->b0 = idx[2]; h->b1 = idx[3];
    h->g0 = hist->grid[0];
    h->g1 = hist->grid[1];
    h->lo0 = hist->lower[0];
    h->lo1 = hist->lower[1];
    // DenseHistogram keeps upper - lower (GetGlobalBin.h:50-56)
    h->delta0 = hist->upper[0] - hist->lower[0];
    h->delta1 = hist->upper[1] - hist->lower[1];
    h->nbins = h->g0 * h->g1 + 2;
    h->lo0f = static_cast<float>(h->lo0);
    h->lo1f = static_cast<float>(h->lo1);
    h->sc0f = static_cast<float>(static_cast<double>(h->g0) / h->delta0);
    h->sc1f = static_cast<float>(static_cast<double>(h->g1) / h->delta1);
    h->g0f = static_cast<float>(h->g0);
    h->g1f = static_cast<float>(h->g1);
    return HPS_OK;
}

template <typename K>
static hps_status hist_smem_setup(K kernel, const DevHist& h, int* use_smem, size_t* smem_bytes)
{
    *use_smem = h.nbins <= kSmemBins ? 1 : 0;
    *smem_bytes = *use_smem ? h.nbins * sizeof(double) : 0;
    if (*smem_bytes > 48 * 1024)
        return cuda_status(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                static_cast<int>(*smem_bytes)),
                           "cudaFuncSetAttribute");
    return HPS_OK;
}

// Enough CTAs to fill the device, few enough that each private histogram is worth clearing.
static unsigned hist_grid(uint64_t n, int use_smem)
{
    return grid_for(n, kHistThreads, use_smem ? 152u * 4u : 152u * 32u);
}

}  // namespace hps

using namespace hps;

extern "C" {

hps_status hps_reweight(int32_t n_daughters, const double* masses, double max_weight, const hps_functor* functor,
                        uint64_t n, const double* const* cols, double* out, double* max_out, void* stream)
{
    HPS_ENTRY();
    ConstCols cc;
    DevChannel ch;
    hps_status st = stored_event_args(n_daughters, masses, n, cols, &cc, &ch, max_weight);
    if (st != HPS_OK) return st;
    DevFunctor fn;
    if ((st = to_device_functor(functor, n_daughters, &fn)) != HPS_OK) return st;
    if (max_out && !aligned(max_out, 8)) return set_error(HPS_ERR_BAD_ARG, "max_out not 8-byte aligned");
    cudaStream_t s = as_stream(stream);
    unsigned long long* key = reinterpret_cast<unsigned long long*>(max_out);
    if (key && (st = cuda_status(cudaMemsetAsync(key, 0, sizeof(*key), s), "cudaMemsetAsync")) != HPS_OK) return st;
    if (n) {
        const unsigned grid = grid_for(n, 256);
#define HPS_BODY(NN) k_reweight<NN><<<grid, 256, 0, s>>>(cc, ch, fn, n, out, key);
        HPS_DISPATCH_N(n_daughters, HPS_BODY)
#undef HPS_BODY
    }
    if (key) k_key_to_double<<<1, 1, 0, s>>>(key);
    return cuda_status(cudaGetLastError(), "hps_reweight launch");
}

hps_status hps_weight_flags(uint64_t n, const double* weights, double max_weight, const double* max_weight_dev,
                            uint64_t unweight_seed, uint64_t first_evt, uint8_t* flags, void* stream)
{
    HPS_ENTRY();
    if (n == 0) return HPS_OK;
    if (!weights || !flags) return set_error(HPS_ERR_BAD_ARG, "weights/flags is NULL");
    if (!range_ok(first_evt, n)) return set_error(HPS_ERR_BAD_ARG, "event range wraps 2^64");
    const unsigned grid = grid_for(n, 256);
    k_weight_flags<<<grid, 256, 0, as_stream(stream)>>>(weights, n, max_weight, max_weight_dev,
                                                         splitmix64(unweight_seed), first_evt, flags);
    return cuda_status(cudaGetLastError(), "hps_weight_flags launch");
}

hps_status hps_dalitz_histogram(int32_t n_daughters, const double* masses, double max_weight, uint64_t n,
                                const double* const* cols, const double* weights, int32_t weight_mode,
                                const hps_hist2d* hist, double* bins, void* stream)
{
    HPS_ENTRY();
    ConstCols cc;
    DevChannel ch;
    hps_status st = stored_event_args(n_daughters, masses, n, cols, &cc, &ch, max_weight);
    if (st != HPS_OK) return st;
    DevHist h;
    if ((st = hist_args(hist, n_daughters, weight_mode, &h)) != HPS_OK) return st;
    if (!bins || !aligned(bins, 8)) return set_error(HPS_ERR_BAD_ARG, "bins NULL or misaligned");
    if (weight_mode == HPS_HIST_COLUMN && n && !weights) return set_error(HPS_ERR_BAD_ARG, "weights is NULL");
    cudaStream_t s = as_stream(stream);
    if ((st = cuda_status(cudaMemsetAsync(bins, 0, h.nbins * sizeof(double), s), "cudaMemsetAsync")) != HPS_OK)
        return st;
    if (n == 0) return HPS_OK;
#define HPS_BODY(NN)                                                                                     \
    {                                                                                                    \
        int use_smem;                                                                                    \
        size_t smem;                                                                                     \
        if ((st = hist_smem_setup(k_dalitz_stored<NN>, h, &use_smem, &smem)) != HPS_OK) return st;       \
        k_dalitz_stored<NN><<<hist_grid(n, use_smem), kHistThreads, smem, s>>>(cc, ch, weights, weight_mode, h, n, \
                                                                              bins, use_smem);          \
    }
    HPS_DISPATCH_N(n_daughters, HPS_BODY)
#undef HPS_BODY
    return cuda_status(cudaGetLastError(), "hps_dalitz_histogram launch");
}

hps_status hps_generate_dalitz(const hps_channel* channel, uint64_t first_evt, uint64_t n, int32_t weight_mode,
                               const hps_hist2d* hist, double* bins, int32_t precision, void* stream)
{
    HPS_ENTRY();
    DevChannel ch;
    hps_status st = to_device_channel(channel, &ch);
    if (st != HPS_OK) return st;
    if (weight_mode == HPS_HIST_COLUMN)
        return set_error(HPS_ERR_BAD_ARG, "HPS_HIST_COLUMN needs stored weights: use hps_dalitz_histogram");
    DevHist h;
    if ((st = hist_args(hist, channel->n_daughters, weight_mode, &h)) != HPS_OK) return st;
    if (!bins || !aligned(bins, 8)) return set_error(HPS_ERR_BAD_ARG, "bins NULL or misaligned");
    if (!range_ok(first_evt, n)) return set_error(HPS_ERR_BAD_ARG, "event range wraps 2^64");
    if (precision != HPS_PREC_FP64 && precision != HPS_PREC_FP32_FIX)
        return set_error(HPS_ERR_BAD_ARG, "unknown precision %d", precision);
    cudaStream_t s = as_stream(stream);
    if ((st = cuda_status(cudaMemsetAsync(bins, 0, h.nbins * sizeof(double), s), "cudaMemsetAsync")) != HPS_OK)
        return st;
    if (n == 0) return HPS_OK;
    if (precision == HPS_PREC_FP32_FIX) {
        DevChannelF chf;
        to_device_channel_f(channel, &chf);
#define HPS_BODY(NN, EE)                                                                                   \
        {                                                                                                  \
            int use_smem;                                                                                  \
            size_t smem;                                                                                   \
            if ((st = hist_smem_setup(k_dalitz_generate_f32<NN, EE>, h, &use_smem, &smem)) != HPS_OK) return st; \
            k_dalitz_generate_f32<NN, EE><<<hist_grid(n, use_smem), kTileThreads, smem, s>>>(             \
                ch, chf, weight_mode, h, first_evt, n, bins, use_smem);                                    \
        }
        HPS_DISPATCH_F32(channel->n_daughters, channel->engine, chf.precise, HPS_BODY)
#undef HPS_BODY
        return cuda_status(cudaGetLastError(), "hps_generate_dalitz launch");
    }
#define HPS_BODY(NN, EE)                                                                                   \
    {                                                                                                      \
        int use_smem;                                                                                      \
        size_t smem;                                                                                       \
        if ((st = hist_smem_setup(k_dalitz_generate<NN, EE>, h, &use_smem, &smem)) != HPS_OK) return st;   \
        k_dalitz_generate<NN, EE><<<hist_grid(n, use_smem), kHistThreads, smem, s>>>(ch, weight_mode, h, first_evt, \
                                                                                    n, bins, use_smem);   \
    }
    HPS_DISPATCH_N_ENGINE(channel->n_daughters, channel->engine, HPS_BODY)
#undef HPS_BODY
    return cuda_status(cudaGetLastError(), "hps_generate_dalitz launch");
}

}  // extern "C"
