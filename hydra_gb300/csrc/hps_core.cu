// hps_core.cu -- channel set-up, error state, and the entry points that walk stored
// events (event weights, unweight flags) or expose the raw random streams.
#include <cmath>
#include <cstring>
#include <functional>

#include "common.h"
#include "store.cuh"

namespace hps {

namespace {
thread_local char g_last_error[512] = "";
}

hps_status set_error(hps_status st, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return st;
}

void clear_error() { g_last_error[0] = '\0'; }

hps_status to_device_channel(const hps_channel* ch, DevChannel* out)
{
    if (!ch) return set_error(HPS_ERR_BAD_ARG, "channel is NULL");
    if (ch->n_daughters < 2 || ch->n_daughters > HPS_MAX_DAUGHTERS)
        return set_error(HPS_ERR_BAD_ARG, "n_daughters %d outside 2..10", ch->n_daughters);
    if (ch->engine == HPS_ENGINE_MINSTD)
        return set_error(HPS_ERR_BAD_ARG, "HPS_ENGINE_MINSTD channels are for hps_generate_range only");
    if (ch->engine != HPS_ENGINE_PHILOX && ch->engine != HPS_ENGINE_SQUARES3)
        return set_error(HPS_ERR_BAD_ARG, "unknown engine %d", ch->engine);
    make_channel(*ch, *out);
    return HPS_OK;
}

void to_device_channel_f(const hps_channel* ch, DevChannelF* out) { f32::make_channel_f(*ch, *out); }

bool float_float_form(const hps_channel* ch) { return f32::float_float_form(*ch); }

hps_status to_device_functor(const hps_functor* f, int n_daughters, DevFunctor* out)
{
    if (!f) return set_error(HPS_ERR_BAD_ARG, "functor is NULL");
    if (f->kind < HPS_FN_ONE || f->kind > HPS_FN_BW2)
        return set_error(HPS_ERR_BAD_ARG, "unknown functor kind %d", f->kind);
    if (f->kind != HPS_FN_ONE &&
        (f->i < 0 || f->i >= n_daughters || f->j < 0 || f->j >= n_daughters))
        return set_error(HPS_ERR_BAD_ARG, "functor daughter indices (%d,%d) outside 0..%d", f->i, f->j,
                         n_daughters - 1);
    out->kind = f->kind;
    out->i = f->i;
    out->j = f->j;
    out->a = f->a;
    out->b = f->b;
    out->fa = static_cast<float>(f->a);
    out->fb = static_cast<float>(f->b);
    return HPS_OK;
}

template <int N>
__global__ void __launch_bounds__(256)
k_event_weights(ConstCols cols, DevChannel ch, uint64_t n, double* __restrict__ out)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
         e += (uint64_t)gridDim.x * blockDim.x) {
        double p[N][4];
        load_event<N>(cols, e, p);
        out[e] = f64::recomputed_weight<N>(ch.masses, ch.max_weight, p);
    }
}

template <int N>
__global__ void __launch_bounds__(256)
k_unweight_flags(ConstCols cols, DevChannel ch, uint64_t n, uint64_t ukey, uint64_t first,
                 uint8_t* __restrict__ flags)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
         e += (uint64_t)gridDim.x * blockDim.x) {
        double p[N][4];
        load_event<N>(cols, e, p);
        const double w = f64::recomputed_weight<N>(ch.masses, ch.max_weight, p);
        const double u = static_cast<double>(squares3_word(ukey, first + e)) * 0x1p-32;
        flags[e] = (f64::dvd(w, ch.max_weight) > u) ? 1 : 0;
    }
}

template <int N, int ENGINE>
__global__ void __launch_bounds__(256)
k_rng_words(uint64_t key, uint64_t first, uint64_t n, uint64_t* __restrict__ out)
{
    constexpr int NW = 3 * N - 4;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
         e += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t w[NW];
        event_words<N, ENGINE>(key, first + e, w);
#pragma unroll
        for (int k = 0; k < NW; ++k) out[e * NW + k] = w[k];
    }
}

hps_status stored_event_args(int32_t n_daughters, const double* masses, uint64_t n,
                                    const double* const* cols, ConstCols* cc, DevChannel* ch,
                                    double max_weight)
{
    if (n_daughters < 2 || n_daughters > HPS_MAX_DAUGHTERS)
        return set_error(HPS_ERR_BAD_ARG, "n_daughters %d outside 2..10", n_daughters);
    if (!masses || !cols) return set_error(HPS_ERR_BAD_ARG, "masses/cols is NULL");
    std::memset(cc, 0, sizeof(*cc));
    std::memset(ch, 0, sizeof(*ch));
    for (int k = 0; k < n_daughters; ++k) {
        if (n && !cols[k]) return set_error(HPS_ERR_BAD_ARG, "column %d is NULL", k);
        if (!aligned(cols[k], 16)) return set_error(HPS_ERR_BAD_ARG, "column %d not 16-byte aligned", k);
        cc->p[k] = cols[k];
        ch->masses[k] = masses[k];
    }
    ch->max_weight = max_weight;
    return HPS_OK;
}

}  // namespace hps

using namespace hps;

extern "C" {

const char* hps_last_error(void) { return g_last_error; }

int32_t hps_abi_version(void) { return HPS_ABI_VERSION; }

uint64_t hps_default_seed(int32_t n, const double* masses)
{
    // hash_combine over the masses (seed ^= h + 0x9e3779b9 + (seed << 6) + (seed >> 2)),
    // then fSeed = 1 * (1 + hash).
    size_t h = 0;
    std::hash<double> hasher;
    for (int i = 0; masses && i < n; ++i) h ^= hasher(masses[i]) + 0x9e3779b9 + (h << 6) + (h >> 2);
    size_t seed = 1;
    seed *= (1 + h);
    return static_cast<uint64_t>(seed);
}

hps_status hps_channel_init(hps_channel* ch, int32_t n, int32_t engine, uint64_t seed,
                            double mother_mass, const double* masses, const double* mother)
{
    HPS_ENTRY();
    if (!ch || !masses) return set_error(HPS_ERR_BAD_ARG, "channel/masses is NULL");
    if (n < 2 || n > HPS_MAX_DAUGHTERS) return set_error(HPS_ERR_BAD_ARG, "n_daughters %d outside 2..10", n);
    if (engine != HPS_ENGINE_PHILOX && engine != HPS_ENGINE_SQUARES3)
        return set_error(HPS_ERR_BAD_ARG, "unknown engine %d", engine);
    std::memset(ch, 0, sizeof(*ch));
    ch->n_daughters = n;
    ch->engine = engine;
    ch->seed = seed;
    // hydra/detail/PhaseSpace.inl:49-61
    if (mother_mass <= 0.0)
        return set_error(HPS_ERR_BAD_ARG,
                         "[hydra::PhaseSpace]: Mass of mother particle is negative or zero. (fMotherMass <=0)");
    for (int i = 0; i < n; ++i) {
        ch->masses[i] = masses[i];
        if (masses[i] <= 0.0)
            return set_error(HPS_ERR_BAD_ARG,
                             "[hydra::PhaseSpace]: Mass of daughter particle is negative or zero. (fMass[] <=0)");
    }
    // PhaseSpace.inl:67-89: ECM and the maximum weight, in the same operation order
    // (host code is compiled with -ffp-contract=off, so nothing is fused).
    double ecm = mother_mass;
    for (int i = 0; i < n; ++i) ecm -= masses[i];
    if (ecm <= 0.0)
        return set_error(HPS_ERR_NO_ENERGY,
                         "[hydra::PhaseSpace]: Not enough energy to generate this decay. ( fECM <=0.");
    ch->ecm = ecm;
    double emmax = ecm + masses[0], emmin = 0.0, wtmax = 1.0;
    for (int i = 1; i < n; ++i) {
        emmin += masses[i - 1];
        emmax += masses[i];
        const double a = emmax, b = emmin, c = masses[i];
        double x = (a - b - c) * (a + b + c) * (a - b + c) * (a + b - c);
        x = std::sqrt(x) / (2 * a);
        wtmax *= x;
    }
    ch->max_weight = 1.0 / wtmax;
    // DecayMother.h:88-98, kept as written: the vector is (E, px, py) * (beta/|p|), so a
    // moving mother gives |beta| >= 1 and no final boost (the reference's behaviour).
    if (mother) {
        const double d3 = std::sqrt(mother[1] * mother[1] + mother[2] * mother[2] + mother[3] * mother[3]);
        const double beta = d3 / mother[0];
        if (beta != 0.0) {
            const double w = beta / d3;
            ch->beta[0] = mother[0] * w;
            ch->beta[1] = mother[1] * w;
            ch->beta[2] = mother[2] * w;
        }
    }
    return HPS_OK;
}

hps_status hps_event_weights(int32_t n_daughters, const double* masses, double max_weight, uint64_t n,
                             const double* const* cols, double* out, void* stream)
{
    HPS_ENTRY();
    ConstCols cc;
    DevChannel ch;
    hps_status st = stored_event_args(n_daughters, masses, n, cols, &cc, &ch, max_weight);
    if (st != HPS_OK) return st;
    if (n == 0) return HPS_OK;
    if (!out) return set_error(HPS_ERR_BAD_ARG, "out is NULL");
    const unsigned grid = grid_for(n, 256);
#define HPS_BODY(NN) k_event_weights<NN><<<grid, 256, 0, as_stream(stream)>>>(cc, ch, n, out);
    HPS_DISPATCH_N(n_daughters, HPS_BODY)
#undef HPS_BODY
    return cuda_status(cudaGetLastError(), "hps_event_weights launch");
}

hps_status hps_unweight_flags(int32_t n_daughters, const double* masses, double max_weight, uint64_t n,
                              const double* const* cols, uint64_t unweight_seed, uint64_t first_evt,
                              uint8_t* flags, void* stream)
{
    HPS_ENTRY();
    ConstCols cc;
    DevChannel ch;
    hps_status st = stored_event_args(n_daughters, masses, n, cols, &cc, &ch, max_weight);
    if (st != HPS_OK) return st;
    if (n == 0) return HPS_OK;
    if (!flags) return set_error(HPS_ERR_BAD_ARG, "flags is NULL");
    if (!range_ok(first_evt, n)) return set_error(HPS_ERR_BAD_ARG, "event range wraps 2^64");
    const uint64_t ukey = splitmix64(unweight_seed);
    const unsigned grid = grid_for(n, 256);
#define HPS_BODY(NN) \
    k_unweight_flags<NN><<<grid, 256, 0, as_stream(stream)>>>(cc, ch, n, ukey, first_evt, flags);
    HPS_DISPATCH_N(n_daughters, HPS_BODY)
#undef HPS_BODY
    return cuda_status(cudaGetLastError(), "hps_unweight_flags launch");
}

hps_status hps_rng_words(int32_t n_daughters, int32_t engine, uint64_t seed, uint64_t first_evt, uint64_t n,
                         uint64_t* out, void* stream)
{
    HPS_ENTRY();
    if (engine != HPS_ENGINE_PHILOX && engine != HPS_ENGINE_SQUARES3)
        return set_error(HPS_ERR_BAD_ARG, "unknown engine %d", engine);
    if (n == 0) return HPS_OK;
    if (!out) return set_error(HPS_ERR_BAD_ARG, "out is NULL");
    if (!range_ok(first_evt, n)) return set_error(HPS_ERR_BAD_ARG, "event range wraps 2^64");
    const uint64_t key = splitmix64(seed);
    const unsigned grid = grid_for(n, 256);
#define HPS_BODY(NN, EE) k_rng_words<NN, EE><<<grid, 256, 0, as_stream(stream)>>>(key, first_evt, n, out);
    HPS_DISPATCH_N_ENGINE(n_daughters, engine, HPS_BODY)
#undef HPS_BODY
    return cuda_status(cudaGetLastError(), "hps_rng_words launch");
}

}  // extern "C"
