// hps_range.cu -- phase_space_range (hydra/detail/PhaseSpaceRange.inl:46-73): the lazy event range
// of GenerateDecay (hydra/detail/functors/GenerateDecay.h:222-334) over thrust's minstd_rand,
// materialised for an index window.  The event body is the DecayMother body; only the engine and
// the constructor differ (ECM and maximum weight from the mother four-vector's mass).
#include <cmath>
#include <cstring>

#include "common.h"
#include "store.cuh"
#include "tiles_f32.cuh"

namespace hps {

template <int N>
__global__ void __launch_bounds__(256)
k_generate_range_f64(DevChannel ch, Cols cols, double* __restrict__ weights, uint64_t first, uint64_t n, int vec32)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
         e += (uint64_t)gridDim.x * blockDim.x) {
        double p[N][4];
        const double wt = f64::event<N, kMinstd>(ch, first + e, p);
#pragma unroll
        for (int k = 0; k < N; ++k) store_vec4(cols.p[k], e, p[k], vec32 != 0);
        if (weights) weights[e] = wt;
    }
}

}  // namespace hps

using namespace hps;

extern "C" {

hps_status hps_range_channel(hps_channel* ch, int32_t n_daughters, const double* masses, const double* mother,
                             uint64_t seed)
{
    HPS_ENTRY();
    if (!ch || !masses || !mother) return set_error(HPS_ERR_BAD_ARG, "channel/masses/mother is NULL");
    // Vector4R::mass() (hydra/detail/Vector4R.inl:196-209): sqrt(E^2 - p^2) when positive, else 0
    const double m2 = mother[0] * mother[0] - mother[1] * mother[1] - mother[2] * mother[2] - mother[3] * mother[3];
    const double M = m2 > 0.0 ? std::sqrt(m2) : 0.0;
    // GenerateDecay keeps the seed as GInt_t and seeds the engine with it (GenerateDecay.h:66, 224)
    const uint64_t seed32 = static_cast<uint32_t>(seed);
    hps_status st = hps_channel_init(ch, n_daughters, HPS_ENGINE_PHILOX, seed32, M, masses, mother);
    if (st != HPS_OK) return st;
    ch->engine = HPS_ENGINE_MINSTD;
    return HPS_OK;
}

hps_status hps_generate_range(const hps_channel* channel, uint64_t first_evt, uint64_t n, double* const* cols,
                              double* weights, void* stream)
{
    HPS_ENTRY();
    if (!channel) return set_error(HPS_ERR_BAD_ARG, "channel is NULL");
    if (channel->engine != HPS_ENGINE_MINSTD)
        return set_error(HPS_ERR_BAD_ARG, "hps_generate_range takes a channel from hps_range_channel");
    hps_channel c = *channel;
    c.engine = HPS_ENGINE_PHILOX;             // validate everything but the engine
    DevChannel ch;
    hps_status st = to_device_channel(&c, &ch);
    if (st != HPS_OK) return st;
    ch.key = lcg_seed_state(channel->seed);
    if (!range_ok(first_evt, n)) return set_error(HPS_ERR_BAD_ARG, "event range wraps 2^64");
    if (n == 0) return HPS_OK;
    if (!cols) return set_error(HPS_ERR_BAD_ARG, "cols is NULL");
    const int N = channel->n_daughters;
    Cols cc{};
    bool all32 = true;
    for (int k = 0; k < N; ++k) {
        if (!cols[k] || !aligned(cols[k], 16)) return set_error(HPS_ERR_BAD_ARG, "column %d NULL or misaligned", k);
        all32 = all32 && aligned(cols[k], 32);
        cc.p[k] = cols[k];
    }
    const unsigned grid = grid_for(n, 256);
#define HPS_BODY(NN) \
    k_generate_range_f64<NN><<<grid, 256, 0, as_stream(stream)>>>(ch, cc, weights, first_evt, n, all32 ? 1 : 0);
    HPS_DISPATCH_N(N, HPS_BODY)
#undef HPS_BODY
    return cuda_status(cudaGetLastError(), "hps_generate_range launch");
}

}  // extern "C"
