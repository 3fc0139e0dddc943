// hps_noalloc.cu -- AverageOn that performs no device allocation of any kind.
//
// hps_average_on needs a small scratch array (one partial StatsPHSP per tile of HPS_AVG_TILE
// events) and takes it from the caller's workspace or from the stream-ordered allocator.  Some
// host programs cannot provide either: a framework that reserves all device memory for its
// own pool when it starts and treats any later cudaMalloc as an error, a process confined to a
// fixed memory quota on a shared GPU, or a latency-critical loop that must never pay for an
// allocator call.  For them the scratch lives in the fixed-size device array below, which the
// CUDA module reserves when it is loaded; every GPU that loads this library keeps it until the
// process exits.
#include <mutex>

#include "common.h"

namespace hps {

constexpr uint64_t kNoallocMaxTiles = HPS_NOALLOC_MAX_EVENTS / HPS_AVG_TILE;
static_assert(kNoallocMaxTiles * HPS_AVG_TILE == HPS_NOALLOC_MAX_EVENTS, "limit is a whole number of tiles");

// 16384 tiles x 24 bytes = 384 KiB per device.
static __device__ __align__(256) hps_stats g_noalloc_partials[kNoallocMaxTiles];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
hps_stats* g_noalloc_addr[kMaxDevices] = {};

// Device address of g_noalloc_partials on the current device.  In host code the symbol is
// only a host-side stand-in, so the address is looked up once per device (with that device
// current) and cached; the first call on a device does this set-up.  The cache assumes that the
// device's primary context lives as long as the process: after cudaDeviceReset the module is
// loaded again, possibly at another address, and the cached one must not be used (a program
// that resets a device does not call this entry point afterwards).
hps_status noalloc_scratch(hps_stats** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return set_error(HPS_ERR_UNSUPPORTED, "device ordinal %d", dev);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_noalloc_partials)");
        g_noalloc_addr[dev] = static_cast<hps_stats*>(p);
    }
    *out = g_noalloc_addr[dev];
    return HPS_OK;
}

}  // namespace
}  // namespace hps

using namespace hps;

extern "C" hps_status hps_average_on_noalloc(const hps_channel* channel, uint64_t first_evt, uint64_t n,
                                             const hps_functor* functor, hps_stats* out, int32_t precision,
                                             void* stream)
{
    HPS_ENTRY();
    DevChannel ch;
    DevFunctor fn;
    hps_status st = average_args(channel, functor, precision, &ch, &fn);
    if (st != HPS_OK) return st;
    if (!out) return set_error(HPS_ERR_BAD_ARG, "out is NULL");
    if (!aligned(out, 8)) return set_error(HPS_ERR_BAD_ARG, "out not 8-byte aligned");
    if (!range_ok(first_evt, n)) return set_error(HPS_ERR_BAD_ARG, "event range wraps 2^64");
    if (n > HPS_NOALLOC_MAX_EVENTS)
        return set_error(HPS_ERR_BAD_ARG,
                         "hps_average_on_noalloc: n = %llu events exceeds the allocation-free limit of %llu "
                         "(HPS_NOALLOC_MAX_EVENTS); split the range or use hps_average_on",
                         static_cast<unsigned long long>(n),
                         static_cast<unsigned long long>(HPS_NOALLOC_MAX_EVENTS));
    hps_stats* partials = nullptr;
    if ((st = noalloc_scratch(&partials)) != HPS_OK) return st;
    // Every partial the merge reads (tiles 0 .. ceil(n/HPS_AVG_TILE)-1) is written earlier on the
    // same stream by this call, so no part of the shared array needs clearing first.
    return launch_average(channel, ch, fn, first_evt, n, out, partials, precision, as_stream(stream));
}
