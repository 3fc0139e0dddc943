// common.h -- host-side helpers shared by the C-ABI translation units of libhps.so.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/hps.h"
#include "genbod.cuh"
#include "genbod_f32.cuh"

namespace hps {

// Per-thread message behind hps_last_error().
hps_status set_error(hps_status st, const char* fmt, ...);
void clear_error();

// Opening of every C-ABI call: clears the calling thread's error message and keeps an NVTX range
// named after the call open for its duration, so a profiler's timeline (Nsight Systems, Nsight
// Compute's NVTX filter) shows each library call around the kernels it launched.  Without a tool
// attached an NVTX push/pop is a test of a null function pointer.
struct EntryScope {
    explicit EntryScope(const char* name)
    {
        clear_error();
        nvtxRangePushA(name);
    }
    ~EntryScope() { nvtxRangePop(); }
    EntryScope(const EntryScope&) = delete;
    EntryScope& operator=(const EntryScope&) = delete;
};
#define HPS_ENTRY() const ::hps::EntryScope hps_entry_scope_(__func__)

inline hps_status cuda_status(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return HPS_OK;
    return set_error(HPS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Validates the channel and converts it to the kernel-side form.
hps_status to_device_channel(const hps_channel* ch, DevChannel* out);
hps_status to_device_functor(const hps_functor* f, int n_daughters, DevFunctor* out);
// Float-side constants for the FP32_FIX kernels (prefix sums formed in double, then rounded).
void to_device_channel_f(const hps_channel* ch, DevChannelF* out);
// Whether the FP32_FIX kernels take the float-float boosts for this channel (N at least
// f32::kPreciseN, or at least f32::kHardMinN with ECM >= f32::kHardRatio x the lightest mass).
bool float_float_form(const hps_channel* ch);

// AverageOn pieces shared by its entry points (hps_average.cu): host-side validation that
// touches no device state, and the tile + final-merge launches into caller-provided partials.
hps_status average_args(const hps_channel* channel, const hps_functor* functor, int32_t precision,
                        DevChannel* ch, DevFunctor* fn);
// With `so`, the tiles also store their events (hps_generate_average).
struct StoreOut;
hps_status launch_average(const hps_channel* channel, const DevChannel& ch, const DevFunctor& fn,
                          uint64_t first_evt, uint64_t n, hps_stats* out, hps_stats* partials,
                          int32_t precision, cudaStream_t stream, const StoreOut* so = nullptr);

// Stored events: N daughter columns of Vector4R (32 bytes per event, 16-byte aligned).
struct ConstCols { const double* p[HPS_MAX_DAUGHTERS]; };

template <int N>
__device__ __forceinline__ void load_event(const ConstCols& cols, uint64_t e, double (&p)[N][4])
{
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const double2 a = __ldg(reinterpret_cast<const double2*>(cols.p[k] + 4 * e));
        const double2 b = __ldg(reinterpret_cast<const double2*>(cols.p[k] + 4 * e) + 1);
        p[k][0] = a.x; p[k][1] = a.y; p[k][2] = b.x; p[k][3] = b.y;
    }
}

// Validates (n_daughters, masses, cols) of a stored sample; ch gets the masses and max_weight.
hps_status stored_event_args(int32_t n_daughters, const double* masses, uint64_t n, const double* const* cols,
                             ConstCols* cc, DevChannel* ch, double max_weight);

// Events [first, first + n) must not run past index 2^64 - 1.
inline bool range_ok(uint64_t first, uint64_t n) { return n == 0 || first + (n - 1) >= first; }

inline bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Grid for a one-thread-per-item kernel with a grid-stride loop: enough CTAs to fill
// the device several times over, never more than the work needs.
inline unsigned grid_for(uint64_t items, unsigned threads, unsigned max_ctas = 152u * 32u)
{
    const uint64_t need = (items + threads - 1) / threads;
    return static_cast<unsigned>(need < max_ctas ? (need == 0 ? 1 : need) : max_ctas);
}

// Instantiates BODY(N, ENGINE) for the runtime (n_daughters, engine) pair.
#define HPS_DISPATCH_N_ENGINE(n_daughters, engine, BODY)                         \
    switch ((n_daughters) * 2 + ((engine) == 0 ? 0 : 1)) {                      \
    case 4:  BODY(2, 0)  break; case 5:  BODY(2, 1)  break;                     \
    case 6:  BODY(3, 0)  break; case 7:  BODY(3, 1)  break;                     \
    case 8:  BODY(4, 0)  break; case 9:  BODY(4, 1)  break;                     \
    case 10: BODY(5, 0)  break; case 11: BODY(5, 1)  break;                     \
    case 12: BODY(6, 0)  break; case 13: BODY(6, 1)  break;                     \
    case 14: BODY(7, 0)  break; case 15: BODY(7, 1)  break;                     \
    case 16: BODY(8, 0)  break; case 17: BODY(8, 1)  break;                     \
    case 18: BODY(9, 0)  break; case 19: BODY(9, 1)  break;                     \
    case 20: BODY(10, 0) break; case 21: BODY(10, 1) break;                     \
    default: return set_error(HPS_ERR_BAD_ARG, "n_daughters %d outside 2..10", (int)(n_daughters)); \
    }

// The same for the FP32_FIX kernels: a channel whose float-side constants ask for the float-float
// boosts (DevChannelF::precise, N = 4..6; from N = 7 on they are always taken) gets the
// instantiation with kPreciseForm in its ENGINE parameter.
#define HPS_DISPATCH_F32(n_daughters, engine, precise, BODY)                    \
    switch ((n_daughters) * 2 + ((engine) == 0 ? 0 : 1)) {                      \
    case 4:  BODY(2, 0)  break; case 5:  BODY(2, 1)  break;                     \
    case 6:  BODY(3, 0)  break; case 7:  BODY(3, 1)  break;                     \
    case 8:  if (precise) { BODY(4, 4) } else { BODY(4, 0) } break;             \
    case 9:  if (precise) { BODY(4, 5) } else { BODY(4, 1) } break;             \
    case 10: if (precise) { BODY(5, 4) } else { BODY(5, 0) } break;             \
    case 11: if (precise) { BODY(5, 5) } else { BODY(5, 1) } break;             \
    case 12: if (precise) { BODY(6, 4) } else { BODY(6, 0) } break;             \
    case 13: if (precise) { BODY(6, 5) } else { BODY(6, 1) } break;             \
    case 14: BODY(7, 0)  break; case 15: BODY(7, 1)  break;                     \
    case 16: BODY(8, 0)  break; case 17: BODY(8, 1)  break;                     \
    case 18: BODY(9, 0)  break; case 19: BODY(9, 1)  break;                     \
    case 20: BODY(10, 0) break; case 21: BODY(10, 1) break;                     \
    default: return set_error(HPS_ERR_BAD_ARG, "n_daughters %d outside 2..10", (int)(n_daughters)); \
    }

#define HPS_DISPATCH_N(n_daughters, BODY)                                        \
    switch (n_daughters) {                                                      \
    case 2: BODY(2) break; case 3: BODY(3) break; case 4: BODY(4) break;        \
    case 5: BODY(5) break; case 6: BODY(6) break; case 7: BODY(7) break;        \
    case 8: BODY(8) break; case 9: BODY(9) break; case 10: BODY(10) break;      \
    default: return set_error(HPS_ERR_BAD_ARG, "n_daughters %d outside 2..10", (int)(n_daughters)); \
    }

}  // namespace hps
