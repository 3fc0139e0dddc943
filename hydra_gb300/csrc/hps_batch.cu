// hps_batch.cu -- many channels of different N in one CUDA-graph launch of persistent kernels.
//
// The items of a plan are cut into work units: a store item into units of store_tile events,
// an AverageOn item into tiles of HPS_AVG_TILE events.  Items are grouped by register class: one
// persistent kernel per (N, form, mode), so a class runs at the occupancy its own register count
// allows (one kernel over every N would hold every channel to the registers of N = 10, and one
// kernel for both modes would hold the store path to the registers of the AverageOn tile).  The
// class kernels run as parallel branches of the graph, so the SMs one class frees at its end take
// CTAs of the others.  A class kernel's 256-thread CTAs take units from the class's device
// counter; each unit dispatches on (N, engine) to the same work-unit functions the single-channel
// FP32_FIX kernels use (tiles_f32.cuh), so an item's outputs do not depend on what else is in the
// batch.  A last kernel merges each AverageOn item's tile partials with the fixed tree of
// hps_average_on.  Counter reset, class kernels and merge are built once into a CUDA graph; the
// item table and its header live in device memory, so new items need no new graph, and each
// class kernel's grid is set from its unit count when the items change (a class with no units
// launches one CTA).
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>
#include <fstream>
#include <sstream>

#include "common.h"
#include "store.cuh"
#include "tiles_f32.cuh"

namespace hps {

struct BatchItemDev {
    DevChannel chd;
    DevChannelF chf;
    DevFunctor fn;
    Cols cols;
    double* weights;
    uint8_t* flags;
    hps_stats* stats;
    uint64_t first, n, ukey;
    uint64_t unit_begin;       // first global work unit of this item
    uint64_t partial_offset;   // AverageOn: offset of its tile partials
    uint64_t units;            // work units of this item
    int32_t mode, N, engine, vec32;
};

// Register classes of the store items: one per N (class c < 9 holds N = c + 2), and for N = 4..6
// one more each for the channels that take the float-float boosts (classes 9..11: N = c - 5),
// which need more registers than the plain form of the same N.  With threads_per_event = 2, the
// store items of N = 7..10 go to classes 12..15 (N = c - 5), whose kernels run two threads per
// event (store_chunk_split_f32).  Half of the daughters per thread does not lower the register
// count much: the event's random words (3N - 4 64-bit values), the stage momenta and the
// float-float weight are held by both threads; ptxas gives the split classes 128 registers, and a
// 3-CTA bound (80 registers) spills 72 to 296 bytes per thread.  The AverageOn items take classes
// 16..27: class 16 + c holds the AverageOn items of store class c < 12.  Each class kernel carries
// both engines of its N and one mode.
constexpr int kBatchClasses = 28;
constexpr int kAvgClass0 = 16;
__host__ __device__ constexpr int class_n(int c)
{
    return c >= kAvgClass0 ? class_n(c - kAvgClass0) : c < 9 ? c + 2 : c - 5;
}
__host__ __device__ constexpr bool class_ff(int c)
{
    return c >= kAvgClass0 ? class_ff(c - kAvgClass0) : (c >= 9 && c < 12);
}
__host__ __device__ constexpr bool class_split(int c) { return c >= 12 && c < kAvgClass0; }
__host__ __device__ constexpr bool class_avg(int c) { return c >= kAvgClass0; }
constexpr int kSplitMinN = 7;
inline bool ff_class_n(int N) { return N >= f32::kHardMinN && N < f32::kPreciseN; }
inline int batch_class(int N, bool ff, int mode, bool split = false)
{
    const int base = N < 2 ? 0 : N > 10 ? 8 : (ff && ff_class_n(N)) ? N + 5 : N - 2;
    if (mode == HPS_MODE_AVERAGE) return kAvgClass0 + base;
    if (split && N >= kSplitMinN && N <= 10) return N + 5;
    return base;
}
// The engine field of a table entry: the engine, with kPreciseForm for the float-float classes.
inline int item_engine(int N, int engine, bool ff) { return engine | ((ff && ff_class_n(N)) ? kPreciseForm : 0); }

struct BatchHeader {
    // next unit of each class, relative; the last one serves the single kernel over every N
    // (reset per launch)
    unsigned long long counter[kBatchClasses + 1];
    uint64_t class_begin[kBatchClasses + 1];     // the units of class c are [class_begin[c], class_begin[c+1])
    int32_t item_begin[kBatchClasses + 1];       // its items are table entries [item_begin[c], item_begin[c+1])
    int32_t n_items;
    int32_t store_tile;
};

// Store loop of the per-class kernels: two events per thread, one after the other, from one
// exchange of the random words of two chunks (store_pair_seq_f32), except for N = 8 and 9, which
// take one chunk per exchange, as the single-channel store kernel does.  On the 256-channel batch
// (ms, store only / mixed): one chunk per exchange for every N 2.488 / 2.494; the single-channel
// kernel's forms (N <= 4 with the two events interleaved) 2.454 / 2.484; this 2.441 / 2.473.  The
// single-channel kernel's 128-thread CTAs for N <= 6 (8 per SM at 64 registers) measured 2.443 /
// 2.478 against 2.442 / 2.467 with 256, so every class runs 256-thread CTAs.
__host__ __device__ constexpr bool batch_store_paired(int N) { return N != 8 && N != 9; }

// One work unit of an item.  MODE_ONLY >= 0 compiles the path of that mode alone (the per-class
// kernels); -1 compiles both and dispatches on the item (the single kernel over every N, whose
// store loop takes one chunk per exchange).
template <int N, int ENGINE, bool SPLIT = false, int MODE_ONLY = -1>
__device__ __forceinline__ void run_unit(const BatchItemDev& it, uint64_t u, int store_tile, hps_stats* partials,
                                         void* smem)
{
    if (MODE_ONLY == HPS_MODE_AVERAGE || (MODE_ONLY < 0 && it.mode != HPS_MODE_STORE)) {
        if constexpr (!SPLIT && MODE_ONLY != HPS_MODE_STORE) {
            const float K0 = *reinterpret_cast<const float*>(it.stats);      // written by k_batch_shift
            const hps_sums r = average_tile_f32<N, ENGINE>(it.chd, it.chf, it.fn, it.first, it.n, u, K0, smem);
            if (threadIdx.x == 0) reinterpret_cast<hps_sums*>(partials)[it.partial_offset + u] = r;
        }
    } else if constexpr (MODE_ONLY != HPS_MODE_AVERAGE) {
        const uint64_t lo = u * (uint64_t)store_tile;
        const uint64_t hi = (lo + store_tile < it.n) ? lo + store_tile : it.n;
        // the unit fetch ends with a __syncthreads, so each unit may start at parity 0
        int parity = 0;
        if constexpr (SPLIT) {
            for (uint64_t cb = lo; cb < hi; cb += kTileThreads / 2, parity ^= 1)
                store_chunk_split_f32<N, ENGINE>(it.chd, it.chf, it.cols, it.weights, it.flags, it.ukey, it.first, hi,
                                                 cb, it.vec32 != 0, smem, parity);
        } else if constexpr (MODE_ONLY == HPS_MODE_STORE && batch_store_paired(N)) {
            for (uint64_t cb = lo; cb < hi; cb += 2 * kTileThreads, parity ^= 1)
                store_pair_seq_f32<N, ENGINE, kTileThreads>(it.chd, it.chf, it.cols, it.weights, it.flags, it.ukey,
                                                            it.first, hi, cb, it.vec32 != 0, smem, parity);
        } else {
            for (uint64_t cb = lo; cb < hi; cb += kTileThreads, parity ^= 1)
                store_chunk_f32<N, ENGINE>(it.chd, it.chf, it.cols, it.weights, it.flags, it.ukey, it.first, hi, cb,
                                           it.vec32 != 0, smem, parity);
        }
    }
}

template <int CLS>
__device__ __forceinline__ void batch_body(const BatchItemDev* __restrict__ items, BatchHeader* __restrict__ hdr,
                                           hps_stats* __restrict__ partials)
{
    // largest shared-memory word exchange of the class (Philox; two chunks at a time in the paired
    // store loops)
    constexpr bool kPairedStore = !class_avg(CLS) && !class_split(CLS) && batch_store_paired(class_n(CLS));
    __shared__ __align__(16) unsigned char
        smem[kPairedStore ? PairedSmem<class_n(CLS), kPhilox>::BYTES : WordShare<class_n(CLS), kPhilox, kTileThreads>::BYTES2];
    __shared__ unsigned long long s_unit;
    __shared__ int s_item;
    // The unit's item, staged in shared memory: the channel constants are then re-read after the
    // barriers of each 256-event chunk instead of being held in registers for the whole unit,
    // which keeps the class kernels near the register counts of the single-channel kernels.
    __shared__ __align__(16) BatchItemDev s_it;
    static_assert(sizeof(BatchItemDev) % 8 == 0, "staged as 8-byte words");
    const uint64_t unit_end = hdr->class_begin[CLS + 1];
    const uint64_t unit_begin = hdr->class_begin[CLS];
    const int item_lo = hdr->item_begin[CLS];
    const int item_hi = hdr->item_begin[CLS + 1] - 1;
    const int store_tile = hdr->store_tile;
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned long long u = unit_begin + atomicAdd(&hdr->counter[CLS], 1ull);
            int lo = item_lo, hi = item_hi;               // last item of the class with unit_begin <= u
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (items[mid].unit_begin <= u) lo = mid; else hi = mid - 1;
            }
            s_unit = u;
            s_item = lo;
        }
        __syncthreads();
        const unsigned long long u = s_unit;
        const int item = s_item;
        if (u >= unit_end) return;                        // the whole CTA (also every class with no items)
        {
            const uint2* src = reinterpret_cast<const uint2*>(items + item);
            uint2* dst = reinterpret_cast<uint2*>(&s_it);
            for (int k = threadIdx.x; k < (int)(sizeof(BatchItemDev) / 8); k += kTileThreads) dst[k] = src[k];
        }
        __syncthreads();                                  // s_it staged; s_unit / s_item read before they change
        const BatchItemDev& it = s_it;
        const uint64_t lu = u - it.unit_begin;
        constexpr int MODE = class_avg(CLS) ? HPS_MODE_AVERAGE : HPS_MODE_STORE;
        constexpr bool SPL = class_split(CLS);
        switch (it.N * 8 + it.engine) {
#define HPS_UNIT(NN)                                                                             \
        case NN * 8 + 0:                                                                         \
            if constexpr (NN == class_n(CLS) && !class_ff(CLS))                                  \
                run_unit<NN, kPhilox, SPL, MODE>(it, lu, store_tile, partials, smem);            \
            break;                                                                               \
        case NN * 8 + 1:                                                                         \
            if constexpr (NN == class_n(CLS) && !class_ff(CLS))                                  \
                run_unit<NN, kSquares3, SPL, MODE>(it, lu, store_tile, partials, smem);          \
            break;                                                                               \
        case NN * 8 + kPreciseForm:                                                              \
            if constexpr (NN == class_n(CLS) && class_ff(CLS))                                   \
                run_unit<NN, kPhilox | kPreciseForm, false, MODE>(it, lu, store_tile, partials, smem);   \
            break;                                                                               \
        case NN * 8 + (kSquares3 | kPreciseForm):                                                \
            if constexpr (NN == class_n(CLS) && class_ff(CLS))                                   \
                run_unit<NN, kSquares3 | kPreciseForm, false, MODE>(it, lu, store_tile, partials, smem); \
            break;
        HPS_UNIT(2) HPS_UNIT(3) HPS_UNIT(4) HPS_UNIT(5) HPS_UNIT(6) HPS_UNIT(7) HPS_UNIT(8) HPS_UNIT(9)
        HPS_UNIT(10)
#undef HPS_UNIT
        default: break;
        }
    }
}

// Resident CTAs per SM the register allocation of a class kernel must allow (second argument of
// __launch_bounds__; 0 leaves the choice to the compiler).  The classes of N >= 7 (both modes) are
// held to 128 registers (2 CTAs per SM), the store classes of N <= 6 to 64 (4 CTAs per SM; the
// compiler gives them up to 98: the unit loop and the staged item add to the event body's).
// Measured on the 256-channel batch (autotuned, ms; store only / every other channel an AverageOn
// item): one kernel per N for both modes 2.564 / 2.700; one per N and mode with the store classes
// of N >= 7 at the single-channel store kernel's bounds (64, 80, 80, 128 registers for N = 7..10;
// they spill 144 to 248 bytes here) 2.558 / 2.537; one per N and mode at 128 registers for N >= 7
// 2.537 / 2.516; and with the store classes of N <= 6 at 64 registers 2.486 / 2.494 (at 48
// registers, spilling up to 112 bytes, 2.517 / 2.522).  The AverageOn classes of N <= 6 keep the
// compiler's 59..80 registers: at 64 registers the mixed batch and an AverageOn-only batch of the
// same channels measured 2.461 / 2.303 ms against 2.472 / 2.297, and 2.461 / 2.310 with paired
// tiles for N = 3..5.  When one kernel carried both modes, holding N >= 7 to 128 registers had
// taken the batch from 2.776 to 2.612 ms.
__host__ __device__ constexpr int batch_min_ctas(int c)
{
    return (!class_split(c) && class_n(c) >= 7) ? 2 : (!class_avg(c) && !class_split(c)) ? 4 : 0;
}

template <int CLS>
__global__ void __launch_bounds__(kTileThreads, batch_min_ctas(CLS))
k_batch_f32(const BatchItemDev* __restrict__ items, BatchHeader* __restrict__ hdr, hps_stats* __restrict__ partials)
{
    batch_body<CLS>(items, hdr, partials);
}



// The single-kernel form (hps_batch_tuning.kernel_form = HPS_BATCH_ONE_KERNEL): one persistent
// kernel takes every unit of every N from one counter and dispatches on N, reading the item from
// global memory.  Its register count is that of the largest N for all of them.
__global__ void __launch_bounds__(kTileThreads)
k_batch_f32_all(const BatchItemDev* __restrict__ items, BatchHeader* __restrict__ hdr,
                hps_stats* __restrict__ partials)
{
    __shared__ __align__(16) unsigned char smem[WordShare<10, kPhilox, kTileThreads>::BYTES2];
    __shared__ unsigned long long s_unit;
    __shared__ int s_item;
    const uint64_t total = hdr->class_begin[kBatchClasses];
    const int n_items = hdr->n_items;
    const int store_tile = hdr->store_tile;
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned long long u = atomicAdd(&hdr->counter[kBatchClasses], 1ull);
            int lo = 0, hi = n_items - 1;                 // last item with unit_begin <= u
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (items[mid].unit_begin <= u) lo = mid; else hi = mid - 1;
            }
            s_unit = u;
            s_item = lo;
        }
        __syncthreads();
        const unsigned long long u = s_unit;
        const int item = s_item;
        __syncthreads();                                  // s_unit / s_item read before they change
        if (u >= total) return;
        const BatchItemDev& it = items[item];
        const uint64_t lu = u - it.unit_begin;
        switch (it.N * 8 + it.engine) {
#define HPS_UNIT(NN)                                                                         \
        case NN * 8 + 0: run_unit<NN, kPhilox>(it, lu, store_tile, partials, smem); break;   \
        case NN * 8 + 1: run_unit<NN, kSquares3>(it, lu, store_tile, partials, smem); break;
#define HPS_UNIT_FF(NN)                                                                      \
        HPS_UNIT(NN)                                                                         \
        case NN * 8 + 4: run_unit<NN, kPhilox | kPreciseForm>(it, lu, store_tile, partials, smem); break; \
        case NN * 8 + 5: run_unit<NN, kSquares3 | kPreciseForm>(it, lu, store_tile, partials, smem); break;
        HPS_UNIT(2) HPS_UNIT(3) HPS_UNIT_FF(4) HPS_UNIT_FF(5) HPS_UNIT_FF(6) HPS_UNIT(7) HPS_UNIT(8) HPS_UNIT(9)
        HPS_UNIT(10)
#undef HPS_UNIT_FF
#undef HPS_UNIT
        default: break;
        }
    }
}

// One CTA per item slot: the shift K0 of each AverageOn item into the first 4 bytes of its stats
// output, as k_shift_f32 does for hps_average_on.
__global__ void k_batch_shift(const BatchItemDev* __restrict__ items, const BatchHeader* __restrict__ hdr)
{
    if ((int)blockIdx.x >= hdr->n_items || threadIdx.x != 0) return;
    const BatchItemDev& it = items[blockIdx.x];
    if (it.mode != HPS_MODE_AVERAGE || it.n == 0) return;
    float K0 = 0.0f;
    switch (it.N * 8 + it.engine) {
#define HPS_SHIFT(NN)                                                                          \
    case NN * 8 + 0: K0 = call_shift<NN, kPhilox>(it.chd, it.chf, it.fn, it.first); break;     \
    case NN * 8 + 1: K0 = call_shift<NN, kSquares3>(it.chd, it.chf, it.fn, it.first); break;
#define HPS_SHIFT_FF(NN)                                                                                  \
    HPS_SHIFT(NN)                                                                                         \
    case NN * 8 + 4: K0 = call_shift<NN, kPhilox | kPreciseForm>(it.chd, it.chf, it.fn, it.first); break;  \
    case NN * 8 + 5: K0 = call_shift<NN, kSquares3 | kPreciseForm>(it.chd, it.chf, it.fn, it.first); break;
    HPS_SHIFT(2) HPS_SHIFT(3) HPS_SHIFT_FF(4) HPS_SHIFT_FF(5) HPS_SHIFT_FF(6) HPS_SHIFT(7) HPS_SHIFT(8) HPS_SHIFT(9)
    HPS_SHIFT(10)
#undef HPS_SHIFT_FF
#undef HPS_SHIFT
    default: break;
    }
    *reinterpret_cast<float*>(it.stats) = K0;
}

// One CTA per item slot: AverageOn items add their tile sums exactly as hps_average_on does.
__global__ void __launch_bounds__(kFinalThreads)
k_batch_merge(const BatchItemDev* __restrict__ items, const BatchHeader* __restrict__ hdr,
              const hps_stats* __restrict__ partials)
{
    if ((int)blockIdx.x >= hdr->n_items) return;
    const BatchItemDev& it = items[blockIdx.x];
    if (it.mode != HPS_MODE_AVERAGE) return;
    // every thread reads K0 before the block reduction's barriers; thread 0 writes the stats after them
    const float K0 = it.units ? *reinterpret_cast<const float*>(it.stats) : 0.0f;
    hps_stats r{0.0, 0.0, 0.0};
    switch (it.N * 8 + engine_of(it.engine)) {     // the merge does not depend on the form
#define HPS_MERGE(NN)                                                                                        \
    case NN * 8 + 0: r = merge_sums<NN, kPhilox>(it.chd, it.chf, it.fn, it.first, partials + it.partial_offset,  \
                                                 it.units, K0); break;                                        \
    case NN * 8 + 1: r = merge_sums<NN, kSquares3>(it.chd, it.chf, it.fn, it.first,                            \
                                                   partials + it.partial_offset, it.units, K0); break;
    HPS_MERGE(2) HPS_MERGE(3) HPS_MERGE(4) HPS_MERGE(5) HPS_MERGE(6) HPS_MERGE(7) HPS_MERGE(8) HPS_MERGE(9)
    HPS_MERGE(10)
#undef HPS_MERGE
    default: break;
    }
    if (threadIdx.x == 0) *it.stats = r;
}

typedef void (*BatchKernel)(const BatchItemDev*, BatchHeader*, hps_stats*);

inline BatchKernel class_kernel(int c)
{
    static const BatchKernel k[kBatchClasses] = {
        k_batch_f32<0>,  k_batch_f32<1>,  k_batch_f32<2>,  k_batch_f32<3>,  k_batch_f32<4>,  k_batch_f32<5>,
        k_batch_f32<6>,  k_batch_f32<7>,  k_batch_f32<8>,  k_batch_f32<9>,  k_batch_f32<10>, k_batch_f32<11>,
        k_batch_f32<12>, k_batch_f32<13>, k_batch_f32<14>, k_batch_f32<15>, k_batch_f32<16>, k_batch_f32<17>,
        k_batch_f32<18>, k_batch_f32<19>, k_batch_f32<20>, k_batch_f32<21>, k_batch_f32<22>, k_batch_f32<23>,
        k_batch_f32<24>, k_batch_f32<25>, k_batch_f32<26>, k_batch_f32<27>};
    return k[c];
}

}  // namespace hps

using namespace hps;

struct hps_batch_plan {
    int device = 0;
    int sm_count = 0;
    int32_t max_items = 0;
    uint64_t max_avg_tiles = 0;
    int32_t precision = HPS_PREC_FP32_FIX;
    hps_batch_tuning tuning{16, 4096, HPS_BATCH_PER_N, 1};   // every kernel at the CTAs that fit; short units
    BatchItemDev* d_items = nullptr;
    BatchHeader* d_header = nullptr;
    hps_stats* d_partials = nullptr;
    BatchItemDev* h_items = nullptr;   // pinned staging
    BatchHeader* h_header = nullptr;   // pinned staging
    cudaEvent_t staged = nullptr;      // staging copy finished
    bool staged_pending = false;
    int32_t n_items = 0;
    std::vector<hps_batch_item> items;  // host copy, re-cut when the store tile changes
    uint64_t total_events = 0;
    std::vector<int> mix;              // item mix signature for the tuning cache
    cudaStream_t own = nullptr;                  // the plan's stream for re-cutting the table
    int occupancy[kBatchClasses + 1] = {};       // resident CTAs per SM of each class kernel, then of
                                                 // the single kernel over every N
    uint64_t class_units[kBatchClasses] = {};    // work units of each class in the current table
    unsigned class_grid_set[kBatchClasses] = {};  // grid of each class kernel node in exec
    cudaGraph_t graph = nullptr;                 // kept while exec lives: its class kernel nodes are
    cudaGraphNode_t class_node[kBatchClasses] = {};   // re-gridded when the table changes
    cudaGraphExec_t exec = nullptr;
};

namespace {

hps_status destroy_graph(hps_batch_plan* p)
{
    cudaError_t e = cudaSuccess;
    if (p->exec) {
        e = cudaGraphExecDestroy(p->exec);
        p->exec = nullptr;
    }
    if (p->graph) {
        const cudaError_t e2 = cudaGraphDestroy(p->graph);
        p->graph = nullptr;
        if (e == cudaSuccess) e = e2;
    }
    for (int c = 0; c < kBatchClasses; ++c) p->class_node[c] = nullptr;
    return e == cudaSuccess ? HPS_OK : cuda_status(e, "destroy batch graph");
}

// Grid of class kernel c: the tuning's CTAs per SM within the kernel's occupancy, no more CTAs than
// the class has units (each CTA takes units from the class counter), and one CTA for an empty class.
unsigned class_grid(const hps_batch_plan* p, int c)
{
    const int ctas = p->tuning.ctas_per_sm < p->occupancy[c] ? p->tuning.ctas_per_sm : p->occupancy[c];
    const uint64_t full = static_cast<uint64_t>(ctas > 0 ? ctas : 1) * static_cast<uint64_t>(p->sm_count);
    const uint64_t units = p->class_units[c];
    return static_cast<unsigned>(units == 0 ? 1 : units < full ? units : full);
}

// Kernel node parameters of one launch of the plan's kernels (all take items, header, partials).
cudaKernelNodeParams kernel_params(void* func, unsigned grid, unsigned block, void** args)
{
    cudaKernelNodeParams kp;
    std::memset(&kp, 0, sizeof(kp));
    kp.func = func;
    kp.gridDim = dim3(grid, 1, 1);
    kp.blockDim = dim3(block, 1, 1);
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    kp.extra = nullptr;
    return kp;
}

// Sets the grid of each class kernel node of the instantiated graph whose unit count changed the
// grid (takes effect from the next launch; a launch in flight keeps its grids).  A graph of the
// single kernel over every N has no class nodes; a change of kernel form builds a new graph.  The
// grids shape the launch only: the CTAs of a class loop on its unit counter, so any grid of one
// CTA or more covers every unit, and a failed update leaves a correct (if slower) graph.
hps_status apply_class_grids(hps_batch_plan* p)
{
    if (!p->exec) return HPS_OK;
    for (int c = 0; c < kBatchClasses; ++c) {
        if (!p->class_node[c]) continue;
        const unsigned g = class_grid(p, c);
        if (g == p->class_grid_set[c]) continue;
        void* args[3] = {&p->d_items, &p->d_header, &p->d_partials};
        const cudaKernelNodeParams kp = kernel_params(reinterpret_cast<void*>(class_kernel(c)), g, kTileThreads, args);
        const cudaError_t e = cudaGraphExecKernelNodeSetParams(p->exec, p->class_node[c], &kp);
        if (e != cudaSuccess) return cuda_status(e, "cudaGraphExecKernelNodeSetParams");
        p->class_grid_set[c] = g;
    }
    return HPS_OK;
}

// The graph, built node by node: counter reset -> K0 shifts -> the class kernels (parallel
// branches) or the single kernel -> per-item merge.
hps_status build_graph(hps_batch_plan* p)
{
    hps_status st = destroy_graph(p);
    if (st != HPS_OK) return st;
    void* args[3] = {&p->d_items, &p->d_header, &p->d_partials};
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaGraphCreate(&graph, 0);
    if (e != cudaSuccess) return cuda_status(e, "cudaGraphCreate");
    cudaGraphNode_t reset = nullptr, shift = nullptr, merge = nullptr;
    std::vector<cudaGraphNode_t> work;
    {
        cudaMemsetParams mp;
        std::memset(&mp, 0, sizeof(mp));
        mp.dst = p->d_header->counter;
        mp.value = 0;
        mp.elementSize = 4;
        mp.width = sizeof(p->d_header->counter) / 4;
        mp.height = 1;
        mp.pitch = 0;
        e = cudaGraphAddMemsetNode(&reset, graph, nullptr, 0, &mp);
    }
    if (e == cudaSuccess) {
        const cudaKernelNodeParams kp =
            kernel_params(reinterpret_cast<void*>(k_batch_shift), static_cast<unsigned>(p->max_items), 32, args);
        e = cudaGraphAddKernelNode(&shift, graph, &reset, 1, &kp);
    }
    if (e == cudaSuccess && p->tuning.kernel_form == HPS_BATCH_ONE_KERNEL) {
        const int ctas = p->tuning.ctas_per_sm < p->occupancy[kBatchClasses] ? p->tuning.ctas_per_sm
                                                                              : p->occupancy[kBatchClasses];
        const cudaKernelNodeParams kp = kernel_params(reinterpret_cast<void*>(k_batch_f32_all),
                                                      static_cast<unsigned>((ctas > 0 ? ctas : 1) * p->sm_count),
                                                      kTileThreads, args);
        cudaGraphNode_t n = nullptr;
        e = cudaGraphAddKernelNode(&n, graph, &shift, 1, &kp);
        work.push_back(n);
    } else if (e == cudaSuccess) {
        for (int c = 0; c < kBatchClasses && e == cudaSuccess; ++c) {
            p->class_grid_set[c] = class_grid(p, c);
            const cudaKernelNodeParams kp =
                kernel_params(reinterpret_cast<void*>(class_kernel(c)), p->class_grid_set[c], kTileThreads, args);
            e = cudaGraphAddKernelNode(&p->class_node[c], graph, &shift, 1, &kp);
            work.push_back(p->class_node[c]);
        }
    }
    if (e == cudaSuccess) {
        const cudaKernelNodeParams kp = kernel_params(reinterpret_cast<void*>(k_batch_merge),
                                                      static_cast<unsigned>(p->max_items), kFinalThreads, args);
        e = cudaGraphAddKernelNode(&merge, graph, work.data(), work.size(), &kp);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&p->exec, graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        for (int c = 0; c < kBatchClasses; ++c) p->class_node[c] = nullptr;
        p->exec = nullptr;
        return cuda_status(e, "batch graph");
    }
    p->graph = graph;
    return HPS_OK;
}

hps_status check_tuning(const hps_batch_tuning* t)
{
    if (t->ctas_per_sm < 1 || t->ctas_per_sm > 16)
        return set_error(HPS_ERR_BAD_ARG, "ctas_per_sm %d outside 1..16", t->ctas_per_sm);
    if (t->store_tile_events < kTileThreads || t->store_tile_events % kTileThreads != 0 ||
        t->store_tile_events > (1 << 24))
        return set_error(HPS_ERR_BAD_ARG, "store_tile_events %d not a multiple of 256 in 256..2^24",
                         t->store_tile_events);
    if (t->kernel_form != HPS_BATCH_PER_N && t->kernel_form != HPS_BATCH_ONE_KERNEL)
        return set_error(HPS_ERR_BAD_ARG, "kernel_form %d is neither HPS_BATCH_PER_N nor HPS_BATCH_ONE_KERNEL",
                         t->kernel_form);
    if (t->threads_per_event < 0 || t->threads_per_event > 2)       // 0 reads as 1
        return set_error(HPS_ERR_BAD_ARG, "threads_per_event %d is neither 1 nor 2", t->threads_per_event);
    if (t->threads_per_event == 2 && t->kernel_form != HPS_BATCH_PER_N)
        return set_error(HPS_ERR_BAD_ARG, "threads_per_event 2 needs kernel_form HPS_BATCH_PER_N");
    return HPS_OK;
}

std::string tuning_key(const hps_batch_plan* p)
{
    cudaDeviceProp prop;
    std::ostringstream os;
    if (cudaGetDeviceProperties(&prop, p->device) == cudaSuccess) {
        std::string name(prop.name);
        for (char& c : name) if (c == ' ') c = '_';
        os << name;
    } else {
        os << "gpu";
    }
    os << "|p" << p->precision << "|";
    for (int v : p->mix) os << v << ",";
    return os.str();
}

hps_status item_error(hps_status st, int i)
{
    char msg[400];
    std::snprintf(msg, sizeof(msg), "%s", hps_last_error());
    return set_error(st, "item %d: %s", i, msg);
}

// Validates items, cuts them into work units with the plan's store tile, fills the pinned
// staging table and uploads it on `s`.
hps_status upload_items(hps_batch_plan* p, const std::vector<hps_batch_item>& items, cudaStream_t s)
{
    // the staging copy of the previous upload must have left the pinned buffer
    if (p->staged_pending) {
        cudaError_t e = cudaEventSynchronize(p->staged);
        if (e != cudaSuccess) return cuda_status(e, "cudaEventSynchronize");
        p->staged_pending = false;
    }
    const int n_items = static_cast<int>(items.size());
    // table order: by register class of N, input order within a class (an N outside 2..10 is
    // rejected below, wherever it sorts)
    std::vector<int> order(n_items);
    int32_t item_begin[kBatchClasses + 1] = {};
    const bool split = p->tuning.threads_per_event == 2;
    auto cls = [&](int i) {
        return batch_class(items[i].channel.n_daughters, float_float_form(&items[i].channel), items[i].mode,
                           split && items[i].mode == HPS_MODE_STORE);
    };
    for (int i = 0; i < n_items; ++i) ++item_begin[cls(i) + 1];
    for (int c = 0; c < kBatchClasses; ++c) item_begin[c + 1] += item_begin[c];
    {
        int32_t next[kBatchClasses];
        for (int c = 0; c < kBatchClasses; ++c) next[c] = item_begin[c];
        for (int i = 0; i < n_items; ++i) order[next[cls(i)]++] = i;
    }
    uint64_t class_begin[kBatchClasses + 1] = {};
    uint64_t unit = 0, partial = 0, events = 0;
    std::vector<int> mix(2 * 11 * 8, 0);
    for (int pos = 0, c = 0; pos < n_items; ++pos) {
        while (c < kBatchClasses && pos == item_begin[c + 1]) class_begin[++c] = unit;
        const int i = order[pos];
        const hps_batch_item& in = items[i];
        BatchItemDev& d = p->h_items[pos];
        std::memset(&d, 0, sizeof(d));
        hps_status st = to_device_channel(&in.channel, &d.chd);
        if (st != HPS_OK) return item_error(st, i);
        to_device_channel_f(&in.channel, &d.chf);
        if (!range_ok(in.first_evt, in.n_events)) return set_error(HPS_ERR_BAD_ARG, "item %d: event range wraps", i);
        const int N = in.channel.n_daughters;
        d.N = N;
        d.engine = item_engine(N, in.channel.engine, d.chf.precise != 0);
        d.mode = in.mode;
        d.first = in.first_evt;
        d.n = in.n_events;
        d.unit_begin = unit;
        if (in.mode == HPS_MODE_STORE) {
            bool all32 = true;
            for (int k = 0; k < N; ++k) {
                if (in.n_events && !in.cols[k]) return set_error(HPS_ERR_BAD_ARG, "item %d: column %d is NULL", i, k);
                if (!aligned(in.cols[k], 16)) return set_error(HPS_ERR_BAD_ARG, "item %d: column %d misaligned", i, k);
                all32 = all32 && aligned(in.cols[k], 32);
                d.cols.p[k] = in.cols[k];
            }
            if (in.weights && !aligned(in.weights, 8)) return set_error(HPS_ERR_BAD_ARG, "item %d: weights misaligned", i);
            d.vec32 = all32 ? 1 : 0;
            d.weights = in.weights;
            d.flags = in.flags;
            d.ukey = splitmix64(in.unweight_seed);
            d.units = (in.n_events + p->tuning.store_tile_events - 1) / p->tuning.store_tile_events;
        } else if (in.mode == HPS_MODE_AVERAGE) {
            st = to_device_functor(&in.functor, N, &d.fn);
            if (st != HPS_OK) return item_error(st, i);
            if (!in.stats || !aligned(in.stats, 8)) return set_error(HPS_ERR_BAD_ARG, "item %d: stats missing", i);
            d.stats = in.stats;
            d.units = (in.n_events + HPS_AVG_TILE - 1) / HPS_AVG_TILE;
            d.partial_offset = partial;
            partial += d.units;
            if (partial > p->max_avg_tiles)
                return set_error(HPS_ERR_BUDGET, "AverageOn tiles %llu exceed the plan's %llu",
                                 (unsigned long long)partial, (unsigned long long)p->max_avg_tiles);
        } else {
            return set_error(HPS_ERR_BAD_ARG, "item %d: unknown mode %d", i, in.mode);
        }
        unit += d.units;
        events += in.n_events;
        mix[(in.mode * 11 + N) * 8 + d.engine] += 1;
    }
    for (int c = 0; c < kBatchClasses; ++c) {
        // classes after the last item's (and every class of an empty table) end at the last unit
        if (item_begin[c + 1] == n_items) class_begin[c + 1] = unit;
        p->h_header->counter[c] = 0;
    }
    for (int c = 0; c <= kBatchClasses; ++c) {
        p->h_header->class_begin[c] = class_begin[c];
        p->h_header->item_begin[c] = item_begin[c];
    }
    for (int c = 0; c < kBatchClasses; ++c) p->class_units[c] = class_begin[c + 1] - class_begin[c];
    p->h_header->n_items = n_items;
    p->h_header->store_tile = p->tuning.store_tile_events;
    p->n_items = n_items;
    p->total_events = events;
    p->mix = mix;
    p->mix.push_back(events ? 63 - __builtin_clzll(events) : 0);   // log2 of the event count
    cudaError_t e = cudaSuccess;
    if (n_items) e = cudaMemcpyAsync(p->d_items, p->h_items, sizeof(BatchItemDev) * n_items, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p->d_header, p->h_header, sizeof(BatchHeader), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaEventRecord(p->staged, s);
    if (e != cudaSuccess) return cuda_status(e, "batch table upload");
    p->staged_pending = true;
    return apply_class_grids(p);
}

}  // namespace

extern "C" {

hps_status hps_batch_create(hps_batch_plan** out, int32_t max_items, uint64_t max_average_tiles, int32_t precision,
                            const hps_batch_tuning* tuning)
{
    HPS_ENTRY();
    if (!out) return set_error(HPS_ERR_BAD_ARG, "plan is NULL");
    *out = nullptr;
    if (max_items < 1 || max_items > (1 << 20)) return set_error(HPS_ERR_BAD_ARG, "max_items %d", max_items);
    if (precision != HPS_PREC_FP32_FIX)
        return set_error(HPS_ERR_UNSUPPORTED, "the batched kernel is built for HPS_PREC_FP32_FIX only");
    if (tuning) {
        hps_status st = check_tuning(tuning);
        if (st != HPS_OK) return st;
    }
    hps_batch_plan* p = new hps_batch_plan();
    p->max_items = max_items;
    p->max_avg_tiles = max_average_tiles ? max_average_tiles : 1;
    p->precision = precision;
    if (tuning) p->tuning = *tuning;
    cudaError_t e = cudaGetDevice(&p->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&p->sm_count, cudaDevAttrMultiProcessorCount, p->device);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_items, sizeof(BatchItemDev) * max_items);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_header, sizeof(BatchHeader));
    if (e == cudaSuccess) e = cudaMalloc(&p->d_partials, sizeof(hps_stats) * p->max_avg_tiles);
    if (e == cudaSuccess) e = cudaMallocHost(&p->h_items, sizeof(BatchItemDev) * max_items);
    if (e == cudaSuccess) e = cudaMallocHost(&p->h_header, sizeof(BatchHeader));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->staged, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->own, cudaStreamNonBlocking);
    for (int c = 0; c < kBatchClasses && e == cudaSuccess; ++c)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p->occupancy[c], class_kernel(c), kTileThreads, 0);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p->occupancy[kBatchClasses], k_batch_f32_all,
                                                          kTileThreads, 0);
    if (e == cudaSuccess) e = cudaMemset(p->d_header, 0, sizeof(BatchHeader));
    if (e != cudaSuccess) {
        hps_status st = (e == cudaErrorMemoryAllocation) ? set_error(HPS_ERR_OOM, "batch plan: %s", cudaGetErrorString(e))
                                                         : cuda_status(e, "batch plan");
        hps_batch_destroy(p);
        return st;
    }
    std::memset(p->h_header, 0, sizeof(BatchHeader));
    hps_status st = build_graph(p);
    if (st != HPS_OK) {
        hps_batch_destroy(p);
        return st;
    }
    *out = p;
    return HPS_OK;
}

hps_status hps_batch_set_items(hps_batch_plan* p, const hps_batch_item* items, int32_t n_items, void* stream)
{
    HPS_ENTRY();
    if (!p) return set_error(HPS_ERR_BAD_ARG, "plan is NULL");
    if (n_items < 0 || n_items > p->max_items)
        return set_error(HPS_ERR_BAD_ARG, "n_items %d outside 0..%d", n_items, p->max_items);
    if (n_items > 0 && !items) return set_error(HPS_ERR_BAD_ARG, "items is NULL");
    std::vector<hps_batch_item> copy(items, items + n_items);
    hps_status st = upload_items(p, copy, as_stream(stream));
    if (st == HPS_OK) p->items.swap(copy);
    return st;
}

hps_status hps_batch_launch(hps_batch_plan* p, void* stream)
{
    HPS_ENTRY();
    if (!p) return set_error(HPS_ERR_BAD_ARG, "plan is NULL");
    if (!p->exec) {
        hps_status st = build_graph(p);
        if (st != HPS_OK) return st;
    }
    return cuda_status(cudaGraphLaunch(p->exec, as_stream(stream)), "cudaGraphLaunch");
}

hps_status hps_batch_get_tuning(const hps_batch_plan* p, hps_batch_tuning* out)
{
    HPS_ENTRY();
    if (!p || !out) return set_error(HPS_ERR_BAD_ARG, "NULL argument");
    *out = p->tuning;
    return HPS_OK;
}

hps_status hps_batch_set_tuning(hps_batch_plan* p, const hps_batch_tuning* t)
{
    HPS_ENTRY();
    if (!p || !t) return set_error(HPS_ERR_BAD_ARG, "NULL argument");
    hps_status st = check_tuning(t);
    if (st != HPS_OK) return st;
    const bool tile_changed = t->store_tile_events != p->tuning.store_tile_events ||
                              t->threads_per_event != p->tuning.threads_per_event;
    p->tuning = *t;
    if (tile_changed && p->n_items > 0) {
        // re-cut the current items into the new store tile; done on the plan's own stream
        st = upload_items(p, p->items, p->own);
        if (st != HPS_OK) return st;
        cudaError_t e = cudaStreamSynchronize(p->own);
        if (e != cudaSuccess) return cuda_status(e, "cudaStreamSynchronize");
    }
    return build_graph(p);
}

hps_status hps_batch_autotune(hps_batch_plan* p, void* stream, const char* cache_path, hps_batch_tuning* chosen)
{
    HPS_ENTRY();
    if (!p) return set_error(HPS_ERR_BAD_ARG, "plan is NULL");
    if (p->n_items == 0) return set_error(HPS_ERR_BAD_ARG, "no items to tune on");
    static std::mutex cache_mu;
    const std::string key = tuning_key(p);
    if (cache_path) {
        std::lock_guard<std::mutex> lock(cache_mu);
        std::ifstream in(cache_path);
        std::string line;
        while (std::getline(in, line)) {
            std::istringstream ls(line);
            std::string k;
            hps_batch_tuning t;
            double ms;
            if ((ls >> k >> t.ctas_per_sm >> t.store_tile_events >> t.kernel_form >> t.threads_per_event >> ms) &&
                k == key &&
                check_tuning(&t) == HPS_OK) {
                hps_status st = hps_batch_set_tuning(p, &t);
                if (st == HPS_OK && chosen) *chosen = t;
                return st;
            }
        }
    }
    cudaStream_t s = as_stream(stream);
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int ctas[] = {1, 2, 3, 4, 6, 8};
    // 2048-event units pay where AverageOn items share the launch (the 256-channel batch with every
    // other channel an AverageOn item: 2.472 ms against 2.482 at 4096); store-only mixes keep 4096
    // (2.450 against 2.441), and 1024 is slower for both (2.497, 2.495)
    const int tiles[] = {2048, 4096, 16384, 65536};
    // threads per event 2 only where there are store items it applies to (N >= 7)
    bool any_split = false;
    for (const hps_batch_item& it : p->items)
        any_split = any_split || (it.mode == HPS_MODE_STORE && it.channel.n_daughters >= kSplitMinN);
    std::vector<hps_batch_tuning> cands;
    for (int form : {HPS_BATCH_PER_N, HPS_BATCH_ONE_KERNEL})
        for (int tile : tiles)
            for (int c : ctas)
                for (int tpe = 1; tpe <= ((any_split && form == HPS_BATCH_PER_N) ? 2 : 1); ++tpe)
                    cands.push_back(hps_batch_tuning{c, tile, form, tpe});
    hps_batch_tuning best = p->tuning;
    float best_ms = 1e30f;
    hps_status st = HPS_OK;
    for (const hps_batch_tuning& t : cands) {
        if ((st = hps_batch_set_tuning(p, &t)) != HPS_OK) break;
        if ((st = hps_batch_launch(p, stream)) != HPS_OK) break;       // warm-up
        cudaEventRecord(a, s);
        for (int r = 0; r < 3 && st == HPS_OK; ++r) st = hps_batch_launch(p, stream);
        cudaEventRecord(b, s);
        cudaError_t e = cudaEventSynchronize(b);
        if (e != cudaSuccess) { st = cuda_status(e, "autotune timing"); break; }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best_ms) { best_ms = ms; best = t; }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (st != HPS_OK) return st;
    st = hps_batch_set_tuning(p, &best);
    if (st != HPS_OK) return st;
    if (cache_path) {
        std::lock_guard<std::mutex> lock(cache_mu);
        std::ofstream outf(cache_path, std::ios::app);
        outf << key << " " << best.ctas_per_sm << " " << best.store_tile_events << " " << best.kernel_form << " "
             << best.threads_per_event << " "
             << best_ms / 3.0f << "\n";
    }
    if (chosen) *chosen = best;
    return HPS_OK;
}

hps_status hps_batch_destroy(hps_batch_plan* p)
{
    if (!p) return HPS_OK;
    destroy_graph(p);
    if (p->staged) { cudaEventSynchronize(p->staged); cudaEventDestroy(p->staged); }
    if (p->own) cudaStreamDestroy(p->own);
    if (p->d_items) cudaFree(p->d_items);
    if (p->d_header) cudaFree(p->d_header);
    if (p->d_partials) cudaFree(p->d_partials);
    if (p->h_items) cudaFreeHost(p->h_items);
    if (p->h_header) cudaFreeHost(p->h_header);
    delete p;
    return HPS_OK;
}

}  // extern "C"
