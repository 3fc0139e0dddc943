// hps_compact.cu -- stable partition of stored events by their unweight flags.
//
// Decays::Unweight (hydra/detail/Decays.inl:415-455) tags each event with FlagDaugthers and calls
// thrust::stable_partition, which moves the accepted events to the front of the container, both
// groups keeping their order.  Here the partition is out of place: accepted events go to
// out[0, A) and rejected ones to out[A, n), in index order, A = number accepted.
//   pass 1  k_flag_counts : accepted count of each tile of 4096 events
//   pass 2  k_scan_counts : exclusive scan of the tile counts (one CTA), total A
//   pass 3  k_scatter     : each tile scans its flags 256 at a time (warp ballots) and copies
//                           every event (N Vector4R + weight) to its place
// Scratch: one uint64 per tile plus one, from the caller's workspace or the stream-ordered
// allocator.
#include "common.h"
#include "store.cuh"

namespace hps {

constexpr int kCompactThreads = 256;
constexpr int kCompactTile = 4096;

__global__ void __launch_bounds__(kCompactThreads)
k_flag_counts(const uint8_t* __restrict__ flags, uint64_t n, uint64_t ntiles, uint64_t* __restrict__ counts)
{
    __shared__ unsigned warp_sum[kCompactThreads / 32];
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        unsigned c = 0;
        for (int k = 0; k < kCompactTile / kCompactThreads; ++k) {
            const uint64_t e = t * kCompactTile + (uint64_t)k * kCompactThreads + threadIdx.x;
            if (e < n && flags[e]) ++c;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) c += __shfl_down_sync(0xffffffffu, c, off);
        if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = c;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned s = 0;
            for (int w = 0; w < kCompactThreads / 32; ++w) s += warp_sum[w];
            counts[t] = s;
        }
        __syncthreads();
    }
}

// One CTA of 1024 threads: thread j scans a contiguous block of tile counts; the block sums
// are scanned in shared memory; offsets[t] = accepted events before tile t, offsets[ntiles] = A.
__global__ void __launch_bounds__(1024)
k_scan_counts(uint64_t* __restrict__ counts, uint64_t ntiles, uint64_t* __restrict__ n_accepted)
{
    __shared__ uint64_t part[1024];
    const uint64_t per = (ntiles + 1023) / 1024;
    const uint64_t lo = threadIdx.x * per;
    const uint64_t hi = (lo + per < ntiles) ? lo + per : ntiles;
    uint64_t s = 0;
    for (uint64_t t = lo; t < hi; ++t) s += counts[t];
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t run = 0;
        for (int j = 0; j < 1024; ++j) {
            const uint64_t v = part[j];
            part[j] = run;
            run += v;
        }
        counts[ntiles] = run;
        if (n_accepted) *n_accepted = run;
    }
    __syncthreads();
    uint64_t run = part[threadIdx.x];
    for (uint64_t t = lo; t < hi; ++t) {
        const uint64_t v = counts[t];
        counts[t] = run;
        run += v;
    }
}

struct CompactCols {
    const double* in[HPS_MAX_DAUGHTERS];
    double* out[HPS_MAX_DAUGHTERS];
};

__global__ void __launch_bounds__(kCompactThreads)
k_scatter(CompactCols cols, int n_daughters, const double* __restrict__ w_in, double* __restrict__ w_out,
          const uint8_t* __restrict__ flags, uint64_t n, uint64_t ntiles, const uint64_t* __restrict__ offsets)
{
    __shared__ unsigned warp_acc[kCompactThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t total_acc = offsets[ntiles];
    for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        uint64_t acc_before = offsets[t];                       // accepted events before this chunk
        uint64_t rej_before = t * kCompactTile - offsets[t];    // rejected events before this chunk
        for (int k = 0; k < kCompactTile / kCompactThreads; ++k) {
            const uint64_t cb = t * kCompactTile + (uint64_t)k * kCompactThreads;
            if (cb >= n) break;                                 // CTA-uniform
            const uint64_t e = cb + threadIdx.x;
            const bool valid = e < n;
            const bool f = valid && flags[e] != 0;
            const unsigned ballot = __ballot_sync(0xffffffffu, f);
            if (lane == 0) warp_acc[warp] = __popc(ballot);
            __syncthreads();
            unsigned before_w = 0, chunk_acc = 0;
            for (int j = 0; j < kCompactThreads / 32; ++j) {
                const unsigned a = warp_acc[j];
                if (j < warp) before_w += a;
                chunk_acc += a;
            }
            const unsigned acc_rank = before_w + __popc(ballot & ((1u << lane) - 1u));
            const unsigned chunk_n = (n - cb < (uint64_t)kCompactThreads) ? (unsigned)(n - cb) : kCompactThreads;
            if (valid) {
                const unsigned rej_rank = threadIdx.x - acc_rank;
                const uint64_t dst = f ? acc_before + acc_rank : total_acc + rej_before + rej_rank;
                for (int d = 0; d < n_daughters; ++d) {
                    const double2* src = reinterpret_cast<const double2*>(cols.in[d] + 4 * e);
                    double2* out = reinterpret_cast<double2*>(cols.out[d] + 4 * dst);
                    out[0] = src[0];
                    out[1] = src[1];
                }
                if (w_in) w_out[dst] = w_in[e];
            }
            acc_before += chunk_acc;
            rej_before += chunk_n - chunk_acc;
            __syncthreads();
        }
    }
}

}  // namespace hps

using namespace hps;

extern "C" {

size_t hps_compact_workspace_size(uint64_t n)
{
    const uint64_t ntiles = (n + kCompactTile - 1) / kCompactTile;
    return static_cast<size_t>((ntiles + 1) * sizeof(uint64_t));
}

hps_status hps_unweight_compact(int32_t n_daughters, uint64_t n, const double* const* cols_in,
                                const double* weights_in, const uint8_t* flags, double* const* cols_out,
                                double* weights_out, uint64_t* n_accepted, void* workspace, size_t workspace_bytes,
                                void* stream)
{
    HPS_ENTRY();
    if (n_daughters < 2 || n_daughters > HPS_MAX_DAUGHTERS)
        return set_error(HPS_ERR_BAD_ARG, "n_daughters %d outside 2..10", n_daughters);
    if (n == 0) {
        // nothing to move; the accepted count is still written (0), in stream order
        if (!n_accepted) return HPS_OK;
        return cuda_status(cudaMemsetAsync(n_accepted, 0, sizeof(uint64_t), as_stream(stream)),
                           "hps_unweight_compact: cudaMemsetAsync(n_accepted)");
    }
    if (!cols_in || !cols_out || !flags) return set_error(HPS_ERR_BAD_ARG, "cols/flags is NULL");
    if ((weights_in == nullptr) != (weights_out == nullptr))
        return set_error(HPS_ERR_BAD_ARG, "weights_in and weights_out must both be given or both be NULL");
    CompactCols cc{};
    for (int k = 0; k < n_daughters; ++k) {
        if (!cols_in[k] || !cols_out[k]) return set_error(HPS_ERR_BAD_ARG, "column %d is NULL", k);
        if (!aligned(cols_in[k], 16) || !aligned(cols_out[k], 16))
            return set_error(HPS_ERR_BAD_ARG, "column %d not 16-byte aligned", k);
        if (cols_in[k] == cols_out[k]) return set_error(HPS_ERR_BAD_ARG, "column %d: out of place only", k);
        cc.in[k] = cols_in[k];
        cc.out[k] = cols_out[k];
    }
    const uint64_t ntiles = (n + kCompactTile - 1) / kCompactTile;
    const size_t need = hps_compact_workspace_size(n);
    cudaStream_t s = as_stream(stream);
    void* scratch = workspace;
    bool owned = false;
    if (workspace) {
        if (workspace_bytes < need) return set_error(HPS_ERR_BAD_ARG, "workspace of %zu bytes, %zu needed",
                                                     workspace_bytes, need);
        if (!aligned(workspace, 8)) return set_error(HPS_ERR_BAD_ARG, "workspace not 8-byte aligned");
    } else {
        cudaError_t e = cudaMallocAsync(&scratch, need, s);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_error(HPS_ERR_OOM, "cudaMallocAsync(%zu): %s", need, cudaGetErrorString(e));
        }
        owned = true;
    }
    uint64_t* counts = static_cast<uint64_t*>(scratch);
    const unsigned grid = static_cast<unsigned>(ntiles < 152u * 8u ? ntiles : 152u * 8u);
    k_flag_counts<<<grid, kCompactThreads, 0, s>>>(flags, n, ntiles, counts);
    k_scan_counts<<<1, 1024, 0, s>>>(counts, ntiles, n_accepted);
    k_scatter<<<grid, kCompactThreads, 0, s>>>(cc, n_daughters, weights_in, weights_out, flags, n, ntiles, counts);
    hps_status st = cuda_status(cudaGetLastError(), "hps_unweight_compact launch");
    if (owned) {
        cudaError_t e = cudaFreeAsync(scratch, s);
        if (st == HPS_OK && e != cudaSuccess) st = cuda_status(e, "cudaFreeAsync");
    }
    return st;
}

}  // extern "C"
