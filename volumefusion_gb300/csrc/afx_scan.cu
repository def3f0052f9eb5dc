// afx_scan.cu -- exclusive prefix sums used for stream compaction and CSR offsets.
// Three phases: per-tile sums, a single-block scan of those sums, then the tile-local scans
// with their offsets added.  Deterministic (integer arithmetic).  The tile phases are
// grid-stride loops over the tiles that hold live items (the live count is read on the device),
// on a grid of at most kScanBlocks, so a large capacity with few items costs one short wave.
#include "afx_internal.h"

namespace afx {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

AFX_D unsigned block_exclusive_scan(unsigned v, unsigned* warp_sums, unsigned* block_total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        unsigned s = lane < nw ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) warp_sums[lane] = s;
    }
    __syncthreads();
    unsigned excl = x - v + (wid > 0 ? warp_sums[wid - 1] : 0u);
    if (block_total) *block_total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return excl;
}

__device__ __forceinline__ long scan_n(const unsigned* count, long n_max) {
    return count ? min((long)*count, n_max) : n_max;
}

constexpr long kScanBlocks = 152;

__global__ void __launch_bounds__(kScanThreads) scan_block_sums(const unsigned* in, const unsigned* count, long n_max,
                                                                 unsigned* sums) {
    __shared__ unsigned ws[32];
    const long n = scan_n(count, n_max);
    const long nt = (n + kScanTile - 1) / kScanTile;
    for (long tile = blockIdx.x; tile < nt; tile += gridDim.x) {
        const long base = tile * kScanTile;
        unsigned s = 0;
        for (int i = 0; i < kScanItems; ++i) {
            long j = base + (long)threadIdx.x * kScanItems + i;
            if (j < n) s += in[j];
        }
        unsigned tot;
        block_exclusive_scan(s, ws, &tot);
        if (threadIdx.x == 0) sums[tile] = tot;
    }
}

__global__ void __launch_bounds__(1024) scan_sums_kernel(unsigned* sums, const unsigned* count, long n_max,
                                                         unsigned* total) {
    __shared__ unsigned ws[32];
    const long nblocks = (scan_n(count, n_max) + kScanTile - 1) / kScanTile;
    unsigned carry = 0;
    for (long base = 0; base < nblocks; base += blockDim.x) {
        long j = base + threadIdx.x;
        unsigned v = j < nblocks ? sums[j] : 0u;
        unsigned tot;
        unsigned e = block_exclusive_scan(v, ws, &tot);
        if (j < nblocks) sums[j] = e + carry;
        carry += tot;
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void __launch_bounds__(kScanThreads) scan_apply(const unsigned* in, unsigned* out, const unsigned* count,
                                                           long n_max, const unsigned* sums) {
    __shared__ unsigned ws[32];
    const long n = scan_n(count, n_max);
    const long nt = (n + kScanTile - 1) / kScanTile;
    for (long tile = blockIdx.x; tile < nt; tile += gridDim.x) {
        const long base = tile * kScanTile;
        unsigned v[kScanItems];
        unsigned s = 0;
        for (int i = 0; i < kScanItems; ++i) {
            long j = base + (long)threadIdx.x * kScanItems + i;
            v[i] = j < n ? in[j] : 0u;
            s += v[i];
        }
        unsigned e = block_exclusive_scan(s, ws, nullptr) + sums[tile];
        for (int i = 0; i < kScanItems; ++i) {
            long j = base + (long)threadIdx.x * kScanItems + i;
            if (j < n) out[j] = e;
            e += v[i];
        }
    }
}

size_t scan_workspace_size(long n) { return (size_t)((n + kScanTile - 1) / kScanTile + 1) * sizeof(unsigned); }

int scan_exclusive_dev(const unsigned* in, unsigned* out, const unsigned* count, long n_max, unsigned* total, void* ws,
                       cudaStream_t st) {
    if (n_max <= 0) {
        if (total) AFX_CUDA(cudaMemsetAsync(total, 0, sizeof(unsigned), st));
        return AFX_OK;
    }
    const long nb = (n_max + kScanTile - 1) / kScanTile;
    const unsigned grid = (unsigned)(nb < kScanBlocks ? nb : kScanBlocks);
    unsigned* sums = static_cast<unsigned*>(ws);
    scan_block_sums<<<grid, kScanThreads, 0, st>>>(in, count, n_max, sums);
    AFX_LAUNCH_CHECK();
    scan_sums_kernel<<<1, 1024, 0, st>>>(sums, count, n_max, total);
    AFX_LAUNCH_CHECK();
    scan_apply<<<grid, kScanThreads, 0, st>>>(in, out, count, n_max, sums);
    AFX_LAUNCH_CHECK();
    return AFX_OK;
}

int scan_exclusive(const unsigned* in, unsigned* out, long n, unsigned* total, void* ws, cudaStream_t st) {
    return scan_exclusive_dev(in, out, nullptr, n, total, ws, st);
}

}  // namespace afx
