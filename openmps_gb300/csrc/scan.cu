// scan.cu - device-wide exclusive prefix sum of int32 counts (three passes, no waits):
// per-block scans, one block scanning the block totals, then the block offsets added.
// Used to lay out the PPE matrix chunks contiguously.
#include "common.cuh"

namespace mpsgb {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

// Exclusive scan of one value per thread over the block; returns the block total.
__device__ int block_exclusive_scan(int v, int* out_excl) {
    __shared__ int warp_tot[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        int w = (lane < nw) ? warp_tot[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < nw) warp_tot[lane] = w;  // inclusive warp prefix
    }
    __syncthreads();
    const int warp_off = (wid > 0) ? warp_tot[wid - 1] : 0;
    *out_excl = warp_off + incl - v;
    const int total = warp_tot[(blockDim.x >> 5) - 1];
    __syncthreads();
    return total;
}

__global__ void k_scan_tiles(const int* in, int* out, int m, int* tile_sums) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = (base + k < m) ? in[base + k] : 0;
        s += v[k];
    }
    int excl;
    const int total = block_exclusive_scan(s, &excl);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < m) out[base + k] = excl;
        excl += v[k];
    }
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// One block: exclusive scan of the tile totals (any count), total at tile_sums[tiles].
__global__ void k_scan_tile_sums(int* tile_sums, int tiles) {
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int start = 0; start < tiles; start += blockDim.x) {
        const int t = start + threadIdx.x;
        const int v = (t < tiles) ? tile_sums[t] : 0;
        int excl;
        const int total = block_exclusive_scan(v, &excl);
        if (t < tiles) tile_sums[t] = carry + excl;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) tile_sums[tiles] = carry;
}

__global__ void k_scan_add(int* out, int m, const int* tile_sums, int tiles) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    const int add = tile_sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
        if (base + k < m) out[base + k] += add;
    if (blockIdx.x == 0 && threadIdx.x == 0) out[m] = tile_sums[tiles];
}

}  // namespace

int scan_scratch_ints(int m) { return (m + kScanTile - 1) / kScanTile + 1; }

void launch_exclusive_scan(const int* in, int* out, int m, int* scratch, cudaStream_t s) {
    const int tiles = (m + kScanTile - 1) / kScanTile;
    if (tiles == 0) {
        cudaMemsetAsync(out, 0, sizeof(int), s);
        return;
    }
    k_scan_tiles<<<tiles, kScanThreads, 0, s>>>(in, out, m, scratch);
    k_scan_tile_sums<<<1, kScanThreads, 0, s>>>(scratch, tiles);
    k_scan_add<<<tiles, kScanThreads, 0, s>>>(out, m, scratch, tiles);
}

}  // namespace mpsgb
