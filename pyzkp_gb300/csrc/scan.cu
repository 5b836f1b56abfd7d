// scan.cu -- device-wide exclusive prefix sum of uint32 counters (CSR row pointers).
//
// Three phases: every CTA scans a tile of 4096 counters in shared memory (warp
// shuffles inside each warp, one warp over the warp totals) and writes its tile
// total; the tile totals are scanned recursively; the tile offsets are added back.
#include "zk_internal.cuh"

namespace zk {

static constexpr int kScanThreads = 1024;
static constexpr int kScanPerThread = 4;
static constexpr int kScanTile = kScanThreads * kScanPerThread;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t o = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += o;
    }
    return v;
}

// In-place exclusive scan of one tile; tile total to sums[blockIdx.x].
__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(uint32_t* data, size_t n, uint32_t* sums) {
    __shared__ uint32_t warp_tot[kScanThreads / 32];
    const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanPerThread;
    uint32_t v[kScanPerThread];
    uint32_t local = 0;
#pragma unroll
    for (int k = 0; k < kScanPerThread; k++) {
        v[k] = (base + k < n) ? data[base + k] : 0u;
        local += v[k];
    }
    uint32_t incl = warp_incl_scan(local);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = warp_tot[lane];
        uint32_t ti = warp_incl_scan(t);
        warp_tot[lane] = ti - t;
        if (lane == 31 && sums != nullptr) sums[blockIdx.x] = ti;
    }
    __syncthreads();
    uint32_t run = warp_tot[warp] + incl - local;
#pragma unroll
    for (int k = 0; k < kScanPerThread; k++) {
        if (base + k < n) data[base + k] = run;
        run += v[k];
    }
}

__global__ void scan_add_kernel(uint32_t* data, size_t n, const uint32_t* offs) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) data[i] += offs[i / kScanTile];
}

// Scratch elements device_exclusive_scan needs for n counters (tile sums of every level).
size_t scan_scratch_elems(size_t n) {
    size_t total = 0;
    while (n > 0) {
        const size_t tiles = (n + kScanTile - 1) / kScanTile;
        total += tiles + 1;
        if (tiles <= 1) break;
        n = tiles;
    }
    return total;
}

// data[0..n) -> exclusive prefix sums; if total != nullptr, *total (device) = sum of the inputs.
// `scratch` (scan_scratch_elems(n) elements) may be given by the caller, for example by a
// pipeline that is captured into a CUDA graph; else it is allocated on the stream.
int device_exclusive_scan(Ctx* c, uint32_t* data, size_t n, uint32_t* total, uint32_t* scratch) {
    if (n == 0) return ZK_OK;
    const size_t tiles = (n + kScanTile - 1) / kScanTile;
    uint32_t* sums = scratch;
    if (sums == nullptr) {
        int rc = scratch_alloc(c, (tiles + 1) * sizeof(uint32_t), reinterpret_cast<void**>(&sums));
        if (rc != ZK_OK) return rc;
    }
    ZK_LAUNCH(c, "scan_tiles", scan_tiles_kernel, (unsigned)tiles, kScanThreads, 0, data, n, sums);
    ZK_TRY_CUDA(cudaGetLastError());
    if (tiles > 1) {
        // sums[tiles] receives the grand total through the recursive scan's total slot
        int rc = device_exclusive_scan(c, sums, tiles, total, scratch ? scratch + tiles + 1 : nullptr);
        if (rc != ZK_OK) return rc;
        ZK_LAUNCH(c, "scan_add", scan_add_kernel, (unsigned)((n + 255) / 256), 256, 0, data, n, sums);
        ZK_TRY_CUDA(cudaGetLastError());
    } else if (total != nullptr) {
        ZK_TRY_CUDA(cudaMemcpyAsync(total, sums, sizeof(uint32_t), cudaMemcpyDeviceToDevice, c->stream));
    }
    if (scratch == nullptr) scratch_free(c, sums);
    return ZK_OK;
}

}  // namespace zk
