// Hash-grid build that allocates nothing (vm_build_grid_noalloc, vm_capi.h).
//
// Some callers cannot let a library allocate device memory: a frame loop
// (an interactive editor stamping edits every frame) where cudaMalloc's
// implicit device synchronisation would stall the frame, or a host program
// that plans every byte of device memory itself and hands libraries only
// pre-sized buffers. This entry point serves them: the caller passes the
// generators and the three output arrays, and the scratch the build needs
// (cell keys, within-cell ranks, per-cell counts, scan-tile sums) lives in
// one file-scope __device__ array of fixed size, which every GPU that loads
// the library holds until the process exits.
//
// The first call on a device looks up that array's device address with
// cudaGetSymbolAddress (the array's name in host code is only a host-side
// stand-in, not a device address); make that first call before any stream
// capture: a first call on a capturing stream returns VM_ERR_UNSUPPORTED
// instead of invalidating the capture. The address is kept for the process;
// a cudaDeviceReset reloads the library's module and invalidates it, so a
// failed launch drops it and the next call looks it up again. Every call
// shares the array, so calls that overlap on the GPU (different streams, or
// different host threads) race and must be ordered by the caller. Each call
// clears the counts it uses before binning.
#include <cstddef>
#include <mutex>

#include "vm_capi.h"
#include "vm_grid.cuh"
#include "vm_host.h"

namespace {

constexpr int kMaxPoints = VM_NOALLOC_MAX_POINTS;
constexpr int kMaxCells = VM_NOALLOC_MAX_CELLS;
constexpr int kMaxTiles = (kMaxCells + kScanTile - 1) / kScanTile;

struct NoAllocScratch {
    int key[kMaxPoints];
    int rank[kMaxPoints];
    int counts[kMaxCells + 1];
    int tileSums[kMaxTiles + 1];
};

__device__ __align__(256) NoAllocScratch g_noallocScratch;

__global__ void __launch_bounds__(256) k_na_bin(VmPointSet S) { vmk::grid_bin_one(S, blockIdx.x * blockDim.x + threadIdx.x, 1); }
__global__ void __launch_bounds__(256) k_na_tile_sum(VmPointSet S) { vmk::grid_tile_sum(S, blockIdx.x); }
__global__ void __launch_bounds__(256) k_na_tile_apply(VmPointSet S) { vmk::grid_tile_apply(S, blockIdx.x); }
__global__ void __launch_bounds__(256) k_na_scatter(VmPointSet S) { vmk::grid_scatter_one(S, blockIdx.x * blockDim.x + threadIdx.x); }
__global__ void __launch_bounds__(256) k_na_canonical(VmPointSet S) { vmk::grid_canonical_one(S, blockIdx.x * blockDim.x + threadIdx.x); }

constexpr int kMaxDevices = 64;
char *g_scratchAddr[kMaxDevices]; // device address of g_noallocScratch, per device
std::mutex g_scratchMutex;

// Per-device set-up with that device current: the device address of the array.
int scratch_for(int dev, cudaStream_t s, char **out)
{
    std::lock_guard<std::mutex> lock(g_scratchMutex);
    if (!g_scratchAddr[dev]) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaError_t ce = cudaStreamIsCapturing(s, &cs);
        if (ce != cudaSuccess) return vmh::cuda_fail(ce, "cudaStreamIsCapturing");
        if (cs != cudaStreamCaptureStatusNone)
            return vmh::fail(VM_ERR_UNSUPPORTED, "vm_build_grid_noalloc: the first call on a device must come "
                                                 "before any stream capture");
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess) return vmh::cuda_fail(e, "cudaGetSymbolAddress");
        g_scratchAddr[dev] = static_cast<char *>(p);
    }
    *out = g_scratchAddr[dev];
    return VM_OK;
}

void scratch_forget(int dev)
{
    std::lock_guard<std::mutex> lock(g_scratchMutex);
    g_scratchAddr[dev] = nullptr;
}

} // namespace

extern "C" int vm_build_grid_noalloc(const float *generators, int n, int gridW, int gridH, float cellSize, int *start,
                                     int *sortedIdx, float *sortedPos, void *stream)
{
    if (n < 0 || gridW < 1 || gridH < 1 || !(cellSize > 0.0f) || !start || (n > 0 && (!generators || !sortedIdx || !sortedPos)))
        return vmh::fail(VM_ERR_ARG, "vm_build_grid_noalloc: bad arguments");
    if (n > kMaxPoints) return vmh::fail(VM_ERR_ARG, "vm_build_grid_noalloc: more than VM_NOALLOC_MAX_POINTS generators");
    if ((long long)gridW * gridH > kMaxCells)
        return vmh::fail(VM_ERR_ARG, "vm_build_grid_noalloc: more than VM_NOALLOC_MAX_CELLS grid cells");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return vmh::cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return vmh::fail(VM_ERR_UNSUPPORTED, "vm_build_grid_noalloc: device index too large");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    char *base = nullptr;
    int rc = scratch_for(dev, s, &base);
    if (rc) return rc;
    // a non-sticky error left pending by earlier, unrelated work is cleared
    // here so that it is not reported as this call's failure
    (void)cudaGetLastError();
    int cells = gridW * gridH;
    int tiles = (cells + kScanTile - 1) / kScanTile;
    VmPointSet S{};
    S.pts = reinterpret_cast<const float2 *>(generators);
    S.n = n;
    S.gridW = gridW;
    S.gridH = gridH;
    S.inv = 1.0f / cellSize;
    S.key = reinterpret_cast<int *>(base + offsetof(NoAllocScratch, key));
    S.rank = reinterpret_cast<int *>(base + offsetof(NoAllocScratch, rank));
    S.counts = reinterpret_cast<int *>(base + offsetof(NoAllocScratch, counts));
    S.tileSums = reinterpret_cast<int *>(base + offsetof(NoAllocScratch, tileSums));
    S.start = start;
    S.outPos = reinterpret_cast<float2 *>(sortedPos);
    S.outIdx = sortedIdx;
    S.canonical = 1;
    S.useIndexOrder = 1;
    // the array keeps the previous call's contents: the counts must start at zero
    if ((e = cudaMemsetAsync(S.counts, 0, sizeof(int) * (size_t)(cells + 1), s)) != cudaSuccess)
        return vmh::cuda_fail(e, "clear counts");
    int blocks = (n + 255) / 256;
    // each launch is checked before the next is enqueued
    auto launched = [&](const char *what) -> int {
        cudaError_t le = cudaGetLastError();
        if (le == cudaSuccess) return VM_OK;
        scratch_forget(dev);
        return vmh::cuda_fail(le, what);
    };
    if (blocks) {
        k_na_bin<<<blocks, 256, 0, s>>>(S);
        if ((rc = launched("vm_build_grid_noalloc: bin"))) return rc;
    }
    k_na_tile_sum<<<tiles, 256, 0, s>>>(S);
    if ((rc = launched("vm_build_grid_noalloc: tile sums"))) return rc;
    k_na_tile_apply<<<tiles, 256, 0, s>>>(S);
    if ((rc = launched("vm_build_grid_noalloc: scan"))) return rc;
    if (blocks) {
        k_na_scatter<<<blocks, 256, 0, s>>>(S);
        if ((rc = launched("vm_build_grid_noalloc: scatter"))) return rc;
    }
    k_na_canonical<<<(cells + 255) / 256, 256, 0, s>>>(S);
    return launched("vm_build_grid_noalloc: canonical order");
}
