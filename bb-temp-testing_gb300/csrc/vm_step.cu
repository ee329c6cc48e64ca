// VoroMesh optimisation step kernels (batch-native).
//
//   k_bin          cell key + atomic count per point        (reference binKernel, voro_optimizer.cu:168-177)
//   k_scan_tiles   per-tile sums of the cell counts; a set's last tile turns
//                  them into tile prefixes           (reference cub ExclusiveSum, :697)
//   k_scan_apply   exclusive scan of each tile from its prefix -> cell start
//   k_scatter      cell-sorted copy (reference scatterKernel :179-187)
//   k_canonical    each cell's run sorted by slot index (before the grid is exported)
//   (k_loss        VoroLoss + analytic gradient per target, vm_loss.cu)
//   k_adam_bin     Adam + clamp, fused with the next step's binning (reference
//                  adamKernel :271-301 + binKernel); its lr and bias corrections
//                  come from adam_schedule in the loss pass
//   k_finalize     publish a loss-only pass (EvaluateLoss, :746-761)
//   k_knn          exact kNN query operator (reference knn<K>, :130-163)
//
// One step of a set of fits is: k_loss -> k_loss_exact -> k_adam_bin ->
// k_scan_tiles -> k_scan_apply -> k_scatter(publish). The grid is therefore
// always built for the current generators between steps, as the reference
// rebuilds it at the start of each step. Nothing in the step depends on the
// order within a cell's run (every argmin breaks ties by index, every sum is
// exact), so k_canonical runs only before the grid is exported.
#include "vm_device.cuh"
#include "vm_adam.cuh"
#include "vm_grid.cuh"
#include "vm_knn.cuh"
#include "vm_kernels.h"

namespace vmk {

// The scatter keeps the 256-site block of the site prefix tables but serves it
// with 64 threads, four sites each: their loads are issued together and the
// whole launch fits on the GPU at once, so each thread's chain of dependent
// loads (key, then the cell's start) is paid once.
constexpr int kSiteBlock = 256;
constexpr int kSiteThreads = 64;
constexpr int kSitesPerThread = kSiteBlock / kSiteThreads;


// ---------------------------------------------------------------------------
// hash grid build over a table of point sets (bodies in vm_grid.cuh)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_bin(const VmPointSet *__restrict__ sets, const int *__restrict__ prefix,
                                             int nSets, int emptyIsNegative)
{
    int f = find_fit(prefix, nSets, blockIdx.x);
    grid_bin_one(sets[f], (blockIdx.x - prefix[f]) * blockDim.x + threadIdx.x, emptyIsNegative);
}

// The scan of the cell counts, one block per scan tile of every set (bodies
// in vm_grid.cuh): tile sums, with each set's tile prefixes made by its last
// tile; then each tile's cells.
__global__ void __launch_bounds__(256) k_scan_tiles(const VmPointSet *__restrict__ sets,
                                                    const int *__restrict__ prefix, int nSets)
{
    int f = find_fit(prefix, nSets, blockIdx.x);
    grid_tile_reduce(sets[f], blockIdx.x - prefix[f]);
}

__global__ void __launch_bounds__(256) k_scan_apply(const VmPointSet *__restrict__ sets,
                                                    const int *__restrict__ prefix, int nSets)
{
    int f = find_fit(prefix, nSets, blockIdx.x);
    grid_tile_scan(sets[f], blockIdx.x - prefix[f]);
}

__global__ void __launch_bounds__(256) k_canonical(const VmPointSet *__restrict__ sets,
                                                   const int *__restrict__ prefix, int nSets)
{
    // kScanTile / 256 blocks per scan tile, one thread per cell
    constexpr int kPer = kScanTile / 256;
    int f = find_fit(prefix, nSets, blockIdx.x / kPer);
    if (sets[f].canonical) grid_canonical_one(sets[f], (blockIdx.x - prefix[f] * kPer) * 256 + threadIdx.x);
}

__global__ void __launch_bounds__(kSiteThreads) k_scatter(const VmPointSet *__restrict__ sets,
                                                          const int *__restrict__ prefix, int nSets,
                                                          const VmFit *__restrict__ publish)
{
    int f = find_fit(prefix, nSets, blockIdx.x);
    int local = blockIdx.x - prefix[f];
    if (publish && local == 0 && threadIdx.x == 0 && publish[f].active) {
        // end of a step: publish the loss pass and advance the step counter
        VmState *st = publish[f].state;
        st->loss = fxl_to_float(st->accLo, st->accHi, publish[f].lossExp);
        st->count = st->accCount;
        st->iter += 1;
        st->accLo = 0;
        st->accHi = 0;
        st->accCount = 0;
        st->needExact = 0;
        st->dUsed = 0;
    }
    // the block's points (grid_scatter_one, several per thread with their
    // loads issued together)
    const VmPointSet &S = sets[f];
    int i0 = local * kSiteBlock + threadIdx.x;
    int c[kSitesPerThread], r[kSitesPerThread];
    float2 q[kSitesPerThread];
#pragma unroll
    for (int k = 0; k < kSitesPerThread; ++k) {
        int i = i0 + k * kSiteThreads;
        c[k] = -1;
        if (i < S.n) {
            c[k] = S.key[i];
            r[k] = S.rank[i];
            q[k] = S.pts[i];
        }
    }
    int at[kSitesPerThread];
#pragma unroll
    for (int k = 0; k < kSitesPerThread; ++k)
        if (c[k] >= 0) at[k] = S.start[c[k]] + r[k];
#pragma unroll
    for (int k = 0; k < kSitesPerThread; ++k)
        if (c[k] >= 0) {
            S.outIdx[at[k]] = i0 + k * kSiteThreads;
            S.outPos[at[k]] = q[k];
        }
}

// Publishes a loss-only pass: loss and count of the accumulator, iteration kept.
__global__ void k_finalize(const VmFit *__restrict__ fits, int nFits, SlowQueue *queue)
{
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f == 0) {
        queue->count = 0;
        queue->nFlagged = 0;
    }
    if (f >= nFits) return;
    VmState *st = fits[f].state;
    st->loss = fxl_to_float(st->accLo, st->accHi, fits[f].lossExp);
    st->count = st->accCount;
    st->fallbacks = st->slowTotal;
    st->accLo = 0;
    st->accHi = 0;
    st->accCount = 0;
}

// ---------------------------------------------------------------------------
// Adam (fused with the next grid's binning). Bound by load latency: the
// slot's loads are issued together, and 32 registers keep 8 blocks resident
// per SM (measured faster than 45 registers at 5 blocks).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 8) k_adam_bin(const VmFit *__restrict__ fits, const int *__restrict__ prefix,
                                                  int nFits, SlowQueue *queue)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        queue->count = 0;
        queue->nFlagged = 0;
    }
    int f = find_fit(prefix, nFits, blockIdx.x);
    const VmFit &F = fits[f];
    if (!F.active) return;
    int i = (blockIdx.x - prefix[f]) * blockDim.x + threadIdx.x;
    if (i >= F.nSlots) return;
    float2 p = adam_slot(F, adam_step(F), i);
    if (p.x < 0.0f) {
        F.key[i] = -1;
        return;
    }
    int c = cell_coord(p.y, F.inv, F.gridH) * F.gridW + cell_coord(p.x, F.inv, F.gridW);
    F.key[i] = c;
    F.rank[i] = atomicAdd(&F.counts[c], 1);
}

// The largest number of targets in any 5x5 block of hash cells (the bound
// behind a fit's fast-path split shift), from the target sort's key starts:
// keys are cell << 2 sub, so a row of cells is one contiguous key range.
__global__ void __launch_bounds__(256) k_block5_max(const int *__restrict__ tstart, int gw, int gh, int sub,
                                                    int *out)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    int sum = 0;
    if (c < gw * gh) {
        int y = c / gw, x = c - y * gw;
        int xa = max(x - 2, 0), xb = min(x + 2, gw - 1);
        for (int yy = max(y - 2, 0); yy <= min(y + 2, gh - 1); ++yy)
            sum += tstart[(size_t)(yy * gw + xb + 1) << (2 * sub)] - tstart[(size_t)(yy * gw + xa) << (2 * sub)];
    }
    sum = __reduce_max_sync(kFull, sum);
    if ((threadIdx.x & 31) == 0 && sum > 0) atomicMax(out, sum);
}

// The loss windows of a fit's cell-sorted targets: the number of windows of
// each cell's run (at most 32 targets each), then each window's start.
__global__ void k_win_count(const int *__restrict__ tstart, int cells, int sub, int *counts)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    int n = tstart[(size_t)(c + 1) << (2 * sub)] - tstart[(size_t)c << (2 * sub)];
    counts[c] = (n + 31) >> 5;
}

__global__ void k_win_fill(const int *__restrict__ tstart, int cells, int sub, const int *__restrict__ wstart,
                           int *twin)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    int s = tstart[(size_t)c << (2 * sub)], n = tstart[(size_t)(c + 1) << (2 * sub)] - s, w = wstart[c];
    for (int k = 0; 32 * k < n; ++k) twin[w + k] = s + 32 * k;
    if (c == cells - 1) twin[wstart[cells]] = tstart[(size_t)cells << (2 * sub)];
}

// Sparse target update (reference scatterTargetsKernel, voro_optimizer.cu:303-307)
__global__ void k_scatter_targets(float2 *targets, const int *slots, const float2 *values, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) targets[slots[i]] = values[i];
}

// ---------------------------------------------------------------------------
// kNN operator over a fit's current grid
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(128) k_knn(const VmFit *__restrict__ fit, const float2 *__restrict__ q, int nq,
                                             int *__restrict__ outIdx, float *__restrict__ outD2)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const VmFit &F = *fit;
    float d2[K];
    int idx[K];
    knn_ring<K>(F.start, F.sortedPos, F.sortedIdx, F.gridW, F.gridH, F.cell, F.inv, q[i], d2, idx);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        outIdx[(size_t)i * K + k] = idx[k];
        outD2[(size_t)i * K + k] = d2[k];
    }
}

} // namespace vmk

// ---------------------------------------------------------------------------
// launch wrappers (host)
// ---------------------------------------------------------------------------
using namespace vmk;

extern "C++" {

cudaError_t vm_launch_bin(const VmPointSet *sets, const int *prefix, int nSets, int totalBlocks, int emptyIsNegative,
                          cudaStream_t s)
{
    if (totalBlocks <= 0) return cudaSuccess;
    k_bin<<<totalBlocks, 256, 0, s>>>(sets, prefix, nSets, emptyIsNegative);
    return cudaGetLastError();
}

cudaError_t vm_launch_scan(const VmPointSet *sets, const int *tilePrefix, int nSets, int totalTiles, cudaStream_t s)
{
    if (totalTiles <= 0) return cudaSuccess;
    k_scan_tiles<<<totalTiles, 256, 0, s>>>(sets, tilePrefix, nSets);
    k_scan_apply<<<totalTiles, 256, 0, s>>>(sets, tilePrefix, nSets);
    return cudaGetLastError();
}

cudaError_t vm_launch_canonical(const VmPointSet *sets, const int *tilePrefix, int nSets, int totalTiles,
                                cudaStream_t s)
{
    if (totalTiles <= 0) return cudaSuccess;
    k_canonical<<<totalTiles * (kScanTile / 256), 256, 0, s>>>(sets, tilePrefix, nSets);
    return cudaGetLastError();
}

cudaError_t vm_launch_scatter(const VmPointSet *sets, const int *prefix, int nSets, int totalBlocks,
                              const VmFit *publish, cudaStream_t s)
{
    if (totalBlocks <= 0) return cudaSuccess;
    k_scatter<<<totalBlocks, kSiteThreads, 0, s>>>(sets, prefix, nSets, publish);
    return cudaGetLastError();
}

cudaError_t vm_launch_finalize(const VmFit *fits, int nFits, void *queue, cudaStream_t s)
{
    if (nFits <= 0) return cudaSuccess;
    k_finalize<<<(nFits + 127) / 128, 128, 0, s>>>(fits, nFits, static_cast<SlowQueue *>(queue));
    return cudaGetLastError();
}

cudaError_t vm_launch_adam_bin(const VmFit *fits, const int *prefix, int nFits, int totalBlocks, void *queue,
                               cudaStream_t s)
{
    if (totalBlocks <= 0) return cudaSuccess;
    k_adam_bin<<<totalBlocks, 256, 0, s>>>(fits, prefix, nFits, static_cast<SlowQueue *>(queue));
    return cudaGetLastError();
}

cudaError_t vm_queue_init(void *queue, void *items, int capacity, cudaStream_t s)
{
    SlowQueue q{0, capacity, static_cast<int2 *>(items)};
    return cudaMemcpyAsync(queue, &q, sizeof(q), cudaMemcpyHostToDevice, s);
}

size_t vm_queue_bytes() { return sizeof(SlowQueue); }

cudaError_t vm_launch_knn(const VmFit *fit, const float2 *q, int nq, int K, int *outIdx, float *outD2, cudaStream_t s)
{
    if (nq <= 0) return cudaSuccess;
    int b = (nq + 127) / 128;
    switch (K) {
    case 8: k_knn<8><<<b, 128, 0, s>>>(fit, q, nq, outIdx, outD2); break;
    case 12: k_knn<12><<<b, 128, 0, s>>>(fit, q, nq, outIdx, outD2); break;
    case 16: k_knn<16><<<b, 128, 0, s>>>(fit, q, nq, outIdx, outD2); break;
    case 24: k_knn<24><<<b, 128, 0, s>>>(fit, q, nq, outIdx, outD2); break;
    case 32: k_knn<32><<<b, 128, 0, s>>>(fit, q, nq, outIdx, outD2); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t vm_launch_block5_max(const int *tstart, int gridW, int gridH, int sub, int *out, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(int), s);
    if (e) return e;
    int cells = gridW * gridH;
    k_block5_max<<<(cells + 255) / 256, 256, 0, s>>>(tstart, gridW, gridH, sub, out);
    return cudaGetLastError();
}

int vm_fast_shift(int block5Max)
{
    int bits = 0; // ceil(log2(max(block5Max, 1)))
    while (bits < 31 && (1LL << bits) < (long long)block5Max) ++bits;
    return 38 - bits;
}

cudaError_t vm_launch_target_windows(const int *tstart, int cells, int sub, const VmPointSet *winSet,
                                     const int *winPre, int tiles, int *counts, const int *start, int *twin,
                                     cudaStream_t s)
{
    if (cells <= 0) return cudaSuccess;
    int b = (cells + 255) / 256;
    k_win_count<<<b, 256, 0, s>>>(tstart, cells, sub, counts);
    cudaError_t e = vm_launch_scan(winSet, winPre, 1, tiles, s);
    if (e) return e;
    k_win_fill<<<b, 256, 0, s>>>(tstart, cells, sub, start, twin);
    return cudaGetLastError();
}

cudaError_t vm_launch_scatter_targets(float2 *targets, const int *slots, const float2 *values, int n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    k_scatter_targets<<<(n + 127) / 128, 128, 0, s>>>(targets, slots, values, n);
    return cudaGetLastError();
}

} // extern "C++"
