// Hash-grid build, per element / per tile (reference binKernel,
// voro_optimizer.cu:168-177; cub ExclusiveSum :697; scatterKernel :179-187).
// Shared by the batch-table kernels (vm_step.cu) and the allocation-free
// entry point (vm_noalloc.cu).
#pragma once

#include "vm_device.cuh"

namespace vmk {

// Keys of a point set: its grid cells, times the sub-cells of each.
__device__ __forceinline__ int grid_keys(const VmPointSet &S) { return (S.gridW * S.gridH) << (2 * S.sub); }

// cell key + atomic rank of point i. Sites: x < 0 is an empty slot
// (reference binKernel :172); targets: NaN x too (vorolossKernel :216).
__device__ __forceinline__ void grid_bin_one(const VmPointSet &S, int i, int emptyIsNegative)
{
    if (i >= S.n) return;
    float2 p = S.pts[i];
    bool empty = emptyIsNegative ? (p.x < 0.0f) : !(p.x >= 0.0f);
    if (empty) {
        S.key[i] = -1;
        return;
    }
    int c;
    if (S.sub) {
        // cell-major key with the sub-cell (row-major within the cell) below it;
        // scaling inv by 2^sub is exact, so key >> 2 sub is the cell itself
        int fx = cell_coord(p.x, S.inv * (float)(1 << S.sub), S.gridW << S.sub);
        int fy = cell_coord(p.y, S.inv * (float)(1 << S.sub), S.gridH << S.sub);
        int m = (1 << S.sub) - 1;
        c = ((((fy >> S.sub) * S.gridW + (fx >> S.sub)) << S.sub | (fy & m)) << S.sub) | (fx & m);
    } else {
        c = cell_coord(p.y, S.inv, S.gridH) * S.gridW + cell_coord(p.x, S.inv, S.gridW);
    }
    S.key[i] = c;
    S.rank[i] = atomicAdd(&S.counts[c], 1);
}

// block-wide exclusive scan of 8 values per thread (256 threads)
__device__ __forceinline__ int block_scan8(int (&v)[8], int *warpSums, int &total)
{
    int run = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        int x = v[k];
        v[k] = run;
        run += x;
    }
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = run;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        int t = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl += t;
    }
    if (lane == 31) warpSums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = lane < 8 ? warpSums[lane] : 0, wi = w;
#pragma unroll
        for (int off = 1; off < 8; off <<= 1) {
            int t = __shfl_up_sync(kFull, wi, off);
            if (lane >= off) wi += t;
        }
        if (lane < 8) warpSums[8 + lane] = wi - w;
        if (lane == 7) warpSums[16] = wi;
    }
    __syncthreads();
    int excl = incl - run + warpSums[8 + warp];
    total = warpSums[16];
    return excl;
}

// tileSums[tile] = sum of the tile's cell counts (256-thread block)
__device__ __forceinline__ void grid_tile_sum(const VmPointSet &S, int tile)
{
    __shared__ int red[8];
    int cells = grid_keys(S);
    int base = tile * kScanTile + threadIdx.x * 8;
    int sum = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (base + k < cells) sum += S.counts[base + k];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) sum += __shfl_down_sync(kFull, sum, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < 8; ++w) t += red[w];
        S.tileSums[tile] = t;
    }
}

// start[] of the tile's cells from the earlier tiles' sums (256-thread block)
__device__ __forceinline__ void grid_tile_apply(const VmPointSet &S, int tile)
{
    __shared__ int ws[24];
    __shared__ int sOffset;
    int cells = grid_keys(S);
    int part = 0;
    for (int t = threadIdx.x; t < tile; t += blockDim.x) part += S.tileSums[t];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) part += __shfl_down_sync(kFull, part, off);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < 8; ++w) t += ws[w];
        sOffset = t;
    }
    __syncthreads();
    int offset = sOffset;
    int base = tile * kScanTile + threadIdx.x * 8;
    int v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = base + k < cells ? S.counts[base + k] : 0;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (base + k < cells) S.counts[base + k] = 0; // zero again for the next build
    int total;
    int excl = block_scan8(v, ws, total);
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (base + k < cells) S.start[base + k] = offset + excl + v[k];
    int tiles = (cells + kScanTile - 1) / kScanTile;
    if (tile == tiles - 1 && threadIdx.x == 0) S.start[cells] = offset + total;
}

// Cell-sorted copy of point i (its rank within the cell is the arrival order
// of the binning atomics).
__device__ __forceinline__ void grid_scatter_one(const VmPointSet &S, int i)
{
    if (i >= S.n) return;
    int c = S.key[i];
    if (c < 0) return;
    int s = S.start[c] + S.rank[i];
    S.outIdx[s] = i;
    S.outPos[s] = S.pts[i];
}

// Canonical order of cell c's run: ascending point index (insertion sort; a
// run holds a few points).
__device__ __forceinline__ void grid_canonical_one(const VmPointSet &S, int c)
{
    if (c >= grid_keys(S)) return;
    int b = S.start[c], e = S.start[c + 1];
    for (int a = b + 1; a < e; ++a) {
        int id = S.outIdx[a];
        float2 ps = S.outPos[a];
        int q = a - 1;
        while (q >= b) {
            int iq = S.outIdx[q];
            if (iq <= id) break;
            S.outIdx[q + 1] = iq;
            S.outPos[q + 1] = S.outPos[q];
            --q;
        }
        S.outIdx[q + 1] = id;
        S.outPos[q + 1] = ps;
    }
}

} // namespace vmk
