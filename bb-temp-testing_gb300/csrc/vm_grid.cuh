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

// ---- two-pass scan with the tile prefixes made by the last tile -------------
// Pass 1 stores each scan tile's sum in the set's tileState word and counts
// the tile as done; the block that counts a set's last tile (every other
// tile's sum is then written) turns the set's sums into exclusive prefixes and
// writes start[cells]. Pass 2 scans each tile from its prefix and zeroes the
// prefix word. Nothing waits, and each tile of pass 2 reads one prefix word
// instead of every earlier tile's sum. tileState[tiles] (low half) is the
// set's done counter. Every word is zero between scans, so a buffer can serve
// a later scan of fewer tiles (its done counter then sits on an old tile word).
__device__ __forceinline__ int grid_tiles(const VmPointSet &S) { return (grid_keys(S) + kScanTile - 1) / kScanTile; }

// The eight counts of this thread in the tile; `zero`: clear them for the next build.
__device__ __forceinline__ void grid_load8(const VmPointSet &S, int base, int cells, int (&v)[8], bool zero)
{
    if (base + 8 <= cells) {
        int4 *c = reinterpret_cast<int4 *>(S.counts + base);
        int4 a = c[0], b = c[1];
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
        if (zero) {
            c[0] = make_int4(0, 0, 0, 0);
            c[1] = make_int4(0, 0, 0, 0);
        }
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            v[k] = base + k < cells ? S.counts[base + k] : 0;
            if (zero && base + k < cells) S.counts[base + k] = 0;
        }
    }
}

// Pass 1 for tile `tile` of S (256-thread block).
__device__ __forceinline__ void grid_tile_reduce(const VmPointSet &S, int tile)
{
    __shared__ int red[24];
    __shared__ int sLast;
    int cells = grid_keys(S), tiles = grid_tiles(S);
    int v[8];
    grid_load8(S, tile * kScanTile + threadIdx.x * 8, cells, v, false);
    int sum = v[0] + v[1] + v[2] + v[3] + v[4] + v[5] + v[6] + v[7];
    sum = __reduce_add_sync(kFull, sum);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
    __syncthreads();
    unsigned *done = reinterpret_cast<unsigned *>(S.tileState + tiles);
    if (threadIdx.x == 0) {
        int t = 0;
#pragma unroll
        for (int w = 0; w < 8; ++w) t += red[w];
        S.tileState[tile] = (unsigned)t;
        __threadfence(); // the sum is visible before the tile counts as done
        sLast = atomicAdd(done, 1u) == (unsigned)tiles - 1u;
    }
    __syncthreads();
    if (!sLast) return;
    // the set's last tile: exclusive prefixes of all its tiles' sums
    __threadfence();
    int carry = 0;
    for (int b = 0; b < tiles; b += kScanTile) {
        int w[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            int t = b + threadIdx.x * 8 + k;
            w[k] = t < tiles ? (int)(unsigned)__ldcg(S.tileState + t) : 0;
        }
        int total;
        int excl = block_scan8(w, red, total);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            int t = b + threadIdx.x * 8 + k;
            if (t < tiles) S.tileState[t] = (unsigned)(carry + excl + w[k]);
        }
        carry += total;
        __syncthreads(); // red is reused by the next chunk
    }
    if (threadIdx.x == 0) {
        S.start[cells] = carry;
        *done = 0;
    }
}

// Pass 2 for tile `tile` of S (256-thread block): start[] of its cells from
// its prefix, counts zeroed again for the next build.
__device__ __forceinline__ void grid_tile_scan(const VmPointSet &S, int tile)
{
    __shared__ int ws[24];
    int cells = grid_keys(S);
    int offset = (int)(unsigned)S.tileState[tile];
    int base = tile * kScanTile + threadIdx.x * 8;
    int v[8];
    grid_load8(S, base, cells, v, true);
    int total;
    int at = offset + block_scan8(v, ws, total);
    // read by this tile only, by every thread before the scan's barriers:
    // zero for the next scan
    if (threadIdx.x == 0) S.tileState[tile] = 0;
    if (base + 8 <= cells) {
        int4 *o = reinterpret_cast<int4 *>(S.start + base);
        o[0] = make_int4(at + v[0], at + v[1], at + v[2], at + v[3]);
        o[1] = make_int4(at + v[4], at + v[5], at + v[6], at + v[7]);
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (base + k < cells) S.start[base + k] = at + v[k];
    }
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
