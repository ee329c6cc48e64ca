// Host-side launch wrappers of the VoroMesh kernels (internal to the library).
#pragma once

#include <cuda_runtime.h>

#include "vm_types.h"

cudaError_t vm_launch_bin(const VmPointSet *sets, const int *prefix, int nSets, int totalBlocks, int emptyIsNegative,
                          cudaStream_t s);
// Exclusive scan of each set's cell counts into start[] (counts zeroed again),
// two launches. Each set's tileState holds one word per scan tile and a done
// counter after them, all zero before the first scan (every scan leaves them
// zero, so the buffer also serves later scans of fewer tiles); launches
// sharing a set's tileState are stream-ordered.
cudaError_t vm_launch_scan(const VmPointSet *sets, const int *tilePrefix, int nSets, int totalTiles, cudaStream_t s);
cudaError_t vm_launch_scatter(const VmPointSet *sets, const int *prefix, int nSets, int totalBlocks,
                              const VmFit *publish, cudaStream_t s);
// Sorts each cell's run by point index (sets with canonical = 0 are skipped);
// one block per scan tile, the same tile prefix as vm_launch_scan.
cudaError_t vm_launch_canonical(const VmPointSet *sets, const int *tilePrefix, int nSets, int totalTiles,
                                cudaStream_t s);
// The loss pass is two launches: the block-certified fast path over all
// targets, then the exact ring search over the targets it deferred to the
// queue (created by vm_queue_init; items hold (fit, target) int2 pairs).
// `variant` picks block size and occupancy target; its block size is also the
// number of targets per tile the prefix table counts. With `windowed`, every
// fit has a window list (VmFit::twin) and a tile is block size / 32 windows.
cudaError_t vm_launch_loss(const VmFit *fits, const int *tilePrefix, int nFits, int totalTiles, int mode,
                           int gridBlocks, int variant, int windowed, void *queue, cudaStream_t s);
// The loss windows of a fit's cell-sorted targets (VmFit::twin): each grid
// cell's run split into windows of at most 32. tstart holds the target sort's
// key starts (cells << 2 sub keys); winSet is a device VmPointSet over `cells`
// keys (counts, start, tileState of tiles + 1 words) and winPre its tile
// prefix {0, tiles}; twin needs room for start[cells] + 1 entries, at most
// live / 32 + min(cells, live) + 1.
cudaError_t vm_launch_target_windows(const int *tstart, int cells, int sub, const VmPointSet *winSet,
                                     const int *winPre, int tiles, int *counts, const int *start, int *twin,
                                     cudaStream_t s);
int vm_loss_variants();
int vm_loss_variant_threads(int variant);
// A fit of at most 4,096 slots and 8,192 grid cells can end its step in one
// block after vm_launch_loss_fast: the deferred targets and Adam schedule,
// Adam, binning, scan and scatter (in place of the exact pass of
// vm_launch_loss, vm_launch_adam_bin, vm_launch_scan and vm_launch_scatter
// with publish), for the one fit of the table `fit`.
bool vm_small_grid_fits(int slots, int cells);
cudaError_t vm_launch_small_grid(const VmFit *fit, void *queue, cudaStream_t s);
// The fast path of vm_launch_loss alone (a step pass; its deferred targets
// and schedule are left to vm_launch_small_grid).
cudaError_t vm_launch_loss_fast(const VmFit *fits, const int *tilePrefix, int nFits, int totalTiles, int gridBlocks,
                                int variant, int windowed, void *queue, cudaStream_t s);
cudaError_t vm_launch_finalize(const VmFit *fits, int nFits, void *queue, cudaStream_t s);
cudaError_t vm_launch_adam_bin(const VmFit *fits, const int *prefix, int nFits, int totalBlocks, void *queue,
                               cudaStream_t s);
cudaError_t vm_queue_init(void *queue, void *items, int capacity, cudaStream_t s);
size_t vm_queue_bytes();
cudaError_t vm_launch_knn(const VmFit *fit, const float2 *q, int nq, int K, int *outIdx, float *outD2,
                          cudaStream_t s);
int vm_loss_occupancy_blocks(int variant);
cudaError_t vm_launch_scatter_targets(float2 *targets, const int *slots, const float2 *values, int n, cudaStream_t s);
// The largest target count of any 5x5 block of cells (*out, device int) from
// a target sort's key starts (sub-cell depth sub), and the fit's fastShift
// from it: 38 - ceil(log2 block5Max), so 2^(fastShift + 24) * block5Max <= 2^62.
cudaError_t vm_launch_block5_max(const int *tstart, int gridW, int gridH, int sub, int *out, cudaStream_t s);
int vm_fast_shift(int block5Max);

// Voronoi cells for extraction (vm_extract.cu); vm_launch_compact_cells packs
// the fixed-size cell slots into CSR order (start: n + 1 offsets).
cudaError_t vm_launch_cells_n(const VmFit *fit, int nSlots, const unsigned long long *masks, int tilesX, int tilesY,
                              float invVoxel, float2 *outVerts, int *outEdges, int *outCount,
                              unsigned char *outInside, int *flags, cudaStream_t s);
cudaError_t vm_launch_compact_cells(const float2 *verts, const int *labels, const int *start, int n, float2 *outV,
                                    int *outL, cudaStream_t s);
// Boundary assembly on the device, in phases: 0 counts each inside cell's
// boundary edges (cnt); 1 emits their vertex keys into the hash table
// (keys/minPos, capacity mask + 1) with eStart = scanned counts; 2 flags the
// first occurrences (first); after an exclusive scan of `first`, 3 numbers
// the vertices and writes edges (2 per boundary edge) and vertex positions.
cudaError_t vm_launch_boundary(int n, const int *start, const int *labels, const float2 *verts,
                               const unsigned char *inside, int *cnt, int phase, const int *eStart,
                               unsigned long long *keys, unsigned mask, int *minPos, unsigned *occSlot, float2 *occPt,
                               int occ, int *first, int *edges, float2 *vertices, int *err, cudaStream_t s);
// Exclusive scan of n ints (out[n] = total; in == out allowed); `partial`
// holds vm_scan_partials(n) ints.
cudaError_t vm_scan_ex(const int *in, int *out, int n, int *partial, cudaStream_t s);
int vm_scan_partials(int n);

// Poisson phase-grid sampler (vm_poisson.cu)
struct PdParams {
    float width, height, radius, cellSize;
    int gridW, gridH;
    unsigned seed;
};
// dependentLaunch: each phase launch a programmatic dependent of the one before
cudaError_t pd_launch_resample(float2 *grid, PdParams p, int x0, int y0, int x1, int y1, int trials,
                               unsigned roundBase, cudaStream_t s, bool dependentLaunch);
// One sampler's region resample for pd_launch_resample_many.
struct PdJob {
    float2 *grid;
    PdParams p;
    int x0, y0, x1, y1, trials;
    unsigned roundBase;
};
// The jobs' regions packed into out, job k's row-major cells at offsets[k]
// (jobs and offsets in device memory).
cudaError_t pd_launch_gather_regions(const PdJob *jobs, const int *offsets, int n, float2 *out, cudaStream_t s);
// 1 when the region runs as one block (every phase in one pass of it).
int pd_small_region(int x0, int y0, int x1, int y1);
// Small regions of distinct samplers (jobs in device memory), one block each.
// stageBytes: the largest pd_stage_bytes among the jobs' regions (the staged
// region and halo size the launch's shared memory).
size_t pd_stage_bytes(int x0, int y0, int x1, int y1);
cudaError_t pd_launch_resample_many(const PdJob *jobs, int n, size_t stageBytes, cudaStream_t s);
