// Phase-grid parallel Poisson-disk dart throwing (reference poisson_disk.cu:74-177,
// after Wei 2008).
//
// The background grid has cell size r/sqrt(2), so a cell holds at most one
// sample and a dart can only conflict with the 5x5 block around its cell.
// Cells are coloured by (x mod 3, y mod 3) relative to the region origin;
// cells of one colour are >= 3 apart and never see each other's writes, so a
// colour phase is race-free. Each round runs the 9 phases in the reference's
// order (py outer, px inner) and draws darts from a stateless hash of
// (cell, round, seed), which makes the sample set a deterministic function of
// the inputs and the sequence of regions resampled.
//
// Each phase is one launch over the phase cells of the region; a small
// region (every phase in one pass of a block) runs as one block-wide launch.
#include <algorithm>

#include "vm_device.cuh"
#include "vm_kernels.h"

namespace vmk {

// Dart coordinate stream `stream` of a round: the per-round part of the hash
// chain, computed once per launch on the host.
__host__ __device__ __forceinline__ unsigned round_key(unsigned round, unsigned seed, unsigned stream)
{
    return pcg_hash(round * 2654435761u ^ pcg_hash(seed + stream * 0x9E3779B9u));
}

// uniform [0,1) of (cell, round, seed, stream): pcg_hash(cell ^ round_key)
__device__ __forceinline__ float prand01(unsigned cell, unsigned key)
{
    unsigned h = pcg_hash(cell ^ key);
    return (float)(h & 0x00FFFFFFu) * (1.0f / 16777216.0f);
}

// The 5x5 block around a cell without the cell itself, by distance.
__constant__ signed char kRingDx[24] = {0, -1, 1, 0, -1, 1, -1, 1, 0, -2, 2, 0, -1, 1, -2, 2, -2, 2, -1, 1, -2, 2, -2, 2};
__constant__ signed char kRingDy[24] = {-1, 0, 0, 1, -1, -1, 1, 1, -2, 0, 0, 2, -2, -2, -1, -1, 1, 1, 2, 2, -2, -2, 2, 2};

// True if any of the N staged neighbours (q.x < 0: an empty cell) is nearer
// than r to the dart (x, y).
template <int N>
__device__ __forceinline__ bool any_conflict(const float2 (&q)[N], float x, float y, float r2)
{
    bool hit = false;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        float dx = q[k].x - x, dy = q[k].y - y;
        hit |= q[k].x >= 0.0f && dx * dx + dy * dy < r2;
    }
    return hit;
}

// Neighbours of an interior cell loaded per batch (nearest first): the own
// cell with the first kFirstBatch, then batches of kBatch.
constexpr int kFirstBatch = 8, kBatch = 4;
static_assert((24 - kFirstBatch) % kBatch == 0, "the rest splits into whole batches");

// One dart for cell (cx, cy) (reference dartPhaseKernel :84-106).
__device__ __forceinline__ void dart(float2 *grid, const PdParams &p, int cx, int cy, unsigned keyX, unsigned keyY)
{
    int cellId = cy * p.gridW + cx;
    float r2 = p.radius * p.radius;
    if (cx >= 2 && cy >= 2 && cx < p.gridW - 2 && cy < p.gridH - 2) {
        // an interior cell: every neighbour is in the grid, and no address
        // depends on a loaded value, so the cell and its 8 nearest
        // neighbours are loaded as one batch, then the 16 at distance 2 in
        // batches of kBatch, each only if no earlier neighbour conflicts
        // (the dart lands only if none conflicts, whatever the order)
        const int dxs[24] = {0, -1, 1, 0, -1, 1, -1, 1, 0, -2, 2, 0, -1, 1, -2, 2, -2, 2, -1, 1, -2, 2, -2, 2};
        const int dys[24] = {-1, 0, 0, 1, -1, -1, 1, 1, -2, 0, 0, 2, -2, -2, -1, -1, 1, 1, 2, 2, -2, -2, 2, 2};
        const float2 *c = grid + cellId;
        const int W = p.gridW;
        float2 own = c[0];
        float2 q1[kFirstBatch];
#pragma unroll
        for (int k = 0; k < kFirstBatch; ++k) q1[k] = c[dys[k] * W + dxs[k]];
        if (own.x >= 0.0f) return;
        float x = ((float)cx + prand01((unsigned)cellId, keyX)) * p.cellSize;
        float y = ((float)cy + prand01((unsigned)cellId, keyY)) * p.cellSize;
        if (x >= p.width || y >= p.height) return;
        if (any_conflict(q1, x, y, r2)) return;
#pragma unroll
        for (int b = kFirstBatch; b < 24; b += kBatch) {
            float2 q2[kBatch];
#pragma unroll
            for (int k = 0; k < kBatch; ++k) q2[k] = c[dys[b + k] * W + dxs[b + k]];
            if (any_conflict(q2, x, y, r2)) return;
        }
        grid[cellId] = make_float2(x, y);
        return;
    }
    if (grid[cellId].x >= 0.0f) return;
    float x = ((float)cx + prand01((unsigned)cellId, keyX)) * p.cellSize;
    float y = ((float)cy + prand01((unsigned)cellId, keyY)) * p.cellSize;
    if (x >= p.width || y >= p.height) return;
    // the 24 neighbours nearest first, so most rejected darts stop early
#pragma unroll 4
    for (int k = 0; k < 24; ++k) {
        int nx = cx + kRingDx[k], ny = cy + kRingDy[k];
        if (nx < 0 || nx >= p.gridW || ny < 0 || ny >= p.gridH) continue;
        float2 q = grid[ny * p.gridW + nx];
        if (q.x < 0.0f) continue;
        float dx = q.x - x, dy = q.y - y;
        if (dx * dx + dy * dy < r2) return;
    }
    grid[cellId] = make_float2(x, y);
}

__global__ void __launch_bounds__(256) k_clear(float2 *grid, int gridW, int x0, int y0, int x1, int y1)
{
    int rw = x1 - x0;
    long long n = (long long)rw * (y1 - y0);
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int cx = x0 + (int)(t % rw), cy = y0 + (int)(t / rw);
        grid[(size_t)cy * gridW + cx] = make_float2(-1.0f, -1.0f);
    }
}

// One phase (px, py) of one round, one thread per phase cell: x across the
// threads of a block row, phase rows over blockIdx.y.
//
// Launched as a programmatic dependent of the previous phase: the hardware
// wait below returns once that phase has completed and its writes are
// visible, and the early trigger lets the next phase's launch overlap this
// one's tail. Without the launch attribute both instructions are no-ops.
__global__ void __launch_bounds__(256) k_phase(float2 *grid, PdParams p, int x0, int y0, int x1, int y1, int px,
                                               int py, unsigned keyX, unsigned keyY)
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    int tw = (x1 - x0 - px + 2) / 3, th = (y1 - y0 - py + 2) / 3;
    int tx = blockIdx.x * blockDim.x + threadIdx.x;
    if (tx >= tw) return;
    for (int ty = blockIdx.y; ty < th; ty += gridDim.y)
        dart(grid, p, x0 + 3 * tx + px, y0 + 3 * ty + py, keyX, keyY);
}

// A whole resample of a small region in one block: the clear, then every
// round's 9 phases separated by block barriers (the same order as the
// one-launch-per-phase path, so the same samples). It replaces 1 + 9 x trials
// launches by one when every phase fits in one pass of the block. The region
// and its 2-cell halo are staged in shared memory for all the phases (the
// halo is only read: no dart outside the region is thrown), and the region
// is written back at the end.
constexpr int kSmallBlock = 1024;
// The largest staged region: (3a + 4)(3b + 4) cells for ab <= kSmallBlock
// phase cells, at most 21,532 (a = 1, b = 1024), as float2.
constexpr int kMaxStageBytes = 21532 * 8;

// One dart (dart above) against the staged copy, tested by a group of 4
// lanes (gmask: the group's lanes of the warp, all active together; sub: this
// lane's place in it). s holds the cells of the rectangle at (hx0, hy0) with
// row length lw; every neighbour of a region cell lies in it, and cells
// outside the grid hold the empty marker, so no bounds test is needed. Each
// lane tests 6 of the 24 neighbours; the dart lands if no lane finds a
// conflict, which does not depend on the order of the tests.
__device__ __forceinline__ void dart_staged(float2 *s, int lw, int hx0, int hy0, const PdParams &p, int cx, int cy,
                                            unsigned keyX, unsigned keyY, int sub, unsigned gmask)
{
    int li = (cy - hy0) * lw + (cx - hx0);
    int cellId = cy * p.gridW + cx;
    float x = ((float)cx + prand01((unsigned)cellId, keyX)) * p.cellSize;
    float y = ((float)cy + prand01((unsigned)cellId, keyY)) * p.cellSize;
    bool ok = s[li].x < 0.0f && x < p.width && y < p.height; // the same for the group
    float r2 = p.radius * p.radius;
    bool hit = false;
    if (ok) {
#pragma unroll
        for (int k = sub; k < 24; k += 4) {
            float2 q = s[li + kRingDy[k] * lw + kRingDx[k]];
            float dx = q.x - x, dy = q.y - y;
            hit |= q.x >= 0.0f && dx * dx + dy * dy < r2;
        }
    }
    if (__ballot_sync(gmask, hit) == 0u && ok && sub == 0) s[li] = make_float2(x, y);
}

__device__ __forceinline__ void resample_block(float2 *grid, const PdParams &p, int x0, int y0, int x1, int y1,
                                               int trials, unsigned roundBase, float2 *s)
{
    int rw = x1 - x0, rh = y1 - y0, lw = rw + 4, lh = rh + 4, hx0 = x0 - 2, hy0 = y0 - 2;
    // the region cleared, the halo copied (cells outside the grid stay empty)
    for (int t = threadIdx.x; t < lw * lh; t += blockDim.x) {
        int gx = hx0 + t % lw, gy = hy0 + t / lw;
        bool region = gx >= x0 && gx < x1 && gy >= y0 && gy < y1;
        bool inGrid = gx >= 0 && gx < p.gridW && gy >= 0 && gy < p.gridH;
        s[t] = !region && inGrid ? grid[(size_t)gy * p.gridW + gx] : make_float2(-1.0f, -1.0f);
    }
    __syncthreads();
    for (int round = 0; round < trials; ++round) {
        unsigned r = roundBase + (unsigned)round;
        unsigned kx = round_key(r, p.seed, 0u), ky = round_key(r, p.seed, 1u);
        for (int py = 0; py < 3; ++py)
            for (int px = 0; px < 3; ++px) {
                int tw = (rw - px + 2) / 3, th = (rh - py + 2) / 3;
                // 4 lanes per dart: the groups are aligned 4-lane slices of a warp
                unsigned gmask = 0xFu << (threadIdx.x & 28u);
                for (int t = threadIdx.x; t < 4 * tw * th; t += blockDim.x) {
                    int d = t >> 2;
                    dart_staged(s, lw, hx0, hy0, p, x0 + 3 * (d % tw) + px, y0 + 3 * (d / tw) + py, kx, ky, t & 3,
                                gmask);
                }
                __syncthreads(); // the next phase sees this phase's samples
            }
    }
    for (int t = threadIdx.x; t < rw * rh; t += blockDim.x) {
        int lx = t % rw, ly = t / rw;
        grid[(size_t)(y0 + ly) * p.gridW + x0 + lx] = s[(ly + 2) * lw + lx + 2];
    }
}

__global__ void __launch_bounds__(kSmallBlock) k_resample_block(float2 *grid, PdParams p, int x0, int y0, int x1,
                                                                 int y1, int trials, unsigned roundBase)
{
    extern __shared__ float2 sStage[];
    resample_block(grid, p, x0, y0, x1, y1, trials, roundBase, sStage);
}

// Many samplers' small regions in one launch, one block each (the samplers'
// grids are disjoint, so the blocks are independent).
__global__ void __launch_bounds__(kSmallBlock) k_resample_many(const PdJob *__restrict__ jobs)
{
    extern __shared__ float2 sStage[];
    PdJob j = jobs[blockIdx.x];
    resample_block(j.grid, j.p, j.x0, j.y0, j.x1, j.y1, j.trials, j.roundBase, sStage);
}

// The cells of each job's region, packed row by row at out + offsets[job]
// (one block per job): one copy to the host serves every region.
__global__ void __launch_bounds__(256) k_gather_regions(const PdJob *__restrict__ jobs, const int *__restrict__ offsets,
                                                        float2 *__restrict__ out)
{
    PdJob j = jobs[blockIdx.x];
    int w = j.x1 - j.x0, cells = w * (j.y1 - j.y0);
    float2 *o = out + offsets[blockIdx.x];
    for (int c = threadIdx.x; c < cells; c += blockDim.x) {
        int y = j.y0 + c / w, x = j.x0 + c % w;
        o[c] = j.grid[(size_t)y * j.p.gridW + x];
    }
}

} // namespace vmk

using namespace vmk;

cudaError_t pd_launch_gather_regions(const PdJob *jobs, const int *offsets, int n, float2 *out, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    k_gather_regions<<<n, 256, 0, s>>>(jobs, offsets, out);
    return cudaGetLastError();
}

// The one-block resamples stage up to kMaxStageBytes of shared memory (set
// once per device).
static cudaError_t stage_attributes()
{
    static bool done[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_resample_block, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxStageBytes)) ||
        (e = cudaFuncSetAttribute(k_resample_many, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxStageBytes)))
        return e;
    if (dev >= 0 && dev < 64) done[dev] = true;
    return cudaSuccess;
}

cudaError_t pd_launch_resample(float2 *grid, PdParams p, int x0, int y0, int x1, int y1, int trials,
                               unsigned roundBase, cudaStream_t s, bool dependentLaunch)
{
    int rw = x1 - x0, rh = y1 - y0;
    if (rw <= 0 || rh <= 0) return cudaSuccess;
    long long cells = (long long)rw * rh;
    long long phaseCells = (long long)((rw + 2) / 3) * ((rh + 2) / 3);
    if (phaseCells <= kSmallBlock) {
        cudaError_t e = stage_attributes();
        if (e) return e;
        size_t smem = pd_stage_bytes(x0, y0, x1, y1);
        k_resample_block<<<1, kSmallBlock, smem, s>>>(grid, p, x0, y0, x1, y1, trials, roundBase);
        return cudaGetLastError();
    }
    int cb = (int)((cells + 255) / 256);
    if (cb > 65535) cb = 65535;
    k_clear<<<cb, 256, 0, s>>>(grid, p.gridW, x0, y0, x1, y1);
    dim3 pb((unsigned)((rw + 2) / 3 + 255) / 256, (unsigned)std::min((rh + 2) / 3, 65535));
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = pb;
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = dependentLaunch ? 1 : 0;
    for (int round = 0; round < trials; ++round) {
        unsigned r = roundBase + (unsigned)round;
        unsigned kx = round_key(r, p.seed, 0u), ky = round_key(r, p.seed, 1u);
        for (int py = 0; py < 3; ++py)
            for (int px = 0; px < 3; ++px) {
                cudaError_t e = cudaLaunchKernelEx(&cfg, k_phase, grid, p, x0, y0, x1, y1, px, py, kx, ky);
                if (e) return e;
            }
    }
    return cudaGetLastError();
}

int pd_small_region(int x0, int y0, int x1, int y1)
{
    long long phaseCells = (long long)((x1 - x0 + 2) / 3) * ((y1 - y0 + 2) / 3);
    return x1 > x0 && y1 > y0 && phaseCells <= kSmallBlock;
}

size_t pd_stage_bytes(int x0, int y0, int x1, int y1)
{
    return sizeof(float2) * (size_t)(x1 - x0 + 4) * (size_t)(y1 - y0 + 4);
}

cudaError_t pd_launch_resample_many(const PdJob *jobs, int n, size_t stageBytes, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    if (stageBytes > (size_t)kMaxStageBytes) return cudaErrorInvalidValue;
    cudaError_t e = stage_attributes();
    if (e) return e;
    k_resample_many<<<n, kSmallBlock, stageBytes, s>>>(jobs);
    return cudaGetLastError();
}
