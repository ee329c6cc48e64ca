// Device-resident Canvas: RasterizeShape and StampDisc of the reference's
// voromesh::Canvas (src/voromesh/canvas.cpp:71-221) as CUDA kernels, behind
// the cv_* C ABI (include/vm_capi.h).
//
// Layout in HBM (tiles = tilesX * tilesY, 8x8 voxels per tile):
//   inside  u64[tiles]        occupancy, the reference's InsideMasks layout
//   smask   u64[tiles]        surface voxels
//   spt     float2[tiles*64]  surface point of each voxel (tile-major)
//   sslot   int[tiles*64]     its target slot
//   slots   float2[cap]       the target slot array (TargetSlots)
//   freel   int[cap]          the free-slot stack
// The surface is dense per voxel instead of the reference's hash map of
// tiles: 12 bytes a voxel buys O(1) addressing with no hashing.
//
// Arithmetic follows the reference literally (IEEE float, no contraction;
// the library is built with --fmad=false). Per-voxel means are double sums
// of float samples; the reference adds them in sample order. Every sample of
// a voxel is an integer multiple of the quantum Q of its smallest one; when
// their magnitudes sum to at most 2^52 Q, every partial sum in any order is
// an integer multiple of Q below 2^53 Q, hence exact in double, so the
// reference's sum is exactly the integer sum of the multiples times Q. That
// integer sum is taken here (64-bit integers, no FP64 pipe in the loop).
// Voxels without the certificate (samples of wildly different magnitude) are
// summed again in double in sample order by one lane.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "vm_capi.h"
#include "vm_host.h"
#include "vm_kernels.h"

using vmh::cuda_fail;
using vmh::DevBuf;
using vmh::fail;

namespace {

constexpr int kScanChunk = 2048;  // elements per block of the multi-block scan
constexpr int kChunk = 1024;      // polygon vertices staged per pass of the scanline kernel
constexpr int kRowCap = 512;      // crossings a warp sorts for one scanline
constexpr int kBigCap = 32768;    // crossings one block sorts for one scanline
constexpr int kMaxVoxelsX = 131072;
constexpr int kBigBlocks = 32;
constexpr int kListBlocks = 1024; // blocks of the tile work-list kernels (8 warps each)
constexpr int kMaxBucketEntries = 1 << 27; // beyond this the scanline kernels test every edge
constexpr int kMaxRimSamples = 1 << 28;    // rim samples of one stamp (radius / voxel size < 10.6M)

enum { kErrSamples = 1, kErrCrossings = 2, kErrRimBox = 4 };

struct CvState {
    int nslots, nfree, surfaceTiles, err;
    long long surfaceCount;
    unsigned long long totalSamples;
    int edgeEntries; // entries of the per-tile-row edge buckets
    int listCount;   // tiles with samples (k_cv_tile_means work list)
    // last edit
    int removed, added, flipped, ndirty;
    int overflowRows;
    // values before the edit, kept for its later kernels
    int nslots0, nfree0, freeAfterPush;
};

struct CvGeom {
    int vx, vy, tilesX, tilesY;
    float vs, inv;
};

struct CvStamp {
    float cx, cy, r2;
    int inside;
    int i0, j0, i1, j1; // voxel box, clamped to the domain
    int bx0, by0, bw, bh; // its tiles
    int nRim;
};

__device__ __forceinline__ int bit_of(int i, int j) { return ((j & 7) << 3) | (i & 7); }

__device__ __forceinline__ unsigned long long lower_bits(int b) { return (1ull << b) - 1ull; }

// ---------------------------------------------------------------------------
// exclusive scans of int arrays: out[0..n] (out[n] = total); in-place allowed
// ---------------------------------------------------------------------------
__device__ int block_exclusive_scan(int v, int *sm, int &total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sm[w] = x;
    __syncthreads();
    if (w == 0) {
        int s = lane < nw ? sm[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        sm[lane] = s;
    }
    __syncthreads();
    total = sm[nw - 1];
    int ex = x - v + (w > 0 ? sm[w - 1] : 0);
    __syncthreads();
    return ex;
}

constexpr int kPerThread = 8; // elements a thread scans serially per pass of a single-block scan

__global__ void __launch_bounds__(1024) k_scan_single(const int *in, int *out, int n)
{
    __shared__ int sm[32];
    int carry = 0;
    for (int base = 0; base < n; base += 1024 * kPerThread) {
        int i0 = base + threadIdx.x * kPerThread;
        int v[kPerThread], sum = 0;
#pragma unroll
        for (int k = 0; k < kPerThread; ++k) {
            v[k] = i0 + k < n ? in[i0 + k] : 0;
            sum += v[k];
        }
        int tot;
        int run = carry + block_exclusive_scan(sum, sm, tot);
#pragma unroll
        for (int k = 0; k < kPerThread; ++k) {
            if (i0 + k < n) out[i0 + k] = run;
            run += v[k];
        }
        carry += tot;
    }
    if (threadIdx.x == 0) out[n] = carry;
}

__global__ void __launch_bounds__(1024) k_scan_reduce(const int *in, int n, int *partial)
{
    __shared__ int sm[32];
    int i0 = blockIdx.x * kScanChunk + 2 * threadIdx.x;
    int v = (i0 < n ? in[i0] : 0) + (i0 + 1 < n ? in[i0 + 1] : 0);
    int tot;
    block_exclusive_scan(v, sm, tot);
    if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_scan_apply(const int *in, int *out, int n, const int *partialEx)
{
    __shared__ int sm[32];
    int i0 = blockIdx.x * kScanChunk + 2 * threadIdx.x;
    int v0 = i0 < n ? in[i0] : 0, v1 = i0 + 1 < n ? in[i0 + 1] : 0;
    int tot;
    int ex = block_exclusive_scan(v0 + v1, sm, tot) + partialEx[blockIdx.x];
    if (i0 < n) out[i0] = ex;
    if (i0 + 1 < n) out[i0 + 1] = ex + v0;
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = partialEx[blockIdx.x] + tot;
}

// three scans of the same length in one block (stamp tile lists are short)
__global__ void __launch_bounds__(1024) k_scan3_single(int *a, int *b, int *c, int n, CvState *st)
{
    __shared__ int sm[32];
    int ca = 0, cb = 0, cc = 0;
    constexpr int P = 8;
    for (int base = 0; base < n; base += 1024 * P) {
        int i0 = base + threadIdx.x * P;
        int va[P], vb[P], vc[P], sa = 0, sb = 0, sc = 0;
#pragma unroll
        for (int k = 0; k < P; ++k) {
            bool in = i0 + k < n;
            va[k] = in ? a[i0 + k] : 0;
            vb[k] = in ? b[i0 + k] : 0;
            vc[k] = in ? c[i0 + k] : 0;
            sa += va[k];
            sb += vb[k];
            sc += vc[k];
        }
        int ta, tb, tc;
        int ra = ca + block_exclusive_scan(sa, sm, ta);
        int rb = cb + block_exclusive_scan(sb, sm, tb);
        int rc = cc + block_exclusive_scan(sc, sm, tc);
#pragma unroll
        for (int k = 0; k < P; ++k) {
            if (i0 + k < n) {
                a[i0 + k] = ra;
                b[i0 + k] = rb;
                c[i0 + k] = rc;
            }
            ra += va[k];
            rb += vb[k];
            rc += vc[k];
        }
        ca += ta;
        cb += tb;
        cc += tc;
    }
    if (threadIdx.x == 0) {
        a[n] = ca;
        b[n] = cb;
        c[n] = cc;
        // a = removed, b = rim voxels, c = rim voxels that need a slot
        int R = ca, M = cb, A = cc;
        int nfree0 = st->nfree, nslots0 = st->nslots;
        int F = nfree0 + R; // free-list length once the removed slots are pushed
        st->nfree0 = nfree0;
        st->nslots0 = nslots0;
        st->freeAfterPush = F;
        st->removed = R;
        st->added = A;
        st->ndirty = R + M;
        st->nfree = F > A ? F - A : 0;
        st->nslots = nslots0 + (A > F ? A - F : 0);
        st->surfaceCount += (long long)A - R;
    }
}

// ---------------------------------------------------------------------------
// per-voxel means of a tile's samples (shared by RasterizeShape and StampDisc)
// ---------------------------------------------------------------------------
// The samples of one voxel's run (record indices run[0..n)) summed in
// double in sample order (canvas.cpp:13-25 adds them so): repeated selection
// of the next sample index, for the short runs one lane reduces.
__device__ __noinline__ void ordered_sum(const float4 *rec, const int *run, int n, double &sx, double &sy)
{
    sx = 0.0;
    sy = 0.0;
    int last = -1;
    for (int k = 0; k < n; ++k) {
        int best = INT_MAX;
        float bx = 0.0f, by = 0.0f;
        for (int r = 0; r < n; ++r) {
            float4 q = rec[run[r]];
            int id = __float_as_int(q.z);
            if (id > last && id < best) {
                best = id;
                bx = q.x;
                by = q.y;
            }
        }
        sx += (double)bx;
        sy += (double)by;
        last = best;
    }
}

// Sorts a long run (record indices) by sample index in place, by the whole
// warp: a bitonic network over the next power of two P >= n in which every
// merge of two sorted blocks opens with the comparators (i, i ^ (k - 1)),
// so that every comparator puts the smaller key first. A comparator whose
// upper position is at or past n is skipped: that is the same network on
// the run padded with +inf keys, which never move. log2(P) (log2(P) + 1) / 2
// stages of P / 2 comparators, 32 a warp step; __syncwarp orders the
// stages' global loads and stores.
__device__ __noinline__ void warp_sort_run(const float4 *__restrict__ rec, int *run, int n)
{
    const int lane = threadIdx.x & 31;
    int P = 1;
    while (P < n) P <<= 1;
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < (P >> 1); i += 32) {
                const int a = ((i & ~(j - 1)) << 1) | (i & (j - 1)); // bit j of a is clear
                const int b = j == (k >> 1) ? a ^ (k - 1) : a | j;
                if (b < n) {
                    const int ra = run[a], rb = run[b];
                    if (__float_as_int(rec[rb].z) < __float_as_int(rec[ra].z)) {
                        run[a] = rb;
                        run[b] = ra;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// The same sum over a run already in sample order.
__device__ __noinline__ void in_order_sum(const float4 *rec, const int *run, int n, double &sx, double &sy)
{
    sx = 0.0;
    sy = 0.0;
    for (int k = 0; k < n; ++k) {
        const float4 q = rec[run[k]];
        sx += (double)q.x;
        sy += (double)q.y;
    }
}

// Split of a float into sign, integer significand M and exponent e with
// |v| = M * 2^(e - 150) (e = 1 for subnormals).
__device__ __forceinline__ void float_split(float v, bool &neg, unsigned &M, int &e)
{
    unsigned u = __float_as_uint(v);
    neg = (u >> 31) != 0;
    int be = (int)((u >> 23) & 0xFFu);
    M = u & 0x7FFFFFu;
    if (be) M |= 0x800000u;
    e = be > 0 ? be : 1;
}

// Exact mean of one voxel whose records are rec[run[k]], k < n.
// Every sample is an integer multiple of Q = 2^(e0 - 150), where e0 is the
// smallest exponent among the tile's non-zero samples (per axis). When the
// voxel's magnitudes sum to at most 2^52 Q, every partial sum of its samples
// in any order is an integer multiple of Q below 2^53 Q, hence exact in
// double: the reference's sample-order double sum (canvas.cpp:13-25) equals
// the 64-bit integer sum of the multiples times Q. Otherwise the samples are
// summed in double in sample order.
//
// A term is at most 2^52 (M < 2^24 shifted by at most 28), and accumulation
// stops as soon as a magnitude sum passes 2^52: every sum stays below 2^53,
// so none can wrap, however many samples a voxel holds.
struct RunSums {
    long long sx = 0, sy = 0;
    unsigned long long ax = 0, ay = 0;
    bool big = false;
    __device__ void add_axis(float v, int e0, long long &s, unsigned long long &a)
    {
        bool sg;
        unsigned M;
        int e;
        float_split(v, sg, M, e);
        if (!M || big) return;
        const int sh = e - e0;
        if (sh > 28) {
            big = true;
            return;
        }
        const unsigned long long t = (unsigned long long)M << sh;
        s += sg ? -(long long)t : (long long)t;
        a += t;
        if (a > (1ull << 52)) big = true;
    }
    __device__ void add(const float4 &q, int ex, int ey)
    {
        add_axis(q.x, ex, sx, ax);
        add_axis(q.y, ey, sy, ay);
    }
    __device__ bool exact() const
    {
        const unsigned long long lim = 1ull << 52;
        return !big && ax <= lim && ay <= lim;
    }
    // sorted: the run is in sample order (a long run after warp_sort_run)
    __device__ float2 mean(const float4 *__restrict__ rec, const int *__restrict__ run, int n, int ex, int ey,
                           bool sorted) const
    {
        double x, y;
        if (exact()) {
            x = ex == INT_MAX ? 0.0 : ldexp((double)sx, ex - 150);
            y = ey == INT_MAX ? 0.0 : ldexp((double)sy, ey - 150);
        } else if (sorted) {
            in_order_sum(rec, run, n, x, y);
        } else {
            ordered_sum(rec, run, n, x, y);
        }
        return make_float2((float)(x / (double)n), (float)(y / (double)n));
    }
};

__device__ float2 voxel_mean(const float4 *__restrict__ rec, const int *__restrict__ run, int n, int ex, int ey)
{
    RunSums r;
    for (int k = 0; k < n; ++k) r.add(rec[run[k]], ex, ey);
    return r.mean(rec, run, n, ex, ey, false);
}

// The same for a long run, by the whole warp: lanes take every 32nd sample
// and the integer sums are combined exactly by shuffles; a run that fails
// the exact-sum bound is sorted into sample order by the warp (its order in
// run[] is otherwise arbitrary). Returns the mean on every lane.
__device__ float2 voxel_mean_warp(const float4 *__restrict__ rec, int *run, int n, int ex, int ey)
{
    const int lane = threadIdx.x & 31;
    RunSums r;
    for (int k = lane; k < n; k += 32) r.add(rec[run[k]], ex, ey);
    for (int o = 16; o > 0; o >>= 1) {
        r.sx += __shfl_xor_sync(0xffffffffu, r.sx, o);
        r.sy += __shfl_xor_sync(0xffffffffu, r.sy, o);
        r.ax += __shfl_xor_sync(0xffffffffu, r.ax, o);
        r.ay += __shfl_xor_sync(0xffffffffu, r.ay, o);
    }
    r.big = __any_sync(0xffffffffu, r.big);
    if (!r.exact()) warp_sort_run(rec, run, n); // the sums are the warp's totals: a uniform branch
    float2 m = make_float2(0.0f, 0.0f);
    if (lane == 0) m = r.mean(rec, run, n, ex, ey, true);
    m.x = __shfl_sync(0xffffffffu, m.x, 0);
    m.y = __shfl_sync(0xffffffffu, m.y, 0);
    return m;
}

constexpr int kLaneRun = 32; // longer voxel runs are reduced by the whole warp

// Counting sort of one tile's records by voxel (one set per warp).
struct TileSort {
    int cnt[64], off[64], fill[64];
};

// One warp per tile of the work list (the tiles that received samples, in
// any order); rec = (x, y, sample index, bit) in tile order (start[t] ..
// start[t+1]). The warp sorts the tile's records by voxel (perm, a scratch
// array as long as rec), then lane l reduces the runs of voxels l and l + 32
// (runs longer than kLaneRun: the whole warp).
// Writes the tile's mask, the mean of each of its voxels and the count of
// voxels. Tiles off the list keep the zero masks and counts they were
// cleared to.
__global__ void __launch_bounds__(256, 2) k_cv_tile_means(const int *__restrict__ list, const int *listCount,
                                                        const int *__restrict__ start, const float4 *__restrict__ rec,
                                                        int *__restrict__ perm,
                                                        unsigned long long *__restrict__ outMask,
                                                        float2 *__restrict__ outPt, int *__restrict__ outCount,
                                                        int *surfaceTiles)
{
    __shared__ TileSort sorts[8];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    TileSort &T = sorts[wib];
    const int nList = *listCount;
    for (int k = blockIdx.x * 8 + wib; k < nList; k += gridDim.x * 8) {
        const int tile = list[k];
        const int beg = start[tile], end = start[tile + 1];
        T.cnt[lane] = T.cnt[lane + 32] = 0;
        T.fill[lane] = T.fill[lane + 32] = 0;
        __syncwarp();
        int ex = INT_MAX, ey = INT_MAX;
        for (int r = beg + lane; r < end; r += 32) {
            const float4 q = rec[r];
            atomicAdd(&T.cnt[__float_as_int(q.w)], 1);
            bool sg;
            unsigned M;
            int e;
            float_split(q.x, sg, M, e);
            if (M) ex = min(ex, e);
            float_split(q.y, sg, M, e);
            if (M) ey = min(ey, e);
        }
        ex = __reduce_min_sync(0xffffffffu, ex);
        ey = __reduce_min_sync(0xffffffffu, ey);
        __syncwarp();
        // exclusive offsets of the 64 voxel runs
        const int c0 = T.cnt[lane], c1 = T.cnt[lane + 32];
        int i0 = c0, i1 = c1;
        for (int o = 1; o < 32; o <<= 1) {
            int y0 = __shfl_up_sync(0xffffffffu, i0, o), y1 = __shfl_up_sync(0xffffffffu, i1, o);
            if (lane >= o) {
                i0 += y0;
                i1 += y1;
            }
        }
        const int tot0 = __shfl_sync(0xffffffffu, i0, 31);
        T.off[lane] = i0 - c0;
        T.off[lane + 32] = tot0 + i1 - c1;
        __syncwarp();
        for (int r = beg + lane; r < end; r += 32) {
            const int b = __float_as_int(rec[r].w);
            perm[beg + T.off[b] + atomicAdd(&T.fill[b], 1)] = r;
        }
        __syncwarp();
        // runs of up to kLaneRun samples: one lane each; longer runs: the whole warp
        if (c0 > 0 && c0 <= kLaneRun)
            outPt[(size_t)tile * 64 + lane] = voxel_mean(rec, perm + beg + T.off[lane], c0, ex, ey);
        if (c1 > 0 && c1 <= kLaneRun)
            outPt[(size_t)tile * 64 + lane + 32] = voxel_mean(rec, perm + beg + T.off[lane + 32], c1, ex, ey);
        unsigned long long longRuns = (unsigned long long)__ballot_sync(0xffffffffu, c0 > kLaneRun) |
                                      ((unsigned long long)__ballot_sync(0xffffffffu, c1 > kLaneRun) << 32);
        while (longRuns) {
            const int b = __ffsll((long long)longRuns) - 1;
            longRuns &= longRuns - 1;
            const float2 m = voxel_mean_warp(rec, perm + beg + T.off[b], T.cnt[b], ex, ey);
            if (lane == 0) outPt[(size_t)tile * 64 + b] = m;
        }
        const unsigned long long mask = (unsigned long long)__ballot_sync(0xffffffffu, c0 > 0) |
                                        ((unsigned long long)__ballot_sync(0xffffffffu, c1 > 0) << 32);
        if (lane == 0) {
            outMask[tile] = mask;
            if (outCount) outCount[tile] = __popcll(mask);
            if (surfaceTiles && mask) atomicAdd(surfaceTiles, 1);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// RasterizeShape: surface samples (canvas.cpp:79-94)
// ---------------------------------------------------------------------------
__global__ void k_cv_seg_counts(const float2 *__restrict__ poly, int n, float step, int *__restrict__ cnt,
                                CvState *st)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    int m = 0;
    if (s < n) {
        float2 a = poly[s], b = poly[s + 1 == n ? 0 : s + 1];
        float dx = b.x - a.x, dy = b.y - a.y;
        // hypot: both squares are exact in double, so this is the correctly
        // rounded root of the exact sum, rounded once more to float
        float len = (float)sqrt((double)dx * (double)dx + (double)dy * (double)dy);
        float q = ceilf(len / step);
        if (q < 16777216.0f) {
            m = q > 1.0f ? (int)q : 1;
        } else {
            m = 1;
            atomicOr(&st->err, kErrSamples);
        }
        cnt[s] = m;
    }
    // the 64-bit total (the int scan must not overflow): one atomic per warp
    unsigned long long w = (unsigned long long)m;
    for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
    if ((threadIdx.x & 31) == 0 && w) atomicAdd(&st->totalSamples, w);
}

__device__ __forceinline__ bool voxel_of(float x, float y, const CvGeom &g, int &i, int &j)
{
    float fx = floorf(x * g.inv), fy = floorf(y * g.inv);
    // InDomain (canvas.h:59) on the float values: NaN and out-of-range fail
    if (!(fx >= 0.0f && fx < (float)g.vx && fy >= 0.0f && fy < (float)g.vy)) return false;
    i = (int)fx;
    j = (int)fy;
    return true;
}

__global__ void k_cv_samples(const float2 *__restrict__ poly, int n, const int *__restrict__ segStart, int total,
                             CvGeom g, int *__restrict__ tileCount, int *__restrict__ recTile,
                             int *__restrict__ recRank, float2 *__restrict__ recXY, int *__restrict__ list,
                             CvState *st)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int tile = -1;
    float x = 0.0f, y = 0.0f;
    if (idx < total) {
        // segment s: the last with segStart[s] <= idx
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (segStart[mid] <= idx) lo = mid;
            else hi = mid - 1;
        }
        int s = lo;
        int m = segStart[s + 1] - segStart[s], k = idx - segStart[s];
        float2 a = poly[s], b = poly[s + 1 == n ? 0 : s + 1];
        float t = (float)k / (float)m;
        x = a.x + t * (b.x - a.x);
        y = a.y + t * (b.y - a.y);
        int i, j;
        if (voxel_of(x, y, g, i, j)) tile = (j >> 3) * g.tilesX + (i >> 3);
    }
    // consecutive samples mostly share a tile: one atomic per tile and warp
    const unsigned grp = __match_any_sync(0xffffffffu, tile);
    const int leader = __ffs(grp) - 1;
    int base = 0;
    if (lane == leader && tile >= 0) {
        base = atomicAdd(&tileCount[tile], __popc(grp));
        if (base == 0) list[atomicAdd(&st->listCount, 1)] = tile;
    }
    base = __shfl_sync(0xffffffffu, base, leader);
    if (idx >= total) return;
    recTile[idx] = tile;
    if (tile < 0) return;
    recRank[idx] = base + __popc(grp & ((1u << lane) - 1u));
    recXY[idx] = make_float2(x, y);
}

__global__ void k_cv_scatter(int total, const int *__restrict__ recTile, const int *__restrict__ recRank,
                             const float2 *__restrict__ recXY, const int *__restrict__ tileStart, CvGeom g,
                             float4 *__restrict__ rec)
{
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    int t = recTile[idx];
    if (t < 0) return;
    float2 p = recXY[idx];
    int i = (int)floorf(p.x * g.inv), j = (int)floorf(p.y * g.inv);
    rec[tileStart[t] + recRank[idx]] = make_float4(p.x, p.y, __int_as_float(idx), __int_as_float(bit_of(i, j)));
}

// Slots in tile-major voxel order (canvas.cpp:96-114): slot = surface voxels
// before this one. One warp per tile of the work list.
__global__ void __launch_bounds__(256) k_cv_assign(const int *__restrict__ list, const int *listCount,
                                                    const unsigned long long *__restrict__ smask,
                                                    const int *__restrict__ surfStart, int nTiles,
                                                    const float2 *__restrict__ spt, int *__restrict__ sslot,
                                                    float2 *__restrict__ slots, CvState *st)
{
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->nslots = surfStart[nTiles];
        st->nfree = 0;
        st->surfaceCount = surfStart[nTiles];
    }
    const int nList = *listCount;
    for (int k = blockIdx.x * 8 + wib; k < nList; k += gridDim.x * 8) {
        const int tile = list[k];
        const unsigned long long mask = smask[tile];
        const int s0 = surfStart[tile];
        for (int b = lane; b < 64; b += 32) {
            if (!((mask >> b) & 1ull)) continue;
            int slot = s0 + __popcll(mask & lower_bits(b));
            size_t v = (size_t)tile * 64 + b;
            sslot[v] = slot;
            slots[slot] = spt[v];
        }
    }
}

// ---------------------------------------------------------------------------
// RasterizeShape: occupancy by even-odd scanline fill (canvas.cpp:116-133)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void set_span(unsigned *row, int i0, int i1)
{
    int w0 = i0 >> 5, w1 = i1 >> 5;
    for (int wd = w0; wd <= w1; ++wd) {
        int lo = wd == w0 ? (i0 & 31) : 0, hi = wd == w1 ? (i1 & 31) : 31;
        unsigned m = (hi == 31 ? 0xffffffffu : ((1u << (hi + 1)) - 1u)) & ~((1u << lo) - 1u);
        atomicOr(&row[wd], m);
    }
}

// Voxels [ceil(x0*inv - 0.5), floor(x1*inv - 0.5)] of one sorted crossing pair.
__device__ __forceinline__ void fill_pair(unsigned *row, float x0, float x1, const CvGeom &g)
{
    float lo = ceilf(x0 * g.inv - 0.5f), hi = floorf(x1 * g.inv - 0.5f);
    lo = fmaxf(lo, 0.0f);
    hi = fminf(hi, (float)(g.vx - 1));
    if (lo <= hi) set_span(row, (int)lo, (int)hi);
}

__device__ __forceinline__ float crossing(float2 a, float2 b, float y)
{
    return a.x + (y - a.y) * (b.x - a.x) / (b.y - a.y);
}

// Tile rows whose scanlines edge (a, b) can cross: rows j with centre
// (j + 0.5) * vs between the edge's end ordinates, widened by one row each
// way for rounding. Horizontal edges cross none.
__device__ __forceinline__ bool edge_tile_rows(float2 a, float2 b, const CvGeom &g, int &r0, int &r1)
{
    if (a.y == b.y) return false;
    float lo = fminf(a.y, b.y), hi = fmaxf(a.y, b.y);
    float jlo = fmaxf(floorf(lo * g.inv - 0.5f) - 1.0f, 0.0f);
    float jhi = fminf(ceilf(hi * g.inv - 0.5f) + 1.0f, (float)(g.vy - 1));
    if (!(jlo <= jhi)) return false;
    r0 = (int)jlo >> 3;
    r1 = (int)jhi >> 3;
    return true;
}

// Edge buckets per tile row: count, then (after a scan) fill. An edge is
// (s, s - 1), the reference's pairing (canvas.cpp:121).
// Edges within one tile row (most of them) are grouped per warp: one atomic
// per row and warp; edges spanning several rows count row by row.
__device__ __forceinline__ int edge_key(const float2 *__restrict__ poly, int n, const CvGeom &g, int s, int &r0,
                                        int &r1)
{
    const int lane = threadIdx.x & 31;
    if (s >= n || !edge_tile_rows(poly[s], poly[s == 0 ? n - 1 : s - 1], g, r0, r1)) {
        r0 = 0;
        r1 = -1;
        return -1 - lane;
    }
    return r0 == r1 ? r0 : -1 - lane;
}

__global__ void k_cv_edge_count(const float2 *__restrict__ poly, int n, CvGeom g, int *__restrict__ rowCount)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int r0, r1;
    const int key = edge_key(poly, n, g, s, r0, r1);
    const unsigned grp = __match_any_sync(0xffffffffu, key);
    if (key >= 0) {
        if (lane == __ffs(grp) - 1) atomicAdd(&rowCount[key], __popc(grp));
    } else {
        for (int r = r0; r <= r1; ++r) atomicAdd(&rowCount[r], 1);
    }
}

__global__ void k_cv_edge_fill(const float2 *__restrict__ poly, int n, CvGeom g, const int *__restrict__ rowStart,
                               int *__restrict__ rowFill, int *__restrict__ bucket)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int r0, r1;
    const int key = edge_key(poly, n, g, s, r0, r1);
    const unsigned grp = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(grp) - 1;
    int base = 0;
    if (key >= 0 && lane == leader) base = atomicAdd(&rowFill[key], __popc(grp));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (key >= 0) {
        bucket[rowStart[key] + base + __popc(grp & ((1u << lane) - 1u))] = s;
    } else {
        for (int r = r0; r <= r1; ++r) bucket[rowStart[r] + atomicAdd(&rowFill[r], 1)] = s;
    }
}

// The edges of tile row ty staged in shared memory as (a.x, a.y, b.x, b.y):
// the row's bucket, or every edge when there are no buckets.
__device__ __forceinline__ void stage_edges(const float2 *__restrict__ poly, int n, const int *__restrict__ bucket,
                                            int c0, int m, float4 *ch)
{
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        int e = bucket ? bucket[c0 + k] : c0 + k;
        float2 a = poly[e], b = poly[e == 0 ? n - 1 : e - 1];
        ch[k] = make_float4(a.x, a.y, b.x, b.y);
    }
}

// One block per tile row, one warp per scanline. Crossings are gathered in
// shared memory, sorted (bitonic) and turned into spans of a row bitmap; the
// block then writes whole tile words. Rows with more than kRowCap crossings
// are left for k_cv_scanline_big. With buckets (rowStart/bucket non-null) a
// block tests only the edges that can reach its rows; otherwise all of them.
__global__ void __launch_bounds__(256) k_cv_scanline(const float2 *__restrict__ poly, int n,
                                                      const int *__restrict__ rowStart, const int *__restrict__ bucket,
                                                      CvGeom g, unsigned long long *__restrict__ inside, int *ovRows,
                                                      CvState *st)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    const int W32 = (g.vx + 31) >> 5;
    float4 *ch = reinterpret_cast<float4 *>(smraw);
    float *buf = reinterpret_cast<float *>(ch + kChunk);
    int *cnt = reinterpret_cast<int *>(buf + 8 * kRowCap);
    unsigned *bits = reinterpret_cast<unsigned *>(cnt + 8);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int ty = blockIdx.x;
    const int j = ty * 8 + w;
    const bool live = j < g.vy;
    const float y = ((float)j + 0.5f) * g.vs;
    for (int k = threadIdx.x; k < 8 * W32; k += 256) bits[k] = 0u;
    if (lane == 0) cnt[w] = 0;
    const int e0 = bucket ? rowStart[ty] : 0, e1 = bucket ? rowStart[ty + 1] : n;
    for (int c0 = e0; c0 < e1; c0 += kChunk) {
        int m = min(kChunk, e1 - c0);
        __syncthreads();
        stage_edges(poly, n, bucket, c0, m, ch);
        __syncthreads();
        if (live) {
            for (int k = lane; k < m; k += 32) {
                float4 q = ch[k];
                float2 a = make_float2(q.x, q.y), b = make_float2(q.z, q.w); // edge (s, s - 1)
                if ((a.y > y) != (b.y > y)) {
                    float x = crossing(a, b, y);
                    int p = atomicAdd(&cnt[w], 1);
                    if (p < kRowCap) buf[w * kRowCap + p] = x;
                }
            }
        }
    }
    __syncwarp();
    const int c = live ? cnt[w] : 0;
    if (c > kRowCap) {
        if (lane == 0) ovRows[atomicAdd(&st->overflowRows, 1)] = j;
    } else if (c >= 2) {
        float *v = buf + w * kRowCap;
        int P2 = 1;
        while (P2 < c) P2 <<= 1;
        for (int k = c + lane; k < P2; k += 32) v[k] = INFINITY;
        __syncwarp();
        for (int kk = 2; kk <= P2; kk <<= 1) {
            for (int jj = kk >> 1; jj > 0; jj >>= 1) {
                for (int i = lane; i < P2; i += 32) {
                    int ixj = i ^ jj;
                    if (ixj > i) {
                        float a = v[i], b = v[ixj];
                        bool up = (i & kk) == 0;
                        if ((a > b) == up) {
                            v[i] = b;
                            v[ixj] = a;
                        }
                    }
                }
                __syncwarp();
            }
        }
        for (int p = lane; 2 * p + 1 < c; p += 32) fill_pair(bits + w * W32, v[2 * p], v[2 * p + 1], g);
    }
    __syncthreads();
    for (int tx = threadIdx.x; tx < g.tilesX; tx += 256) {
        unsigned long long word = 0ull;
        for (int r = 0; r < 8; ++r) {
            unsigned wb = bits[r * W32 + (tx >> 2)];
            word |= (unsigned long long)((wb >> ((tx & 3) * 8)) & 0xffu) << (8 * r);
        }
        inside[(size_t)ty * g.tilesX + tx] = word;
    }
}

// Rows with more than kRowCap crossings: one block per row, up to kBigCap
// crossings sorted in shared memory; the row's byte of each tile word is
// written directly (the rows of one tile row own distinct bytes).
__global__ void __launch_bounds__(1024) k_cv_scanline_big(const float2 *__restrict__ poly, int n,
                                                           const int *__restrict__ rowStart,
                                                           const int *__restrict__ bucket, CvGeom g,
                                                           unsigned long long *__restrict__ inside,
                                                           const int *__restrict__ ovRows, CvState *st)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    float *v = reinterpret_cast<float *>(smraw);
    unsigned *row = reinterpret_cast<unsigned *>(v + kBigCap);
    __shared__ int cnt;
    const int W32 = (g.vx + 31) >> 5;
    const int nrows = st->overflowRows;
    for (int r = blockIdx.x; r < nrows; r += gridDim.x) {
        const int j = ovRows[r];
        const float y = ((float)j + 0.5f) * g.vs;
        if (threadIdx.x == 0) cnt = 0;
        for (int k = threadIdx.x; k < W32; k += blockDim.x) row[k] = 0u;
        __syncthreads();
        const int e0 = bucket ? rowStart[j >> 3] : 0, e1 = bucket ? rowStart[(j >> 3) + 1] : n;
        for (int k = e0 + threadIdx.x; k < e1; k += blockDim.x) {
            int s = bucket ? bucket[k] : k;
            float2 a = poly[s], b = poly[s == 0 ? n - 1 : s - 1];
            if ((a.y > y) != (b.y > y)) {
                float x = crossing(a, b, y);
                int p = atomicAdd(&cnt, 1);
                if (p < kBigCap) v[p] = x;
            }
        }
        __syncthreads();
        const int c = cnt;
        if (c > kBigCap) {
            if (threadIdx.x == 0) atomicOr(&st->err, kErrCrossings);
            __syncthreads();
            continue;
        }
        int P2 = 1;
        while (P2 < c) P2 <<= 1;
        for (int k = c + threadIdx.x; k < P2; k += blockDim.x) v[k] = INFINITY;
        __syncthreads();
        for (int kk = 2; kk <= P2; kk <<= 1) {
            for (int jj = kk >> 1; jj > 0; jj >>= 1) {
                for (int i = threadIdx.x; i < P2; i += blockDim.x) {
                    int ixj = i ^ jj;
                    if (ixj > i) {
                        float a = v[i], b = v[ixj];
                        bool up = (i & kk) == 0;
                        if ((a > b) == up) {
                            v[i] = b;
                            v[ixj] = a;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (int p = threadIdx.x; 2 * p + 1 < c; p += blockDim.x) fill_pair(row, v[2 * p], v[2 * p + 1], g);
        __syncthreads();
        unsigned char *bytes = reinterpret_cast<unsigned char *>(inside);
        for (int tx = threadIdx.x; tx < g.tilesX; tx += blockDim.x)
            bytes[((size_t)(j >> 3) * g.tilesX + tx) * 8 + (j & 7)] =
                (unsigned char)((row[tx >> 2] >> ((tx & 3) * 8)) & 0xffu);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// StampDisc (canvas.cpp:136-221)
// ---------------------------------------------------------------------------
// 1. rim samples on the other side of the current occupancy, binned by tile
//    of the stamp's tile box (canvas.cpp:148-158)
__global__ void k_cv_rim_bin(const float2 *__restrict__ rimXY, CvStamp p, CvGeom g,
                             const unsigned long long *__restrict__ inside, int *__restrict__ boxCount,
                             int *__restrict__ recTile, int *__restrict__ recRank, int *__restrict__ list,
                             CvState *st)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= p.nRim) return;
    float2 q = rimXY[k];
    int i, j;
    recTile[k] = -1;
    if (!voxel_of(q.x, q.y, g, i, j)) return;
    int in = (int)((inside[(size_t)(j >> 3) * g.tilesX + (i >> 3)] >> bit_of(i, j)) & 1ull);
    if (in == p.inside) return;
    int tx = (i >> 3) - p.bx0, ty = (j >> 3) - p.by0;
    if (tx < 0 || ty < 0 || tx >= p.bw || ty >= p.bh) {
        atomicOr(&st->err, kErrRimBox);
        return;
    }
    int lt = ty * p.bw + tx;
    recTile[k] = lt;
    int rank = atomicAdd(&boxCount[lt], 1);
    recRank[k] = rank;
    if (rank == 0) list[atomicAdd(&st->listCount, 1)] = lt;
}

// 2-3. per box tile: surface samples strictly inside the disc (removed),
// occupancy flips of voxel centres inside the disc, and the rim voxels that
// keep their slot or need a new one (canvas.cpp:160-197, 204-211). One warp a
// tile; each tile word is owned by one warp.
__global__ void __launch_bounds__(256) k_cv_stamp_tiles(CvStamp p, CvGeom g, int nBox,
                                                         unsigned long long *__restrict__ inside,
                                                         const unsigned long long *__restrict__ smask,
                                                         const float2 *__restrict__ spt,
                                                         const unsigned long long *__restrict__ rimMask,
                                                         unsigned long long *__restrict__ remMask,
                                                         unsigned long long *__restrict__ origMask,
                                                         int *__restrict__ nRem, int *__restrict__ nRim,
                                                         int *__restrict__ nNew, CvState *st)
{
    const int lane = threadIdx.x & 31;
    const int lt = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (lt >= nBox) return;
    const int tx = p.bx0 + lt % p.bw, ty = p.by0 + lt / p.bw;
    const size_t t = (size_t)ty * g.tilesX + tx;
    const unsigned long long before = smask[t];
    const unsigned long long word = inside[t];
    unsigned long long rem = 0ull, flip = 0ull;
    for (int half = 0; half < 2; ++half) {
        int b = lane + 32 * half;
        bool r = false, f = false;
        if ((before >> b) & 1ull) {
            float2 q = spt[t * 64 + b];
            float d = (q.x - p.cx) * (q.x - p.cx) + (q.y - p.cy) * (q.y - p.cy);
            r = !(d >= p.r2);
        }
        int i = tx * 8 + (b & 7), j = ty * 8 + (b >> 3);
        if (i >= p.i0 && i <= p.i1 && j >= p.j0 && j <= p.j1) {
            float dy = ((float)j + 0.5f) * g.vs - p.cy;
            float dx = ((float)i + 0.5f) * g.vs - p.cx;
            if (!(dx * dx + dy * dy >= p.r2)) f = (int)((word >> b) & 1ull) != p.inside;
        }
        rem |= (unsigned long long)__ballot_sync(0xffffffffu, r) << (32 * half);
        flip |= (unsigned long long)__ballot_sync(0xffffffffu, f) << (32 * half);
    }
    if (lane == 0) {
        if (flip) {
            inside[t] = word ^ flip;
            atomicAdd(&st->flipped, __popcll(flip));
        }
        unsigned long long rm = rimMask[lt];
        unsigned long long after = before & ~rem;
        remMask[lt] = rem;
        origMask[lt] = before;
        nRem[lt] = __popcll(rem);
        nRim[lt] = __popcll(rm);
        nNew[lt] = __popcll(rm & ~after);
    }
}

// 4a. removed samples: their slots are freed (pushed in tile-major voxel
// order, the reference's loop order) and reported dirty (canvas.cpp:172-176)
__global__ void __launch_bounds__(256) k_cv_stamp_remove(CvStamp p, CvGeom g, int nBox,
                                                          const unsigned long long *__restrict__ remMask,
                                                          const int *__restrict__ remStart,
                                                          const int *__restrict__ sslot, float2 *__restrict__ slots,
                                                          int *__restrict__ freel, int *__restrict__ dirty,
                                                          const CvState *st)
{
    const int lane = threadIdx.x & 31;
    const int lt = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (lt >= nBox) return;
    const unsigned long long rem = remMask[lt];
    if (!rem) return;
    const int tx = p.bx0 + lt % p.bw, ty = p.by0 + lt / p.bw;
    const size_t t = (size_t)ty * g.tilesX + tx;
    const int nfree0 = st->nfree0;
    for (int b = lane; b < 64; b += 32) {
        if (!((rem >> b) & 1ull)) continue;
        int q = remStart[lt] + __popcll(rem & lower_bits(b));
        int s = sslot[t * 64 + b];
        dirty[q] = s;
        freel[nfree0 + q] = s;
        slots[s] = make_float2(-1.0f, -1.0f);
    }
}

// 4b. the kept rim becomes surface (canvas.cpp:199-214): rim voxels in
// tile-major order take slots from the top of the free list, then new ones.
__global__ void __launch_bounds__(256) k_cv_stamp_rim(CvStamp p, CvGeom g, int nBox,
                                                       const unsigned long long *__restrict__ rimMask,
                                                       const float2 *__restrict__ rimPt,
                                                       const unsigned long long *__restrict__ remMask,
                                                       const unsigned long long *__restrict__ origMask,
                                                       const int *__restrict__ rimStart,
                                                       const int *__restrict__ newStart,
                                                       unsigned long long *__restrict__ smask,
                                                       float2 *__restrict__ spt, int *__restrict__ sslot,
                                                       float2 *__restrict__ slots, const int *__restrict__ freel,
                                                       int *__restrict__ dirty, CvState *st)
{
    const int lane = threadIdx.x & 31;
    const int lt = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (lt >= nBox) return;
    const unsigned long long rm = rimMask[lt], rem = remMask[lt], orig = origMask[lt];
    if (!rm && !rem) return;
    const int tx = p.bx0 + lt % p.bw, ty = p.by0 + lt / p.bw;
    const size_t t = (size_t)ty * g.tilesX + tx;
    const unsigned long long after = orig & ~rem;
    const unsigned long long fresh = rm & ~after;
    const int R = st->removed, F = st->freeAfterPush, nslots0 = st->nslots0;
    for (int b = lane; b < 64; b += 32) {
        if (!((rm >> b) & 1ull)) continue;
        size_t v = t * 64 + b;
        float2 q = rimPt[(size_t)lt * 64 + b];
        int s;
        if ((after >> b) & 1ull) {
            s = sslot[v];
        } else {
            int k = newStart[lt] + __popcll(fresh & lower_bits(b));
            s = k < F ? freel[F - 1 - k] : nslots0 + (k - F);
            sslot[v] = s;
        }
        slots[s] = q;
        spt[v] = q;
        dirty[R + rimStart[lt] + __popcll(rm & lower_bits(b))] = s;
    }
    if (lane == 0) {
        unsigned long long fin = after | rm;
        smask[t] = fin;
        int d = (fin != 0ull) - (orig != 0ull);
        if (d) atomicAdd(&st->surfaceTiles, d);
    }
}

__global__ void k_cv_gather_dirty(const int *__restrict__ dirty, const float2 *__restrict__ slots,
                                  float2 *__restrict__ values, const CvState *st)
{
    const int n = st->ndirty;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) values[k] = slots[dirty[k]];
}

__global__ void k_cv_fill(float2 *__restrict__ p, size_t n, float2 v)
{
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) p[k] = v;
}

__global__ void k_cv_copy_rect(const unsigned long long *__restrict__ src, unsigned long long *__restrict__ dst,
                               int pitch, int tx0, int ty0, int w, int h)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= w * h) return;
    size_t o = (size_t)(ty0 + k / w) * pitch + tx0 + k % w;
    dst[o] = src[o];
}

cudaError_t scan_ex(const int *in, int *out, int n, int *partial, cudaStream_t s)
{
    if (n <= 8192) {
        k_scan_single<<<1, 1024, 0, s>>>(in, out, n);
    } else {
        int nb = (n + kScanChunk - 1) / kScanChunk;
        k_scan_reduce<<<nb, 1024, 0, s>>>(in, n, partial);
        k_scan_single<<<1, 1024, 0, s>>>(partial, partial, nb);
        k_scan_apply<<<nb, 1024, 0, s>>>(in, out, n, partial);
    }
    return cudaGetLastError();
}

int scan_partials(int n) { return n <= 8192 ? 1 : (n + kScanChunk - 1) / kScanChunk + 1; }

} // namespace

// ===========================================================================
// canvas handle
// ===========================================================================
struct cv_canvas {
    float width = 0, height = 0;
    CvGeom g{};
    size_t tiles = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    CvState *hostState = nullptr; // pinned
    CvState st{};                 // the last state read
    cv_edit lastEdit{};
    int smemScan = 0, smemBig = 0;

    DevBuf<unsigned long long> inside, smask;
    DevBuf<float2> spt, slots, recXY, poly, rimPt, dirtyVal;
    DevBuf<int> sslot, freel, dirty, segCnt, tileCount, surfCount, partial, recTile, recRank, ovRows;
    DevBuf<int> rowStart, rowFill, bucket; // edge buckets per tile row
    DevBuf<int> tileList;                  // tiles with samples
    DevBuf<float4> rec;
    DevBuf<CvState> dState;
    // stamp scratch
    DevBuf<unsigned long long> rimMask, remMask, origMask;
    DevBuf<int> boxCount, nRem, nRim, nNew;
    DevBuf<float2> rimXY;
    std::vector<float2> rimHost;
};

namespace {

int read_state(cv_canvas *c)
{
    cudaError_t e;
    if ((e = cudaMemcpyAsync(c->hostState, c->dState.p, sizeof(CvState), cudaMemcpyDeviceToHost, c->stream)) ||
        (e = cudaStreamSynchronize(c->stream)))
        return cuda_fail(e, "canvas state");
    c->st = *c->hostState;
    return VM_OK;
}

// grows a buffer, keeping its first `keep` elements
template <class T> int grow_keep(DevBuf<T> &b, size_t need, size_t keep, cudaStream_t s)
{
    if (need <= b.n && b.p) return VM_OK;
    size_t cap = std::max(need, b.n + b.n / 2 + 64);
    T *p = nullptr;
    cudaError_t e = cudaMalloc(&p, cap * sizeof(T));
    if (e) return cuda_fail(e, "cudaMalloc");
    if (keep && b.p && (e = cudaMemcpyAsync(p, b.p, keep * sizeof(T), cudaMemcpyDeviceToDevice, s))) {
        cudaFree(p);
        return cuda_fail(e, "grow copy");
    }
    if (b.p) {
        cudaStreamSynchronize(s);
        cudaFree(b.p);
    }
    b.p = p;
    b.n = cap;
    return VM_OK;
}

int blocks_for(long long n, int per) { return (int)std::max(1LL, (n + per - 1) / per); }

} // namespace

extern "C" {

int cv_create(float width, float height, float voxelSize, cv_canvas **out)
{
    if (!out) return fail(VM_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (!(width > 0.0f) || !(height > 0.0f) || !(voxelSize > 0.0f)) return fail(VM_ERR_ARG, "cv_create: sizes must be > 0");
    // canvas.cpp:33-38
    float fx = std::ceil(width / voxelSize), fy = std::ceil(height / voxelSize);
    if (!(fx <= (float)kMaxVoxelsX) || !(fy <= 1.0e8f)) return fail(VM_ERR_UNSUPPORTED, "cv_create: too many voxels per row");
    cv_canvas *c = new cv_canvas();
    c->width = width;
    c->height = height;
    c->g.vx = (int)fx;
    c->g.vy = (int)fy;
    c->g.tilesX = (c->g.vx + 7) / 8;
    c->g.tilesY = (c->g.vy + 7) / 8;
    c->g.vs = voxelSize;
    c->g.inv = 1.0f / voxelSize;
    c->tiles = (size_t)c->g.tilesX * c->g.tilesY;
    int rc;
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) || (e = cudaEventCreate(&c->ev0)) ||
        (e = cudaEventCreate(&c->ev1)) || (e = cudaMallocHost((void **)&c->hostState, sizeof(CvState)))) {
        rc = cuda_fail(e, "cv_create");
        cv_destroy(c);
        return rc;
    }
    if ((rc = c->inside.alloc(c->tiles)) || (rc = c->smask.alloc(c->tiles)) || (rc = c->spt.alloc(c->tiles * 64)) ||
        (rc = c->sslot.alloc(c->tiles * 64)) || (rc = c->dState.alloc(1)) || (rc = c->ovRows.alloc(c->g.vy + 1))) {
        cv_destroy(c);
        return rc;
    }
    int W32 = (c->g.vx + 31) / 32;
    c->smemScan = (int)(kChunk * sizeof(float4) + 8 * kRowCap * sizeof(float) + 8 * sizeof(int) +
                        8 * (size_t)W32 * sizeof(unsigned));
    c->smemBig = (int)(kBigCap * sizeof(float) + (size_t)W32 * sizeof(unsigned));
    if ((e = cudaFuncSetAttribute(k_cv_scanline, cudaFuncAttributeMaxDynamicSharedMemorySize, c->smemScan)) ||
        (e = cudaFuncSetAttribute(k_cv_scanline_big, cudaFuncAttributeMaxDynamicSharedMemorySize, c->smemBig)) ||
        (e = cudaMemsetAsync(c->inside.p, 0, c->tiles * 8, c->stream)) ||
        (e = cudaMemsetAsync(c->smask.p, 0, c->tiles * 8, c->stream)) ||
        (e = cudaMemsetAsync(c->dState.p, 0, sizeof(CvState), c->stream)) || (e = cudaStreamSynchronize(c->stream))) {
        rc = cuda_fail(e, "cv_create");
        cv_destroy(c);
        return rc;
    }
    *out = c;
    return VM_OK;
}

int cv_destroy(cv_canvas *c)
{
    if (!c) return VM_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->hostState) cudaFreeHost(c->hostState);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return VM_OK;
}

int cv_rasterize(cv_canvas *c, const float *xy, int n, float *gpuMs)
{
    vmh::NvtxRange range("cv_rasterize");
    if (!c || n < 0 || (n > 0 && !xy)) return fail(VM_ERR_ARG, "cv_rasterize: bad arguments");
    for (long long k = 0; k < 2LL * n; ++k)
        if (!std::isfinite(xy[k])) return fail(VM_ERR_ARG, "cv_rasterize: polygon coordinates must be finite");
    cudaStream_t s = c->stream;
    const CvGeom g = c->g;
    const int T = (int)c->tiles;
    cudaError_t e;
    int rc;
    c->lastEdit = cv_edit{};
    if ((e = cudaEventRecord(c->ev0, s)) || (e = cudaMemsetAsync(c->dState.p, 0, sizeof(CvState), s)) ||
        (e = cudaMemsetAsync(c->inside.p, 0, c->tiles * 8, s)) || (e = cudaMemsetAsync(c->smask.p, 0, c->tiles * 8, s)))
        return cuda_fail(e, "cv_rasterize");
    if (n > 0) {
        if ((rc = c->poly.reserve(n)) || (rc = c->segCnt.reserve((size_t)n + 1)) ||
            (rc = c->partial.reserve((size_t)std::max(scan_partials(n + 1), scan_partials(T + 1)))) ||
            (rc = c->rowStart.reserve((size_t)g.tilesY + 1)) || (rc = c->rowFill.reserve((size_t)g.tilesY + 1)))
            return rc;
        if ((e = cudaMemcpyAsync(c->poly.p, xy, sizeof(float2) * (size_t)n, cudaMemcpyHostToDevice, s)) ||
            (e = cudaMemsetAsync(c->rowStart.p, 0, sizeof(int) * ((size_t)g.tilesY + 1), s)))
            return cuda_fail(e, "upload polygon");
        k_cv_seg_counts<<<blocks_for(n, 256), 256, 0, s>>>(c->poly.p, n, 0.25f * g.vs, c->segCnt.p, c->dState.p);
        if ((e = scan_ex(c->segCnt.p, c->segCnt.p, n, c->partial.p, s))) return cuda_fail(e, "segment scan");
        // edge buckets per tile row (sized by the same read-back as the samples)
        k_cv_edge_count<<<blocks_for(n, 256), 256, 0, s>>>(c->poly.p, n, g, c->rowStart.p);
        if ((e = scan_ex(c->rowStart.p, c->rowStart.p, g.tilesY, c->partial.p, s)) ||
            (e = cudaMemcpyAsync(&c->dState.p->edgeEntries, c->rowStart.p + g.tilesY, sizeof(int),
                                 cudaMemcpyDeviceToDevice, s)))
            return cuda_fail(e, "edge buckets");
        if ((rc = read_state(c))) return rc;
        if (c->st.err & kErrSamples) return fail(VM_ERR_UNSUPPORTED, "cv_rasterize: a polygon edge spans too many voxels");
        if (c->st.totalSamples > (unsigned long long)INT_MAX) return fail(VM_ERR_UNSUPPORTED, "cv_rasterize: too many surface samples");
        const int total = (int)c->st.totalSamples;
        if ((rc = c->recTile.reserve(total)) || (rc = c->recRank.reserve(total)) || (rc = c->recXY.reserve(total)) ||
            (rc = c->rec.reserve(total)) || (rc = c->tileCount.reserve((size_t)T + 1)) ||
            (rc = c->surfCount.reserve((size_t)T + 1)) || (rc = c->tileList.reserve((size_t)std::min(T, total))))
            return rc;
        // a surface voxel holds at least one sample: `total` bounds the slots
        size_t cap = (size_t)std::min<long long>(total, (long long)T * 64);
        if ((rc = c->slots.reserve(std::max<size_t>(cap, 1))) || (rc = c->freel.reserve(std::max<size_t>(cap, 1))))
            return rc;
        if ((e = cudaMemsetAsync(c->tileCount.p, 0, sizeof(int) * ((size_t)T + 1), s)) ||
            (e = cudaMemsetAsync(c->surfCount.p, 0, sizeof(int) * ((size_t)T + 1), s)))
            return cuda_fail(e, "memset");
        // VM_CANVAS_BUCKET_CAP lowers the bucket limit (0 = always test every edge)
        long long bucketCap = kMaxBucketEntries;
        if (const char *env = std::getenv("VM_CANVAS_BUCKET_CAP")) bucketCap = std::min(bucketCap, std::atoll(env));
        const int entries = c->st.edgeEntries;
        const bool buckets = entries >= 0 && entries <= bucketCap && bucketCap > 0;
        if (buckets) {
            if ((rc = c->bucket.reserve((size_t)std::max(entries, 1)))) return rc;
            if ((e = cudaMemsetAsync(c->rowFill.p, 0, sizeof(int) * ((size_t)g.tilesY + 1), s)))
                return cuda_fail(e, "memset");
            k_cv_edge_fill<<<blocks_for(n, 256), 256, 0, s>>>(c->poly.p, n, g, c->rowStart.p, c->rowFill.p,
                                                              c->bucket.p);
        }
        const int *rs = buckets ? c->rowStart.p : nullptr;
        const int *bk = buckets ? c->bucket.p : nullptr;
        k_cv_samples<<<blocks_for(total, 256), 256, 0, s>>>(c->poly.p, n, c->segCnt.p, total, g, c->tileCount.p,
                                                            c->recTile.p, c->recRank.p, c->recXY.p, c->tileList.p,
                                                            c->dState.p);
        if ((e = scan_ex(c->tileCount.p, c->tileCount.p, T, c->partial.p, s))) return cuda_fail(e, "tile scan");
        k_cv_scatter<<<blocks_for(total, 256), 256, 0, s>>>(total, c->recTile.p, c->recRank.p, c->recXY.p,
                                                            c->tileCount.p, g, c->rec.p);
        const int listGrid = std::min(blocks_for(std::min(T, total), 8), kListBlocks);
        // recTile is free once the records are scattered: it holds the per-tile voxel sort
        k_cv_tile_means<<<listGrid, 256, 0, s>>>(c->tileList.p, &c->dState.p->listCount, c->tileCount.p, c->rec.p,
                                                 c->recTile.p, c->smask.p, c->spt.p, c->surfCount.p,
                                                 &c->dState.p->surfaceTiles);
        if ((e = scan_ex(c->surfCount.p, c->surfCount.p, T, c->partial.p, s))) return cuda_fail(e, "surface scan");
        k_cv_assign<<<listGrid, 256, 0, s>>>(c->tileList.p, &c->dState.p->listCount, c->smask.p, c->surfCount.p, T,
                                             c->spt.p, c->sslot.p, c->slots.p,
                                               c->dState.p);
        k_cv_scanline<<<g.tilesY, 256, c->smemScan, s>>>(c->poly.p, n, rs, bk, g, c->inside.p, c->ovRows.p,
                                                         c->dState.p);
        k_cv_scanline_big<<<kBigBlocks, 1024, c->smemBig, s>>>(c->poly.p, n, rs, bk, g, c->inside.p, c->ovRows.p,
                                                               c->dState.p);
        if ((e = cudaGetLastError())) return cuda_fail(e, "cv_rasterize launch");
    }
    if ((e = cudaEventRecord(c->ev1, s))) return cuda_fail(e, "event");
    if ((rc = read_state(c))) return rc;
    if (c->st.err & kErrCrossings) {
        // leave the canvas empty, as a rasterisation of no polygon does
        if ((e = cudaMemsetAsync(c->dState.p, 0, sizeof(CvState), s)) ||
            (e = cudaMemsetAsync(c->inside.p, 0, c->tiles * 8, s)) ||
            (e = cudaMemsetAsync(c->smask.p, 0, c->tiles * 8, s)))
            return cuda_fail(e, "cv_rasterize reset");
        if ((rc = read_state(c))) return rc;
        return fail(VM_ERR_UNSUPPORTED, "cv_rasterize: more than 32768 polygon edges cross one scanline");
    }
    if (gpuMs && (e = cudaEventElapsedTime(gpuMs, c->ev0, c->ev1))) return cuda_fail(e, "event time");
    return VM_OK;
}

int cv_stamp_disc(cv_canvas *c, float cx, float cy, float radius, int inside, cv_edit *out)
{
    vmh::NvtxRange range("cv_stamp_disc");
    if (!c || !out) return fail(VM_ERR_ARG, "cv_stamp_disc: bad arguments");
    *out = cv_edit{};
    c->lastEdit = cv_edit{};
    if (!std::isfinite(cx) || !std::isfinite(cy) || !std::isfinite(radius))
        return fail(VM_ERR_ARG, "cv_stamp_disc: centre and radius must be finite");
    const CvGeom g = c->g;
    cudaStream_t s = c->stream;
    // canvas.cpp:138-146, the same float operations as the reference; the
    // voxel indices are clamped before the conversion to int (lower bounds to
    // [0, size], upper to [-1, size - 1]), which keeps i0 > i1 exactly when
    // the reference's box is empty
    const float inv = 1.0f / g.vs;
    const float r2 = radius * radius;
    auto index = [](float v, int lo, int hi) {
        float f = std::floor(v);
        return f < (float)lo ? lo : f > (float)hi ? hi : (int)f;
    };
    int i0 = index((cx - radius) * inv, 0, g.vx);
    int j0 = index((cy - radius) * inv, 0, g.vy);
    int i1 = index((cx + radius) * inv, -1, g.vx - 1);
    int j1 = index((cy + radius) * inv, -1, g.vy - 1);
    if (i0 > i1 || j0 > j1) return VM_OK;
    // rim sample positions: the reference's host trigonometry (canvas.cpp:151-154)
    const float rimF = std::ceil(2.0f * 3.14159265f * radius / (0.25f * g.vs));
    if (!(rimF <= (float)kMaxRimSamples)) return fail(VM_ERR_UNSUPPORTED, "cv_stamp_disc: radius too large");
    int n = std::max(16, (int)rimF);
    c->rimHost.resize((size_t)n);
    for (int k = 0; k < n; ++k) {
        float a = 2.0f * 3.14159265f * (float)k / (float)n;
        c->rimHost[k] = make_float2(cx + radius * ::cosf(a), cy + radius * ::sinf(a));
    }
    CvStamp p{};
    p.cx = cx;
    p.cy = cy;
    p.r2 = r2;
    p.inside = inside ? 1 : 0;
    p.i0 = i0; p.j0 = j0; p.i1 = i1; p.j1 = j1;
    p.bx0 = i0 >> 3; p.by0 = j0 >> 3;
    p.bw = (i1 >> 3) - p.bx0 + 1;
    p.bh = (j1 >> 3) - p.by0 + 1;
    p.nRim = n;
    const int nBox = p.bw * p.bh;
    int rc;
    cudaError_t e;
    const int nslots = c->st.nslots;
    if ((rc = c->rimXY.reserve(n)) || (rc = c->recTile.reserve(n)) || (rc = c->recRank.reserve(n)) ||
        (rc = c->rec.reserve(n)) || (rc = c->boxCount.reserve((size_t)nBox + 1)) ||
        (rc = c->nRem.reserve((size_t)nBox + 1)) || (rc = c->nRim.reserve((size_t)nBox + 1)) ||
        (rc = c->nNew.reserve((size_t)nBox + 1)) || (rc = c->rimMask.reserve(nBox)) ||
        (rc = c->remMask.reserve(nBox)) || (rc = c->origMask.reserve(nBox)) ||
        (rc = c->rimPt.reserve((size_t)nBox * 64)) || (rc = c->partial.reserve((size_t)scan_partials(nBox + 1))) ||
        (rc = c->tileList.reserve((size_t)std::min(nBox, n))) ||
        (rc = c->dirty.reserve((size_t)nBox * 64 + n)) || (rc = c->dirtyVal.reserve((size_t)nBox * 64 + n)) ||
        (rc = grow_keep(c->slots, (size_t)nslots + n, (size_t)nslots, s)) ||
        (rc = grow_keep(c->freel, (size_t)nslots + n, (size_t)c->st.nfree, s)))
        return rc;
    // the edit's counters: removed, added, flipped, ndirty, overflowRows; and the error flags
    if ((e = cudaMemcpyAsync(c->rimXY.p, c->rimHost.data(), sizeof(float2) * (size_t)n, cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemsetAsync(&c->dState.p->removed, 0, 5 * sizeof(int), s)) ||
        (e = cudaMemsetAsync(&c->dState.p->err, 0, sizeof(int), s)) ||
        (e = cudaMemsetAsync(&c->dState.p->listCount, 0, sizeof(int), s)) ||
        (e = cudaMemsetAsync(c->rimMask.p, 0, sizeof(unsigned long long) * (size_t)nBox, s)) ||
        (e = cudaMemsetAsync(c->boxCount.p, 0, sizeof(int) * ((size_t)nBox + 1), s)))
        return cuda_fail(e, "cv_stamp_disc");
    k_cv_rim_bin<<<blocks_for(n, 256), 256, 0, s>>>(c->rimXY.p, p, g, c->inside.p, c->boxCount.p, c->recTile.p,
                                                    c->recRank.p, c->tileList.p, c->dState.p);
    if ((e = scan_ex(c->boxCount.p, c->boxCount.p, nBox, c->partial.p, s))) return cuda_fail(e, "rim scan");
    k_cv_scatter<<<blocks_for(n, 256), 256, 0, s>>>(n, c->recTile.p, c->recRank.p, c->rimXY.p, c->boxCount.p, g,
                                                    c->rec.p);
    k_cv_tile_means<<<std::min(blocks_for(std::min(nBox, n), 8), kListBlocks), 256, 0, s>>>(
        c->tileList.p, &c->dState.p->listCount, c->boxCount.p, c->rec.p, c->recTile.p, c->rimMask.p, c->rimPt.p,
        nullptr, nullptr);
    k_cv_stamp_tiles<<<blocks_for(nBox, 8), 256, 0, s>>>(p, g, nBox, c->inside.p, c->smask.p, c->spt.p, c->rimMask.p,
                                                         c->remMask.p, c->origMask.p, c->nRem.p, c->nRim.p,
                                                         c->nNew.p, c->dState.p);
    k_scan3_single<<<1, 1024, 0, s>>>(c->nRem.p, c->nRim.p, c->nNew.p, nBox, c->dState.p);
    k_cv_stamp_remove<<<blocks_for(nBox, 8), 256, 0, s>>>(p, g, nBox, c->remMask.p, c->nRem.p, c->sslot.p,
                                                          c->slots.p, c->freel.p, c->dirty.p, c->dState.p);
    k_cv_stamp_rim<<<blocks_for(nBox, 8), 256, 0, s>>>(p, g, nBox, c->rimMask.p, c->rimPt.p, c->remMask.p,
                                                       c->origMask.p, c->nRim.p, c->nNew.p, c->smask.p, c->spt.p,
                                                       c->sslot.p, c->slots.p, c->freel.p, c->dirty.p, c->dState.p);
    k_cv_gather_dirty<<<32, 256, 0, s>>>(c->dirty.p, c->slots.p, c->dirtyVal.p, c->dState.p);
    if ((e = cudaGetLastError())) return cuda_fail(e, "cv_stamp_disc launch");
    if ((rc = read_state(c))) return rc;
    if (c->st.err & kErrRimBox) return fail(VM_ERR_CUDA, "cv_stamp_disc: rim sample outside the stamp box");
    cv_edit &E = c->lastEdit;
    E.tx0 = p.bx0;
    E.ty0 = p.by0;
    E.tx1 = (i1 >> 3) + 1;
    E.ty1 = (j1 >> 3) + 1;
    E.removed = c->st.removed;
    E.added = c->st.added;
    E.flipped = c->st.flipped;
    E.ndirty = c->st.ndirty;
    *out = E;
    return VM_OK;
}

int cv_edit_dirty(cv_canvas *c, int *dirty, float *values, int cap)
{
    if (!c || cap < 0) return fail(VM_ERR_ARG, "cv_edit_dirty: bad arguments");
    int n = std::min(cap, c->lastEdit.ndirty);
    if (n <= 0) return VM_OK;
    cudaError_t e = cudaSuccess;
    if (dirty) e = cudaMemcpyAsync(dirty, c->dirty.p, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
    if (!e && values)
        e = cudaMemcpyAsync(values, c->dirtyVal.p, sizeof(float2) * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    return e ? cuda_fail(e, "cv_edit_dirty") : VM_OK;
}

int cv_info(cv_canvas *c, cv_info_t *out)
{
    if (!c || !out) return fail(VM_ERR_ARG, "cv_info: bad arguments");
    out->voxelsX = c->g.vx;
    out->voxelsY = c->g.vy;
    out->tilesX = c->g.tilesX;
    out->tilesY = c->g.tilesY;
    out->voxelSize = c->g.vs;
    out->numSlots = c->st.nslots;
    out->freeSlots = c->st.nfree;
    out->surfaceCount = c->st.surfaceCount;
    out->surfaceTiles = c->st.surfaceTiles;
    return VM_OK;
}

int cv_get_slots(cv_canvas *c, float *xy)
{
    if (!c || (!xy && c->st.nslots)) return fail(VM_ERR_ARG, "cv_get_slots: bad arguments");
    if (!c->st.nslots) return VM_OK;
    cudaError_t e = cudaMemcpyAsync(xy, c->slots.p, sizeof(float2) * (size_t)c->st.nslots, cudaMemcpyDeviceToHost,
                                    c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    return e ? cuda_fail(e, "cv_get_slots") : VM_OK;
}

int cv_get_inside(cv_canvas *c, uint64_t *masks)
{
    if (!c || !masks) return fail(VM_ERR_ARG, "cv_get_inside: bad arguments");
    cudaError_t e = cudaMemcpyAsync(masks, c->inside.p, c->tiles * 8, cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    return e ? cuda_fail(e, "cv_get_inside") : VM_OK;
}

int cv_get_inside_rect(cv_canvas *c, uint64_t *masks, int tx0, int ty0, int tx1, int ty1)
{
    if (!c || !masks) return fail(VM_ERR_ARG, "cv_get_inside_rect: bad arguments");
    tx0 = std::max(tx0, 0), ty0 = std::max(ty0, 0);
    tx1 = std::min(tx1, c->g.tilesX), ty1 = std::min(ty1, c->g.tilesY);
    if (tx0 >= tx1 || ty0 >= ty1) return VM_OK;
    size_t pitch = (size_t)c->g.tilesX * 8, off = (size_t)ty0 * c->g.tilesX + tx0;
    cudaError_t e = cudaMemcpy2DAsync(masks + off, pitch, c->inside.p + off, pitch, (size_t)(tx1 - tx0) * 8,
                                      (size_t)(ty1 - ty0), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    return e ? cuda_fail(e, "cv_get_inside_rect") : VM_OK;
}

int cv_get_surface(cv_canvas *c, uint64_t *masks, float *points, int *slots)
{
    if (!c) return fail(VM_ERR_ARG, "cv_get_surface: NULL handle");
    std::vector<unsigned long long> m(c->tiles);
    cudaError_t e = cudaMemcpyAsync(m.data(), c->smask.p, c->tiles * 8, cudaMemcpyDeviceToHost, c->stream);
    if (!e && points) e = cudaMemcpyAsync(points, c->spt.p, c->tiles * 64 * sizeof(float2), cudaMemcpyDeviceToHost, c->stream);
    if (!e && slots) e = cudaMemcpyAsync(slots, c->sslot.p, c->tiles * 64 * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    if (e) return cuda_fail(e, "cv_get_surface");
    if (masks) std::memcpy(masks, m.data(), c->tiles * 8);
    // voxels off the surface read (-1, -1) / -1
    for (size_t t = 0; t < c->tiles; ++t) {
        for (int b = 0; b < 64; ++b) {
            if ((m[t] >> b) & 1ull) continue;
            if (points) points[2 * (t * 64 + b)] = points[2 * (t * 64 + b) + 1] = -1.0f;
            if (slots) slots[t * 64 + b] = -1;
        }
    }
    return VM_OK;
}

int cv_get_free(cv_canvas *c, int *freeList)
{
    if (!c || (!freeList && c->st.nfree)) return fail(VM_ERR_ARG, "cv_get_free: bad arguments");
    if (!c->st.nfree) return VM_OK;
    cudaError_t e = cudaMemcpyAsync(freeList, c->freel.p, sizeof(int) * (size_t)c->st.nfree, cudaMemcpyDeviceToHost,
                                    c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    return e ? cuda_fail(e, "cv_get_free") : VM_OK;
}

static int cv_bit(cv_canvas *c, const unsigned long long *words, int i, int j, int *out)
{
    if (!c || !out) return fail(VM_ERR_ARG, "bad arguments");
    *out = 0;
    if (i < 0 || j < 0 || i >= c->g.vx || j >= c->g.vy) return VM_OK;
    unsigned long long w = 0;
    cudaError_t e = cudaMemcpyAsync(&w, words + (size_t)(j >> 3) * c->g.tilesX + (i >> 3), 8, cudaMemcpyDeviceToHost,
                                    c->stream);
    if (!e) e = cudaStreamSynchronize(c->stream);
    if (e) return cuda_fail(e, "canvas query");
    *out = (int)((w >> (((j & 7) << 3) | (i & 7))) & 1ull);
    return VM_OK;
}

int cv_is_inside(cv_canvas *c, int i, int j, int *out) { return cv_bit(c, c ? c->inside.p : nullptr, i, j, out); }

int cv_is_surface(cv_canvas *c, int i, int j, int *out) { return cv_bit(c, c ? c->smask.p : nullptr, i, j, out); }

} // extern "C"

cudaError_t vm_scan_ex(const int *in, int *out, int n, int *partial, cudaStream_t s)
{
    return scan_ex(in, out, n, partial, s);
}

int vm_scan_partials(int n) { return scan_partials(n); }

// Internal view for the optimiser hand-off (vm_runtime.cu).
namespace vmh {

int canvas_view(cv_canvas *c, CanvasView *v)
{
    if (!c || !v) return fail(VM_ERR_ARG, "NULL canvas");
    v->slots = c->slots.p;
    v->nslots = c->st.nslots;
    v->inside = c->inside.p;
    v->tilesX = c->g.tilesX;
    v->tilesY = c->g.tilesY;
    v->voxelSize = c->g.vs;
    v->dirty = c->dirty.p;
    v->dirtyValues = c->dirtyVal.p;
    v->ndirty = c->lastEdit.ndirty;
    v->tx0 = c->lastEdit.tx0;
    v->ty0 = c->lastEdit.ty0;
    v->tx1 = c->lastEdit.tx1;
    v->ty1 = c->lastEdit.ty1;
    v->stream = c->stream;
    return VM_OK;
}

cudaError_t canvas_fill_empty(float2 *p, size_t n, cudaStream_t s)
{
    if (!n) return cudaSuccess;
    k_cv_fill<<<(int)std::min<size_t>((n + 255) / 256, 1024), 256, 0, s>>>(p, n, make_float2(-1.0f, -1.0f));
    return cudaGetLastError();
}

cudaError_t canvas_copy_rect(const unsigned long long *src, unsigned long long *dst, int pitch, int tx0, int ty0,
                             int tx1, int ty1, cudaStream_t s)
{
    int w = tx1 - tx0, h = ty1 - ty0;
    if (w <= 0 || h <= 0) return cudaSuccess;
    k_cv_copy_rect<<<blocks_for((long long)w * h, 256), 256, 0, s>>>(src, dst, pitch, tx0, ty0, w, h);
    return cudaGetLastError();
}

} // namespace vmh
