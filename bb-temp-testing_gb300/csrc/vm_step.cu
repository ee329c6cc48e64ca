// VoroMesh optimisation step kernels (batch-native).
//
//   k_bin          cell key + atomic count per point        (reference binKernel, voro_optimizer.cu:168-177)
//   k_scan_tiles   per-tile sums of the cell counts          (reference cub ExclusiveSum, :697)
//   k_scan_apply   exclusive scan -> cell start
//   k_scatter      cell-sorted copy; the last writer of each cell sorts its run by
//                  slot index, so the ordering is canonical (reference scatterKernel :179-187)
//   k_loss         VoroLoss + analytic gradient per target  (reference vorolossKernel :199-266)
//   k_adam_bin     Adam + MultiStepLR + clamp, fused with the next step's binning
//                  (reference adamKernel :271-301 + binKernel)
//   k_finalize     publish a loss-only pass (EvaluateLoss, :746-761)
//   k_knn          exact kNN query operator (reference knn<K>, :130-163)
//
// One step of a set of fits is: k_loss -> k_adam_bin -> k_scan_tiles ->
// k_scan_apply -> k_scatter(publish). The grid is therefore always built for
// the current generators between steps, as the reference rebuilds it at the
// start of each step.
#include "vm_device.cuh"
#include "vm_grid.cuh"
#include "vm_knn.cuh"
#include "vm_kernels.h"

namespace vmk {

// ---------------------------------------------------------------------------
// hash grid build over a table of point sets (bodies in vm_grid.cuh)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_bin(const VmPointSet *__restrict__ sets, const int *__restrict__ prefix,
                                             int nSets, int emptyIsNegative)
{
    int f = find_fit(prefix, nSets, blockIdx.x);
    grid_bin_one(sets[f], (blockIdx.x - prefix[f]) * blockDim.x + threadIdx.x, emptyIsNegative);
}

__global__ void __launch_bounds__(256) k_scan_tiles(const VmPointSet *__restrict__ sets,
                                                    const int *__restrict__ prefix, int nSets)
{
    int f = find_fit(prefix, nSets, blockIdx.x);
    grid_tile_sum(sets[f], blockIdx.x - prefix[f]);
}

__global__ void __launch_bounds__(256) k_scan_apply(const VmPointSet *__restrict__ sets,
                                                    const int *__restrict__ prefix, int nSets)
{
    int f = find_fit(prefix, nSets, blockIdx.x);
    grid_tile_apply(sets[f], blockIdx.x - prefix[f]);
}

__global__ void __launch_bounds__(256) k_scatter(const VmPointSet *__restrict__ sets, const int *__restrict__ prefix,
                                                 int nSets, const VmFit *__restrict__ publish)
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
    }
    grid_scatter_one(sets[f], local * blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------------------------
// VoroLoss
// ---------------------------------------------------------------------------
struct TgtOut {
    int i0, j;
    float loss, gjx, gjy, g0x, g0y;
};

// Gradient of d^2 for target p, nearest site c0 and bisector neighbour cj,
// in the reference's operation order (voro_optimizer.cu:245-253).
__device__ __forceinline__ void grad_terms(float2 p, float2 c0, float2 cj, float bestD, TgtOut &o)
{
    float ux = p.x - c0.x, uy = p.y - c0.y;
    float ex = cj.x - c0.x, ey = cj.y - c0.y;
    float l = sqrtf(ex * ex + ey * ey);
    float il = 1.0f / l;
    float nx = il * ex, ny = il * ey;
    float un = ux * nx + uy * ny;
    float tx = ux - un * nx, ty = uy - un * ny;
    float il2 = 1.0f / l;
    float dcx = il2 * tx - 0.5f * nx, dcy = il2 * ty - 0.5f * ny;
    float s = 2.0f * bestD;
    o.gjx = s * dcx;
    o.gjy = s * dcy;
    o.g0x = -s * (nx + dcx);
    o.g0y = -s * (ny + dcy);
}

// Fast path: nearest site and bisector argmin from the (2R+1)^2 cell block
// around p, with certificates that no site outside the block can change
// either choice and that the chosen neighbour is among the K nearest.
// Returns 1 (used), 0 (unused: no neighbour) or -1 (not certified).
__device__ __noinline__ int loss_block(const VmFit &F, float2 p, int R, int K, TgtOut &o)
{
    int gw = F.gridW, gh = F.gridH;
    int cx = cell_coord(p.x, F.inv, gw), cy = cell_coord(p.y, F.inv, gh);
    int xlo = max(cx - R, 0), xhi = min(cx + R, gw - 1), ylo = max(cy - R, 0), yhi = min(cy + R, gh - 1);
    const int *__restrict__ start = F.start;
    const float2 *__restrict__ pos = F.sortedPos;
    const int *__restrict__ sid = F.sortedIdx;

    // pass 1: nearest site by (d2, index)
    float d0 = FLT_MAX;
    int i0 = -1, nblk = 0;
    float2 c0 = make_float2(0.0f, 0.0f);
    for (int y = ylo; y <= yhi; ++y) {
        int s0 = __ldg(&start[y * gw + xlo]), s1 = __ldg(&start[y * gw + xhi + 1]);
        nblk += s1 - s0;
        for (int s = s0; s < s1; ++s) {
            float2 q = __ldg(&pos[s]);
            int id = __ldg(&sid[s]);
            float dx = q.x - p.x, dy = q.y - p.y;
            float dd = dx * dx + dy * dy;
            if (key_less(dd, id, d0, i0)) {
                d0 = dd;
                i0 = id;
                c0 = q;
            }
        }
    }
    if (nblk == 0) return -1;

    // distance from p to the block's edge, less a slack covering the float
    // rounding of cell boundaries; sides on the grid border are unbounded
    float h = F.cell;
    float S = FLT_MAX;
    if (xlo > 0) S = fminf(S, p.x - (float)xlo * h);
    if (xhi < gw - 1) S = fminf(S, (float)(xhi + 1) * h - p.x);
    if (ylo > 0) S = fminf(S, p.y - (float)ylo * h);
    if (yhi < gh - 1) S = fminf(S, (float)(yhi + 1) * h - p.y);
    bool bounded = S < FLT_MAX;
    float S2 = FLT_MAX;
    if (bounded) {
        float scale = fmaxf(fmaxf(fabsf(p.x), fabsf(p.y)), (float)(max(xhi, yhi) + 1) * h);
        S = S - scale * 9.5367431640625e-07f; // 2^-20
        if (!(S > 0.0f)) return -1;
        S2 = S * S * 0.99999904632568359375f; // (1 - 2^-20)
        if (!(d0 < S2)) return -1;
    }

    // pass 2: argmin over j != c0 of (d^2, d2, index), reference arithmetic for d
    float ux = p.x - c0.x, uy = p.y - c0.y;
    float bdsq = FLT_MAX, bd = 0.0f, bdd = 0.0f;
    int bj = -1;
    float2 cj = make_float2(0.0f, 0.0f);
    for (int y = ylo; y <= yhi; ++y) {
        int s0 = __ldg(&start[y * gw + xlo]), s1 = __ldg(&start[y * gw + xhi + 1]);
        for (int s = s0; s < s1; ++s) {
            int id = __ldg(&sid[s]);
            if (id == i0) continue;
            float2 q = __ldg(&pos[s]);
            float ex = q.x - c0.x, ey = q.y - c0.y;
            float l = sqrtf(ex * ex + ey * ey);
            if (l < 1e-12f) continue;
            float d = (ux * ex + uy * ey) / l - 0.5f * l;
            float dsq = d * d;
            float dx = q.x - p.x, dy = q.y - p.y;
            float dd = dx * dx + dy * dy;
            bool better = bj < 0 ? dsq < FLT_MAX : (dsq < bdsq || (dsq == bdsq && key_less(dd, id, bdd, bj)));
            if (better) {
                bdsq = dsq;
                bd = d;
                bdd = dd;
                bj = id;
                cj = q;
            }
        }
    }
    if (bj < 0) return bounded ? -1 : 0;

    if (bounded) {
        // no site beyond the edge can reach d^2 <= bdsq: |d_s| >= (D_s - D0)/2
        float D0 = sqrtf(d0) * 1.00000095367431640625f;
        float L = 0.5f * (S - D0) - 3.814697265625e-06f * (S + D0); // 2^-18
        if (!(L > 0.0f) || !(L * L > bdsq * 1.000003814697265625f)) return -1;
        if (!(bdd < S2)) return -1;
    }
    if (nblk > K) {
        // rank of bj among all sites (all closer ones are inside the block)
        int rank = 0;
        for (int y = ylo; y <= yhi; ++y) {
            int s0 = __ldg(&start[y * gw + xlo]), s1 = __ldg(&start[y * gw + xhi + 1]);
            for (int s = s0; s < s1; ++s) {
                float2 q = __ldg(&pos[s]);
                float dx = q.x - p.x, dy = q.y - p.y;
                rank += key_less(dx * dx + dy * dy, __ldg(&sid[s]), bdd, bj) ? 1 : 0;
            }
        }
        if (rank >= K) return -1;
    }
    o.i0 = i0;
    o.j = bj;
    o.loss = bdsq;
    grad_terms(p, c0, cj, bd, o);
    return 1;
}

// Exact path: the reference's kNN ring search and bisector loop.
template <int K>
__device__ int loss_ring(const VmFit &F, float2 p, TgtOut &o)
{
    float d2[K];
    int idx[K];
    knn_ring<K>(F.start, F.sortedPos, F.sortedIdx, F.gridW, F.gridH, F.cell, F.inv, p, d2, idx);
    if (idx[0] < 0) return 0;
    int i0 = idx[0];
    float2 c0 = F.gen[i0];
    float ux = p.x - c0.x, uy = p.y - c0.y;
    float best = FLT_MAX, bestD = 0.0f;
    int bestJ = -1;
    float2 cj = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int k = 1; k < K; ++k) {
        int j = idx[k];
        if (j < 0) break;
        float2 g = F.gen[j];
        float ex = g.x - c0.x, ey = g.y - c0.y;
        float l = sqrtf(ex * ex + ey * ey);
        if (l < 1e-12f) continue;
        float d = (ux * ex + uy * ey) / l - 0.5f * l;
        if (d * d < best) {
            best = d * d;
            bestD = d;
            bestJ = j;
            cj = g;
        }
    }
    if (bestJ < 0) return 0;
    o.i0 = i0;
    o.j = bestJ;
    o.loss = best;
    grad_terms(p, c0, cj, bestD, o);
    return 1;
}

__device__ __noinline__ int loss_exact(const VmFit &F, float2 p, TgtOut &o)
{
    switch (F.K) {
    case 8: return loss_ring<8>(F, p, o);
    case 12: return loss_ring<12>(F, p, o);
    case 16: return loss_ring<16>(F, p, o);
    case 24: return loss_ring<24>(F, p, o);
    default: return loss_ring<32>(F, p, o);
    }
}

// Targets the block certificates could not settle are deferred to a queue and
// resolved by k_loss_exact in dense warps, so one hard target does not stall
// the 31 other lanes of its warp on the long ring search. The queue holds
// every live target, so it cannot overflow.
struct SlowQueue {
    int count;
    int capacity;
    int2 *items; // (fit, local target index)
};

constexpr int kStage = 64; // staged candidates per warp (5x5 cell block)

// Per-warp staging of the 5x5 cell block around the warp's shared cell:
// ring-1 cells first (entries [0, m1)), then ring 2 (entries [m1, m2)).
// dmin/dmax bound the squared distance from any point of the cell's box to
// the site, so warp-uniform tests can skip sites no lane can need.
struct WarpStage {
    float x[kStage], y[kStage], dmin[kStage];
    int id[kStage];
    int segStart[11], segOff[11];
    // compacted candidate lists: sites that can be nearest to a box point
    // (built at staging) and the ring-2 sites some lane may need (per batch)
    float nx[kStage], ny[kStage], rx[kStage], ry[kStage];
    int nid[kStage], nk[kStage], rid[kStage], rk[kStage];
    int nNear, nRing;
};

// Appends the entries e of [lo, hi) with keep(e) to a compacted list in
// index order (warp-cooperative, two entries per lane).
template <class Keep, class Put>
__device__ __forceinline__ int warp_compact(int lo, int hi, Keep keep, Put put)
{
    int lane = threadIdx.x & 31;
    int n = 0;
    for (int base = lo; base < hi; base += 32) {
        int e = base + lane;
        bool k = e < hi && keep(e);
        unsigned b = __ballot_sync(kFull, k);
        if (k) put(n + __popc(b & ((1u << lane) - 1u)), e);
        n += __popc(b);
    }
    return n;
}

// All sites of the block, exact argmin of (d^2, d2, index) (the rare case
// where two candidates' error bounds overlap).
__device__ __noinline__ int staged_exact_argmin(const WarpStage &W, int m, float2 p, int i0, float c0x, float c0y,
                                                float &bdsq, float &bd, float &bdd, int &kb)
{
    float ux = p.x - c0x, uy = p.y - c0y;
    int bj = -1;
    kb = -1;
    for (int k = 0; k < m; ++k) {
        int id = W.id[k];
        if (id == i0) continue;
        float ex = W.x[k] - c0x, ey = W.y[k] - c0y;
        float l = sqrtf(ex * ex + ey * ey);
        if (l < 1e-12f) continue;
        float d = (ux * ex + uy * ey) / l - 0.5f * l;
        float dsq = d * d;
        float dx = W.x[k] - p.x, dy = W.y[k] - p.y;
        float dd = dx * dx + dy * dy;
        bool better = bj < 0 ? dsq < FLT_MAX : (dsq < bdsq || (dsq == bdsq && key_less(dd, id, bdd, bj)));
        if (better) {
            bdsq = dsq;
            bd = d;
            bdd = dd;
            bj = id;
            kb = k;
        }
    }
    return bj;
}

__device__ __noinline__ int staged_rank(const WarpStage &W, int m, float2 p, float bdd, int bj)
{
    int rank = 0;
    for (int k = 0; k < m; ++k) {
        float dx = W.x[k] - p.x, dy = W.y[k] - p.y;
        rank += key_less(dx * dx + dy * dy, W.id[k], bdd, bj) ? 1 : 0;
    }
    return rank;
}

// Staged fast path. Every lane of the warp calls it (take = this lane's
// target is in the pass); `prune` says every taking lane lies in the cell
// box, which makes the dmin/dmax bounds valid for all of them. Returns
// 1 used, 0 unused, -1 not certified; l0/lj are the staged indices of the
// nearest site and the bisector neighbour.
__device__ __forceinline__ int loss_staged(const VmFit &F, const WarpStage &W, bool take, float2 p, int m1, int m2,
                                           float U, bool prune, int xlo, int xhi, int ylo, int yhi,
                                           TgtOut &o, int &l0, int &lj, float &bddOut)
{
    // pass 1: nearest by (d2, index) among the sites that can be nearest to
    // some point of the box (dmin <= U, U >= every point's nearest distance^2)
    float d0 = FLT_MAX;
    int i0 = -1, k0 = 0;
    int nNear = W.nNear;
    for (int q = 0; q < nNear; ++q) {
        float dx = W.nx[q] - p.x, dy = W.ny[q] - p.y;
        float dd = dx * dx + dy * dy;
        int id = W.nid[q];
        if (key_less(dd, id, d0, i0)) {
            d0 = dd;
            i0 = id;
            k0 = q;
        }
    }
    k0 = W.nk[k0];
    float c0x = W.x[k0], c0y = W.y[k0];
    float ux = p.x - c0x, uy = p.y - c0y;
    // pass 2a: rsqrt estimates of |d| with a rigorous 2^-19 relative bound;
    // ring-1 sites for every lane, ring-2 sites only if some lane could need
    // them: |d_s| >= (D_s - D0)/2, so s cannot beat the best estimate when
    // d2(p, s) > (D0 + 2 (best + eps))^2.
    float best = FLT_MAX, bestEps = 0.0f, lowOther = FLT_MAX;
    int kb = -1;
    bool special = false;
    float sqD0 = sqrtf(d0);
    auto consider = [&](float sx_, float sy_, int k) {
        float ex = sx_ - c0x, ey = sy_ - c0y;
        float ee = ex * ex + ey * ey;
        float dot = ux * ex + uy * ey;
        bool tiny = ee <= 1e-20f;
        special |= tiny && k != k0;
        float rs = rsqrtf(ee);
        float a = dot * rs, b = 0.5f * (ee * rs);
        float est = fabsf(a - b);
        float eps = 1.9073486328125e-06f * (fabsf(a) + b) + 1e-30f;
        if (k == k0 || tiny) est = FLT_MAX;
        if (est < best) {
            lowOther = fminf(lowOther, best - bestEps);
            best = est;
            bestEps = eps;
            kb = k;
        } else {
            lowOther = fminf(lowOther, est - eps);
        }
    };
    for (int k = 0; k < m1; ++k) consider(W.x[k], W.y[k], k);
    if (m2 > m1) {
        // 0.1% slack covers every float rounding in this chain of bounds
        float T = best < FLT_MAX ? 1.001f * (sqD0 + 2.0f * (best + bestEps)) : FLT_MAX;
        T = T < FLT_MAX ? T * T + 1e-30f : FLT_MAX;
        if (!take) T = 0.0f;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) T = fmaxf(T, __shfl_xor_sync(kFull, T, off));
        float Tmax = prune ? T : FLT_MAX;
        WarpStage &Wm = const_cast<WarpStage &>(W);
        int nr = warp_compact(m1, m2, [&](int e) { return W.dmin[e] <= Tmax; },
                              [&](int slot, int e) {
                                  Wm.rx[slot] = W.x[e];
                                  Wm.ry[slot] = W.y[e];
                                  Wm.rk[slot] = e;
                              });
        __syncwarp();
        for (int q = 0; q < nr; ++q) consider(W.rx[q], W.ry[q], W.rk[q]);
        __syncwarp();
    }
    if (!take) return 0;
    if (i0 < 0) return -1;
    // pass 2b: exact reference value of the best; full exact argmin only when
    // another candidate's bound overlaps it
    float bdsq = FLT_MAX, bd = 0.0f, bdd = 0.0f;
    int bj = -1;
    if (special || lowOther <= best + bestEps) {
        bj = staged_exact_argmin(W, m2, p, i0, c0x, c0y, bdsq, bd, bdd, kb);
    } else if (kb >= 0) {
        float ex = W.x[kb] - c0x, ey = W.y[kb] - c0y;
        float l = sqrtf(ex * ex + ey * ey);
        float d = (ux * ex + uy * ey) / l - 0.5f * l;
        bdsq = d * d;
        if (bdsq < FLT_MAX) {
            bd = d;
            float dx = W.x[kb] - p.x, dy = W.y[kb] - p.y;
            bdd = dx * dx + dy * dy;
            bj = W.id[kb];
        }
    }
    // certificates against the sites outside the 5x5 block
    int gw = F.gridW, gh = F.gridH;
    float h = F.cell;
    float S = FLT_MAX;
    if (xlo > 0) S = fminf(S, p.x - (float)xlo * h);
    if (xhi < gw - 1) S = fminf(S, (float)(xhi + 1) * h - p.x);
    if (ylo > 0) S = fminf(S, p.y - (float)ylo * h);
    if (yhi < gh - 1) S = fminf(S, (float)(yhi + 1) * h - p.y);
    bool bounded = S < FLT_MAX;
    if (bj < 0) return bounded ? -1 : 0;
    if (bounded) {
        float scale = fmaxf(fmaxf(fabsf(p.x), fabsf(p.y)), (float)(max(xhi, yhi) + 1) * h);
        S = S - scale * 9.5367431640625e-07f; // 2^-20
        if (!(S > 0.0f)) return -1;
        float S2 = S * S * 0.99999904632568359375f;
        if (!(d0 < S2) || !(bdd < S2)) return -1;
        float D0 = sqD0 * 1.00000095367431640625f;
        float L = 0.5f * (S - D0) - 3.814697265625e-06f * (S + D0);
        if (!(L > 0.0f) || !(L * L > bdsq * 1.000003814697265625f)) return -1;
    }
    o.i0 = i0;
    o.j = bj;
    o.loss = bdsq;
    grad_terms(p, make_float2(c0x, c0y), make_float2(W.x[kb], W.y[kb]), bd, o);
    l0 = k0;
    lj = kb;
    bddOut = bdd;
    return 1;
}

// 64-bit exact accumulation in shared memory from native 32-bit atomics: the
// low word's carry is detected from its old value and added to the high word.
struct Acc32 {
    unsigned lo;
    int hi;
};

__device__ __forceinline__ void acc32_add(Acc32 &a, long long v)
{
    unsigned lo = (unsigned)(unsigned long long)v;
    int hi = (int)(v >> 32);
    unsigned old = atomicAdd(&a.lo, lo);
    if (old + lo < old) hi += 1;
    if (hi) atomicAdd(&a.hi, hi);
}

__device__ __forceinline__ unsigned long long acc32_take(Acc32 &a)
{
    unsigned long long v = ((unsigned long long)(unsigned)a.hi << 32) | a.lo;
    a.lo = 0;
    a.hi = 0;
    return v;
}

// Stages the 5x5 block around cell (cx, cy) into W; returns m2 (> kStage:
// not staged) and m1 (ring-1 entries). Also U, the upper bound of every box
// point's squared nearest distance, and the dmin bounds.
__device__ __forceinline__ int stage_block(const VmFit &F, WarpStage &W, int cx, int cy, float bx0, float bx1,
                                           float by0, float by1, int &m1, float &U)
{
    int lane = threadIdx.x & 31;
    int gw = F.gridW, gh = F.gridH;
    int s0 = 0, n = 0;
    if (lane < 11) {
        int y, xa, xb;
        if (lane < 3) {
            y = cy - 1 + lane; xa = cx - 1; xb = cx + 1;
        } else if (lane < 5) {
            y = lane == 3 ? cy - 2 : cy + 2; xa = cx - 2; xb = cx + 2;
        } else if (lane < 8) {
            y = cy - 1 + (lane - 5); xa = xb = cx - 2;
        } else {
            y = cy - 1 + (lane - 8); xa = xb = cx + 2;
        }
        xa = max(xa, 0);
        xb = min(xb, gw - 1);
        if (y >= 0 && y < gh && xa <= xb) {
            s0 = __ldg(&F.start[y * gw + xa]);
            n = __ldg(&F.start[y * gw + xb + 1]) - s0;
        }
    }
    int incl = n;
#pragma unroll
    for (int off = 1; off < 16; off <<= 1) {
        int t = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl += t;
    }
    m1 = __shfl_sync(kFull, incl, 2);
    int m2 = __shfl_sync(kFull, incl, 10);
    if (m2 > kStage) return m2;
    if (lane < 11) {
        W.segStart[lane] = s0;
        W.segOff[lane] = incl - n;
    }
    __syncwarp();
    float dmaxLo = FLT_MAX;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        int e = lane + 32 * r;
        if (e < m2) {
            int k = 10;
            while (W.segOff[k] > e) --k;
            int s = W.segStart[k] + (e - W.segOff[k]);
            float2 q = __ldg(&F.sortedPos[s]);
            W.x[e] = q.x;
            W.y[e] = q.y;
            W.id[e] = __ldg(&F.sortedIdx[s]);
            float gx = fmaxf(fmaxf(bx0 - q.x, q.x - bx1), 0.0f), gy = fmaxf(fmaxf(by0 - q.y, q.y - by1), 0.0f);
            W.dmin[e] = (gx * gx + gy * gy) * 0.9999961853027344f; // (1 - 2^-18)
            float fx = fmaxf(fabsf(q.x - bx0), fabsf(q.x - bx1)), fy = fmaxf(fabsf(q.y - by0), fabsf(q.y - by1));
            dmaxLo = fminf(dmaxLo, (fx * fx + fy * fy) * 1.0000038146972656f); // (1 + 2^-18)
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) dmaxLo = fminf(dmaxLo, __shfl_xor_sync(kFull, dmaxLo, off));
    U = dmaxLo;
    __syncwarp();
    return m2;
}

// The compacted list of sites that can be nearest to some point of the box
// (all of them when the bounds do not hold for every lane).
__device__ __forceinline__ void stage_near(WarpStage &W, int m2, float U, bool prune)
{
    int n = warp_compact(0, m2, [&](int e) { return !prune || W.dmin[e] <= U; },
                         [&](int slot, int e) {
                             W.nx[slot] = W.x[e];
                             W.ny[slot] = W.y[e];
                             W.nid[slot] = W.id[e];
                             W.nk[slot] = e;
                         });
    if ((threadIdx.x & 31) == 0) W.nNear = n;
    __syncwarp();
}

// AGG selects how a warp's gradient terms reach the int64 accumulators:
//   0 shared-memory 64-bit atomics on the staged sites, 1 a global reduction
//   per term, 2 match_any + shuffle tree per distinct site, 3 shared-memory
//   accumulation from 32-bit atomics. All four give the identical integer sum.
template <int THREADS, int MINB, int AGG>
__global__ void __launch_bounds__(THREADS, MINB)
    k_loss(const VmFit *__restrict__ fits, const int *__restrict__ prefix, int nFits, int mode, int maxR,
           SlowQueue *queue)
{
    constexpr int NW = THREADS / 32;
    __shared__ unsigned long long sLo[NW], sHi[NW];
    __shared__ int sCnt[NW], sSlow[NW];
    __shared__ WarpStage sStage[NW];
    __shared__ unsigned long long sAcc[AGG == 0 ? NW : 1][kStage][2];
    __shared__ Acc32 sAcc32[AGG == 3 ? NW : 1][kStage][2];
    int totalTiles = prefix[nFits];
    long long t0 = (long long)blockIdx.x * totalTiles / gridDim.x;
    long long t1 = (long long)(blockIdx.x + 1) * totalTiles / gridDim.x;
    if (t0 >= t1) return;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    WarpStage &W = sStage[warp];
    unsigned long long(*acc)[2] = sAcc[AGG == 0 ? warp : 0];
    Acc32(*acc32)[2] = sAcc32[AGG == 3 ? warp : 0];
    for (int r = 0; r < 2; ++r) {
        if (AGG == 0) {
            acc[lane + 32 * r][0] = 0;
            acc[lane + 32 * r][1] = 0;
        }
        if (AGG == 3) {
            acc32[lane + 32 * r][0] = Acc32{0u, 0};
            acc32[lane + 32 * r][1] = Acc32{0u, 0};
        }
    }
    int f = find_fit(prefix, nFits, (int)t0);
    unsigned long long aLo = 0, aHi = 0;
    int aCnt = 0, aSlow = 0;
    int stCell = -1, stFit = -1, stM1 = 0, stM2 = 0, stPrune = -1; // this warp's staged block
    float stU = FLT_MAX;
    for (long long t = t0; t <= t1; ++t) {
        bool flush = (t == t1) || (t >= prefix[f + 1]);
        if (flush) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                unsigned long long olo = __shfl_down_sync(kFull, aLo, off);
                unsigned long long ohi = __shfl_down_sync(kFull, aHi, off);
                add128(aLo, aHi, olo, ohi);
                aCnt += __shfl_down_sync(kFull, aCnt, off);
                aSlow += __shfl_down_sync(kFull, aSlow, off);
            }
            if (lane == 0) {
                sLo[warp] = aLo;
                sHi[warp] = aHi;
                sCnt[warp] = aCnt;
                sSlow[warp] = aSlow;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                unsigned long long lo = 0, hi = 0;
                int cnt = 0, slow = 0;
                for (int w = 0; w < NW; ++w) {
                    add128(lo, hi, sLo[w], sHi[w]);
                    cnt += sCnt[w];
                    slow += sSlow[w];
                }
                VmState *st = fits[f].state;
                if (fits[f].active || mode == 1) {
                    atomic_add128(&st->accLo, &st->accHi, lo, hi);
                    if (cnt) atomicAdd(&st->accCount, cnt);
                    if (slow) atomicAdd(&st->slowTotal, slow);
                }
            }
            __syncthreads();
            aLo = aHi = 0;
            aCnt = aSlow = 0;
            if (t == t1) break;
            while (t >= prefix[f + 1]) ++f;
        }
        const VmFit &F = fits[f];
        bool active = F.active || mode == 1;
        int local = (int)(t - prefix[f]) * THREADS + threadIdx.x;
        bool valid = active && local < F.nTargets;
        float2 p = make_float2(0.0f, 0.0f);
        bool take = false;
        int cx = 0, cy = 0;
        if (valid) {
            p = F.tpos[local];
            take = true;
            if (mode == 0) {
                take = p.x >= F.bx0 && p.x <= F.bx1 && p.y >= F.by0 && p.y <= F.by1;
                if (take && F.fraction < 1.0f)
                    take = rand01((unsigned)F.tslot[local], (unsigned)(F.state->iter + 1), F.seed) < F.fraction;
            }
            cx = cell_coord(p.x, F.inv, F.gridW);
            cy = cell_coord(p.y, F.inv, F.gridH);
        }
        // one staged 5x5 block for the whole warp when all its targets share a cell
        unsigned takers = __ballot_sync(kFull, take);
        int leader = takers ? __ffs(takers) - 1 : 0;
        int cell = cy * F.gridW + cx;
        int lcell = __shfl_sync(kFull, cell, leader);
        bool uniform = takers != 0 && __all_sync(kFull, !take || cell == lcell);
        int m1 = 0, m2 = 0;
        float U = FLT_MAX;
        bool prune = false;
        int xlo = 0, xhi = 0, ylo = 0, yhi = 0;
        if (uniform) {
            int gw = F.gridW;
            int lcy = lcell / gw, lcx = lcell - lcy * gw;
            float h = F.cell;
            float bsl = (float)(max(lcx, lcy) + 2) * h * 9.5367431640625e-07f + 1e-30f; // 2^-20 slack
            float bx0 = (float)lcx * h - bsl, bx1 = (float)(lcx + 1) * h + bsl;
            float by0 = (float)lcy * h - bsl, by1 = (float)(lcy + 1) * h + bsl;
            prune = __all_sync(kFull, !take || (p.x >= bx0 && p.x <= bx1 && p.y >= by0 && p.y <= by1));
            if (lcell != stCell || f != stFit) {
                // restage only when the warp moves to another cell
                stM2 = stage_block(F, W, lcx, lcy, bx0, bx1, by0, by1, stM1, stU);
                stCell = lcell;
                stFit = f;
                stPrune = -1;
            }
            m1 = stM1;
            m2 = stM2;
            U = stU;
            if (m2 > kStage) {
                uniform = false;
            } else {
                if (stPrune != (int)prune) {
                    stage_near(W, m2, U, prune);
                    stPrune = (int)prune;
                }
                xlo = max(lcx - 2, 0), xhi = min(lcx + 2, gw - 1);
                ylo = max(lcy - 2, 0), yhi = min(lcy + 2, F.gridH - 1);
            }
        }
        TgtOut o;
        int used = 0, slow = 0, l0 = -1, lj = -1;
        bool deferred = false;
        int r = -1;
        if (uniform) {
            float bdd = 0.0f;
            r = loss_staged(F, W, take, p, m1, m2, U, prune, xlo, xhi, ylo, yhi, o, l0, lj, bdd);
            if (m2 > F.K) {
                // bj must rank below K among all sites; every closer site is staged
                // (certified), and a site s is closer only if dmin(s) <= d2(p, bj).
                // One warp vote settles it unless K staged sites are that near.
                float lim = (take && r > 0) ? bdd * 1.0000038146972656f : 0.0f;
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) lim = fmaxf(lim, __shfl_xor_sync(kFull, lim, off));
                int cnt = __popc(__ballot_sync(kFull, lane < m2 && W.dmin[lane] <= lim)) +
                          __popc(__ballot_sync(kFull, lane + 32 < m2 && W.dmin[lane + 32] <= lim));
                if ((cnt >= F.K || !prune) && take && r > 0 && staged_rank(W, m2, p, bdd, o.j) >= F.K) r = -1;
            }
        }
        if (take) {
            if (!uniform) {
                r = loss_block(F, p, 1, F.K, o);
                if (r < 0) r = loss_block(F, p, 2, F.K, o);
            }
            if (r < 0) {
                int q = atomicAdd(&queue->count, 1);
                queue->items[q] = make_int2(f, local); // capacity >= live targets
                r = 0;
                deferred = true;
                slow = 1;
            }
            used = r;
        }
        if (!used) l0 = lj = -1;
        if (F.dbgI0 && valid && !deferred) {
            F.dbgI0[local] = used ? o.i0 : -1;
            F.dbgJ[local] = used ? o.j : -1;
            F.dbgLoss[local] = used ? o.loss : 0.0f;
        }
        if (used) {
            unsigned long long lo, hi;
            fxl_from_float(o.loss, F.lossExp, lo, hi);
            add128(aLo, aHi, lo, hi);
            aCnt += 1;
        }
        aSlow += slow;
        if (mode == 0) {
            int e = F.gradExp;
            long long gjx = used ? fx_from_float(o.gjx, e) : 0, gjy = used ? fx_from_float(o.gjy, e) : 0;
            long long g0x = used ? fx_from_float(o.g0x, e) : 0, g0y = used ? fx_from_float(o.g0y, e) : 0;
            bool staged = used && l0 >= 0;
            unsigned long long *G = reinterpret_cast<unsigned long long *>(F.gradX);
            if (AGG == 1 || (AGG == 3 && !uniform)) {
                // one fire-and-forget global reduction per term
                if (used) {
                    atomicAdd(&G[2 * (size_t)o.j], (unsigned long long)gjx);
                    atomicAdd(&G[2 * (size_t)o.j + 1], (unsigned long long)gjy);
                    atomicAdd(&G[2 * (size_t)o.i0], (unsigned long long)g0x);
                    atomicAdd(&G[2 * (size_t)o.i0 + 1], (unsigned long long)g0y);
                }
            } else if (AGG == 2 || (AGG == 0 && !uniform)) {
                if (__any_sync(kFull, used)) {
                    warp_add_pair(F.gradX, used ? o.j : -1, gjx, gjy);
                    warp_add_pair(F.gradX, used ? o.i0 : -1, g0x, g0y);
                }
            } else {
                // uniform warp, AGG 0 or 3: accumulate the staged sites in shared
                // memory, flush once per warp; other lanes reduce straight to global
                if (staged) {
                    if (AGG == 0) {
                        atomicAdd(&acc[lj][0], (unsigned long long)gjx);
                        atomicAdd(&acc[lj][1], (unsigned long long)gjy);
                        atomicAdd(&acc[l0][0], (unsigned long long)g0x);
                        atomicAdd(&acc[l0][1], (unsigned long long)g0y);
                    } else {
                        acc32_add(acc32[lj][0], gjx);
                        acc32_add(acc32[lj][1], gjy);
                        acc32_add(acc32[l0][0], g0x);
                        acc32_add(acc32[l0][1], g0y);
                    }
                } else if (used) {
                    atomicAdd(&G[2 * (size_t)o.j], (unsigned long long)gjx);
                    atomicAdd(&G[2 * (size_t)o.j + 1], (unsigned long long)gjy);
                    atomicAdd(&G[2 * (size_t)o.i0], (unsigned long long)g0x);
                    atomicAdd(&G[2 * (size_t)o.i0 + 1], (unsigned long long)g0y);
                }
                __syncwarp();
                for (int e = lane; e < m2; e += 32) {
                    unsigned long long ax, ay;
                    if (AGG == 0) {
                        ax = acc[e][0];
                        ay = acc[e][1];
                        acc[e][0] = 0;
                        acc[e][1] = 0;
                    } else {
                        ax = acc32_take(acc32[e][0]);
                        ay = acc32_take(acc32[e][1]);
                    }
                    unsigned long long *g = G + 2 * (size_t)W.id[e];
                    if (ax) atomicAdd(&g[0], ax);
                    if (ay) atomicAdd(&g[1], ay);
                }
                __syncwarp();
            }
        }
    }
}

// The deferred targets: exact ring search, one target per thread, with the
// loss, count and gradient added straight into the fit's accumulators.
__global__ void __launch_bounds__(128) k_loss_exact(const VmFit *__restrict__ fits, int mode, SlowQueue *queue)
{
    int n = min(queue->count, queue->capacity);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        int2 it = queue->items[q];
        const VmFit &F = fits[it.x];
        float2 p = F.tpos[it.y];
        TgtOut o;
        int used = loss_exact(F, p, o);
        if (F.dbgI0) {
            F.dbgI0[it.y] = used ? o.i0 : -1;
            F.dbgJ[it.y] = used ? o.j : -1;
            F.dbgLoss[it.y] = used ? o.loss : 0.0f;
        }
        if (!used) continue;
        unsigned long long lo, hi;
        fxl_from_float(o.loss, F.lossExp, lo, hi);
        atomic_add128(&F.state->accLo, &F.state->accHi, lo, hi);
        atomicAdd(&F.state->accCount, 1);
        if (mode == 0) {
            int e = F.gradExp;
            unsigned long long *g = reinterpret_cast<unsigned long long *>(F.gradX);
            atomicAdd(&g[2 * (size_t)o.j], (unsigned long long)fx_from_float(o.gjx, e));
            atomicAdd(&g[2 * (size_t)o.j + 1], (unsigned long long)fx_from_float(o.gjy, e));
            atomicAdd(&g[2 * (size_t)o.i0], (unsigned long long)fx_from_float(o.g0x, e));
            atomicAdd(&g[2 * (size_t)o.i0 + 1], (unsigned long long)fx_from_float(o.g0y, e));
        }
    }
}

// Publishes a loss-only pass: loss and count of the accumulator, iteration kept.
__global__ void k_finalize(const VmFit *__restrict__ fits, int nFits, SlowQueue *queue)
{
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f == 0) queue->count = 0;
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
// Adam (fused with the next grid's binning)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float pow_det(float base, int t)
{
    double r = 1.0, x = (double)base;
    unsigned e = t < 0 ? 0u : (unsigned)t;
    while (e) {
        if (e & 1u) r = __dmul_rn(r, x);
        x = __dmul_rn(x, x);
        e >>= 1;
    }
    return __double2float_rn(r);
}

__global__ void __launch_bounds__(256) k_adam_bin(const VmFit *__restrict__ fits, const int *__restrict__ prefix,
                                                  int nFits, SlowQueue *queue)
{
    __shared__ float sLr, sBc1, sBc2, sScale;
    if (blockIdx.x == 0 && threadIdx.x == 0) queue->count = 0;
    int f = find_fit(prefix, nFits, blockIdx.x);
    const VmFit &F = fits[f];
    if (!F.active) return;
    if (threadIdx.x == 0) {
        int t = F.state->iter + 1;
        float lr = F.lr;
        for (int k = 0; k < 4; ++k)
            if (t - 1 >= F.milestones[k]) lr *= F.gamma;
        sLr = lr;
        sBc1 = 1.0f - pow_det(F.beta1, t);
        sBc2 = 1.0f - pow_det(F.beta2, t);
        int count = F.state->accCount;
        sScale = 1.0f / (float)(count > 1 ? count : 1);
    }
    __syncthreads();
    int i = (blockIdx.x - prefix[f]) * blockDim.x + threadIdx.x;
    if (i >= F.nSlots) return;
    longlong2 gq = reinterpret_cast<const longlong2 *>(F.gradX)[i];
    if (gq.x | gq.y) reinterpret_cast<longlong2 *>(F.gradX)[i] = make_longlong2(0, 0);
    float2 p = F.gen[i];
    int sx = i % F.slotsW, sy = i / F.slotsW;
    if (p.x >= 0.0f && sx >= F.cx0 && sx < F.cx1 && sy >= F.cy0 && sy < F.cy1) {
        float grx = sScale * fx_to_float(gq.x, F.gradExp);
        float gry = sScale * fx_to_float(gq.y, F.gradExp);
        float2 m = F.m[i], v = F.v[i];
        float b1 = F.beta1, b2 = F.beta2;
        float mx = b1 * m.x + (1.0f - b1) * grx;
        float my = b1 * m.y + (1.0f - b1) * gry;
        float vx = b2 * v.x + (1.0f - b2) * (grx * grx);
        float vy = b2 * v.y + (1.0f - b2) * (gry * gry);
        F.m[i] = make_float2(mx, my);
        F.v[i] = make_float2(vx, vy);
        float lr = sLr, bc1 = sBc1, bc2 = sBc2, eps = F.eps;
        p.x -= lr * (mx / bc1) / (sqrtf(vx / bc2) + eps);
        p.y -= lr * (my / bc1) / (sqrtf(vy / bc2) + eps);
        p.x = fminf(fmaxf(p.x, 0.0f), F.width);
        p.y = fminf(fmaxf(p.y, 0.0f), F.height);
        F.gen[i] = p;
    }
    if (p.x < 0.0f) {
        F.key[i] = -1;
        return;
    }
    int c = cell_coord(p.y, F.inv, F.gridH) * F.gridW + cell_coord(p.x, F.inv, F.gridW);
    F.key[i] = c;
    F.rank[i] = atomicAdd(&F.counts[c], 1);
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

cudaError_t vm_launch_scatter(const VmPointSet *sets, const int *prefix, int nSets, int totalBlocks,
                              const VmFit *publish, cudaStream_t s)
{
    if (totalBlocks <= 0) return cudaSuccess;
    k_scatter<<<totalBlocks, 256, 0, s>>>(sets, prefix, nSets, publish);
    return cudaGetLastError();
}

// Loss kernel variants (block size, min blocks per SM, gradient aggregation).
struct LossVariant {
    int threads, minBlocks, agg;
};
static const LossVariant kVariants[] = {{256, 4, 0}, {256, 4, 1}, {256, 4, 2}, {256, 4, 3},
                                        {256, 3, 1}, {256, 3, 3}, {64, 16, 1}, {64, 16, 3}};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

int vm_loss_variants() { return kNumVariants; }
int vm_loss_variant_threads(int v) { return kVariants[v < 0 || v >= kNumVariants ? 0 : v].threads; }

template <int T, int B, int A> static void *loss_fn() { return (void *)k_loss<T, B, A>; }

static void *variant_fn(int v)
{
    switch (v) {
    case 0: return loss_fn<256, 4, 0>();
    case 1: return loss_fn<256, 4, 1>();
    case 2: return loss_fn<256, 4, 2>();
    case 3: return loss_fn<256, 4, 3>();
    case 4: return loss_fn<256, 3, 1>();
    case 5: return loss_fn<256, 3, 3>();
    case 6: return loss_fn<64, 16, 1>();
    default: return loss_fn<64, 16, 3>();
    }
}

cudaError_t vm_launch_loss(const VmFit *fits, const int *tilePrefix, int nFits, int totalTiles, int mode, int maxR,
                           int gridBlocks, int variant, void *queue, cudaStream_t s)
{
    if (totalTiles <= 0) return cudaSuccess;
    int g = gridBlocks < totalTiles ? gridBlocks : totalTiles;
    if (g < 1) g = 1;
    SlowQueue *q = static_cast<SlowQueue *>(queue);
    void *args[] = {(void *)&fits, (void *)&tilePrefix, (void *)&nFits, (void *)&mode, (void *)&maxR, (void *)&q};
    cudaError_t e = cudaLaunchKernel(variant_fn(variant), dim3(g), dim3(vm_loss_variant_threads(variant)), args, 0, s);
    if (e) return e;
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    k_loss_exact<<<sms * 2, 128, 0, s>>>(fits, mode, q);
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

cudaError_t vm_launch_scatter_targets(float2 *targets, const int *slots, const float2 *values, int n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    k_scatter_targets<<<(n + 127) / 128, 128, 0, s>>>(targets, slots, values, n);
    return cudaGetLastError();
}

int vm_loss_occupancy_blocks(int variant)
{
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, variant_fn(variant), vm_loss_variant_threads(variant), 0);
    if (per < 1) per = 1;
    return sms * per;
}

} // extern "C++"
