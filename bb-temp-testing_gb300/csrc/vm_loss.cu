// VoroLoss pass over a set of fits (reference vorolossKernel,
// voro_optimizer.cu:199-266): per live target the nearest site i0, the
// bisector neighbour j among its K nearest sites, the loss d^2 and the
// analytic gradient terms, summed in fixed point (order independent).
//
//   k_loss        warp-staged 5x5 cell blocks with certificates; uncertain
//                 targets go to a queue
//   k_loss_exact  the queued targets: exact ring search, one per thread
//   k_small_grid  the rest of a small fit's step in one block: the queued
//                 targets and Adam schedule, Adam, binning, scan, scatter
//                 (here beside k_loss_exact, whose pass it runs first)
#include "vm_device.cuh"
#include "vm_adam.cuh"
#include "vm_knn.cuh"
#include "vm_kernels.h"

namespace vmk {


// ---------------------------------------------------------------------------
// VoroLoss
// ---------------------------------------------------------------------------
struct TgtOut {
    int i0, j;
    float loss, gjx, gjy, g0x, g0y;
};

// Gradient of d^2 for target p, nearest site c0 and bisector neighbour cj,
// in the reference's operation order (voro_optimizer.cu:245-253).
// u = p - c0, e = cj - c0, l = |e| (sqrtf of ex*ex + ey*ey).
__device__ __forceinline__ void grad_terms_e(float ux, float uy, float ex, float ey, float l, float bestD, TgtOut &o)
{
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

__device__ __forceinline__ void grad_terms(float2 p, float2 c0, float2 cj, float bestD, TgtOut &o)
{
    float ux = p.x - c0.x, uy = p.y - c0.y;
    float ex = cj.x - c0.x, ey = cj.y - c0.y;
    grad_terms_e(ux, uy, ex, ey, sqrtf(ex * ex + ey * ey), bestD, o);
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

// ---------------------------------------------------------------------------
// warp-staged fast path
// ---------------------------------------------------------------------------
constexpr int kStage = 64; // staged candidates per warp (5x5 cell block)

__device__ __forceinline__ float warp_min(float v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fminf(v, __shfl_xor_sync(kFull, v, off));
    return v;
}

__device__ __forceinline__ float warp_max(float v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fmaxf(v, __shfl_xor_sync(kFull, v, off));
    return v;
}

// Per-warp shared staging of the 5x5 cell block around a group's cell, the
// per-group distance bounds dmin[e] <= d2(p, site e) for every target p of
// the group, and two compacted candidate lists of (x, y, index, entry):
// near[] the sites that can be nearest or second nearest to a point of the
// group's box, far[] the other sites some lane may still need.
struct WarpStage {
    float x[kStage], y[kStage];
    int id[kStage];
    float dmin[kStage];
    float4 near[kStage], far[kStage];
    int segStart[11], segOff[11];
};

__device__ __forceinline__ float4 cand(const WarpStage &W, int e)
{
    return make_float4(W.x[e], W.y[e], __int_as_float(W.id[e]), __int_as_float(e));
}

// Appends the staged entries e < m with keep(e) to list[] (in entry order);
// returns the count. Warp-cooperative, two entries per lane.
__device__ __forceinline__ int warp_compact(const WarpStage &W, float4 *list, int m, bool keep0, bool keep1)
{
    int lane = threadIdx.x & 31;
    unsigned b0 = __ballot_sync(kFull, keep0 && lane < m);
    unsigned b1 = __ballot_sync(kFull, keep1 && lane + 32 < m);
    unsigned below = (1u << lane) - 1u;
    int n0 = __popc(b0);
    if (keep0 && lane < m) list[__popc(b0 & below)] = cand(W, lane);
    if (keep1 && lane + 32 < m) list[n0 + __popc(b1 & below)] = cand(W, lane + 32);
    return n0 + __popc(b1);
}

// Exact argmin of (d^2, d2, index) over a candidate list, c0 excluded: the
// rare case where two candidates' error bounds overlap.
struct ArgMin {
    float dsq, d, dd; // d^2, d, d2(p, site)
    int j, k;         // site index (-1: none), staged entry
};

__device__ __noinline__ ArgMin list_exact_argmin(const float4 *list, int n, float2 p, int i0, float c0x, float c0y,
                                                 ArgMin b)
{
    float ux = p.x - c0x, uy = p.y - c0y;
    for (int q = 0; q < n; ++q) {
        float4 c = list[q];
        int id = __float_as_int(c.z);
        if (id == i0) continue;
        float ex = c.x - c0x, ey = c.y - c0y;
        float l = sqrtf(ex * ex + ey * ey);
        if (l < 1e-12f) continue;
        float d = (ux * ex + uy * ey) / l - 0.5f * l;
        float dsq = d * d;
        float dx = c.x - p.x, dy = c.y - p.y;
        float dd = dx * dx + dy * dy;
        bool better = b.j < 0 ? dsq < FLT_MAX : (dsq < b.dsq || (dsq == b.dsq && key_less(dd, id, b.dd, b.j)));
        if (better) b = ArgMin{dsq, d, dd, id, __float_as_int(c.w)};
    }
    return b;
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

// Stages the 5x5 block around cell (cx, cy) into W (positions and indices);
// returns its site count m2 (> kStage: not staged).
__device__ __forceinline__ int stage_block(const VmFit &F, WarpStage &W, int cx, int cy)
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
    int m2 = __shfl_sync(kFull, incl, 10);
    if (m2 > kStage) return m2;
    if (lane < 11) {
        W.segStart[lane] = s0;
        W.segOff[lane] = incl - n;
    }
    __syncwarp();
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
        }
    }
    __syncwarp();
    return m2;
}

// The two smallest of a warp's values (two per lane), for every lane.
__device__ __forceinline__ void warp_min2(float a, float b, float &m1, float &m2)
{
    m1 = fminf(a, b);
    m2 = fmaxf(a, b);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        float o1 = __shfl_xor_sync(kFull, m1, off), o2 = __shfl_xor_sync(kFull, m2, off);
        float lo = fminf(m1, o1);
        m2 = fminf(fmaxf(m1, o1), fminf(m2, o2));
        m1 = lo;
    }
}

// Staged fast path, called by every lane of the warp (take = this lane's
// target is in the group; the group's box [bx0,bx1]x[by0,by1] holds every
// taking lane's target). Returns 1 used, 0 unused, -1 not certified.
//
// Bounds, exact in float: rounding is monotone, so for every p in the box
// dmin(s) <= d2(p, s) <= dmax(s) hold for the float values the reference
// computes. U2, the second smallest dmax, is >= every p's second nearest d2,
// so the sites with dmin <= U2 hold the nearest and second nearest of every
// lane (list near[]). For a site s, |d_s| >= (D_s - D0)/2 (D = distance), so
// a site beats the best estimate B only if D_s <= D0 + 2B: far[] keeps the
// other sites with dmin below the warp's largest such bound.
__device__ __forceinline__ int loss_staged(const VmFit &F, WarpStage &W, bool take, float2 p, int m2, float bx0,
                                           float bx1, float by0, float by1, int xlo, int xhi, int ylo, int yhi,
                                           TgtOut &o, float &bddOut, bool &rankSure)
{
    int lane = threadIdx.x & 31;
    float dm[2], dx2[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        int e = lane + 32 * r;
        dm[r] = FLT_MAX;
        dx2[r] = FLT_MAX;
        if (e < m2) {
            float sx = W.x[e], sy = W.y[e];
            float gx = fmaxf(fmaxf(bx0 - sx, sx - bx1), 0.0f), gy = fmaxf(fmaxf(by0 - sy, sy - by1), 0.0f);
            dm[r] = gx * gx + gy * gy;
            W.dmin[e] = dm[r];
            float fx = fmaxf(fabsf(sx - bx0), fabsf(sx - bx1)), fy = fmaxf(fabsf(sy - by0), fabsf(sy - by1));
            dx2[r] = fx * fx + fy * fy;
        }
    }
    float U1, U2;
    warp_min2(dx2[0], dx2[1], U1, U2);
    int n1 = warp_compact(W, W.near, m2, dm[0] <= U2, dm[1] <= U2);
    __syncwarp();
    // pass 1: nearest by (d2, index)
    float d0 = FLT_MAX;
    int i0 = -1;
    float c0x = 0.0f, c0y = 0.0f;
    for (int q = 0; q < n1; ++q) {
        float4 c = W.near[q];
        float dx = c.x - p.x, dy = c.y - p.y;
        float dd = dx * dx + dy * dy;
        int id = __float_as_int(c.z);
        if (key_less(dd, id, d0, i0)) {
            d0 = dd;
            i0 = id;
            c0x = c.x;
            c0y = c.y;
        }
    }
    float ux = p.x - c0x, uy = p.y - c0y;
    // pass 2a: rsqrt estimates of |d| with a rigorous 2^-19 relative bound
    float best = FLT_MAX, bestEps = 0.0f, lowOther = FLT_MAX;
    int kb = -1;
    bool special = false;
    auto consider = [&](float4 c) {
        int id = __float_as_int(c.z);
        float ex = c.x - c0x, ey = c.y - c0y;
        float ee = ex * ex + ey * ey;
        float dot = ux * ex + uy * ey;
        bool tiny = ee <= 1e-20f;
        special |= tiny && id != i0;
        float rs = rsqrtf(ee);
        float a = dot * rs, b = 0.5f * (ee * rs);
        float est = fabsf(a - b);
        float eps = 1.9073486328125e-06f * (fabsf(a) + b) + 1e-30f; // 2^-19
        if (id == i0 || tiny) est = FLT_MAX;
        if (est < best) {
            lowOther = fminf(lowOther, best - bestEps);
            best = est;
            bestEps = eps;
            kb = __float_as_int(c.w);
        } else {
            lowOther = fminf(lowOther, est - eps);
        }
    };
    for (int q = 0; q < n1; ++q) consider(W.near[q]);
    // 0.1% slack covers every float rounding in this chain of bounds; sqD0 is
    // within 4 ulp of sqrt(d0) (only bounds use it)
    float sqD0 = d0 > 0.0f ? d0 * rsqrtf(d0) : 0.0f;
    float T = best < FLT_MAX ? 1.001f * (sqD0 + 2.0f * (best + bestEps)) : FLT_MAX;
    T = T < FLT_MAX ? T * T + 1e-30f : FLT_MAX;
    if (!take) T = 0.0f;
    float Tmax = warp_max(T);
    float listedTo = fmaxf(U2, Tmax); // near and far hold every site with dmin <= listedTo
    int n2 = warp_compact(W, W.far, m2, dm[0] > U2 && dm[0] <= Tmax, dm[1] > U2 && dm[1] <= Tmax);
    __syncwarp();
    for (int q = 0; q < n2; ++q) consider(W.far[q]);
    bool listedOk = n1 + n2 <= F.K;
    if (!take) return 0;
    if (i0 < 0) return -1;
    // squares of |d| below 1e-18 may round to equal floats: settle exactly
    special |= best + bestEps < 1e-18f;
    // pass 2b: the exact reference value of the best; the exact argmin over
    // both lists only when another candidate's bound overlaps it
    float bdsq = FLT_MAX, bd = 0.0f, bdd = 0.0f;
    int bj = -1;
    if (special || lowOther <= best + bestEps) {
        ArgMin am{FLT_MAX, 0.0f, 0.0f, -1, -1};
        am = list_exact_argmin(W.near, n1, p, i0, c0x, c0y, am);
        am = list_exact_argmin(W.far, n2, p, i0, c0x, c0y, am);
        bdsq = am.dsq;
        bd = am.d;
        bdd = am.dd;
        bj = am.j;
        kb = am.k;
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
    bddOut = bdd;
    // every site nearer p than bj has dmin <= bdd; when bdd is within the
    // listed range, those sites are all listed, so bj ranks below n1 + n2
    rankSure = listedOk && bdd <= listedTo;
    return 1;
}

// Copies fit f's descriptor and its next step number into shared memory
// (block-wide; the block is synchronised on return).
__device__ __forceinline__ void load_fit(const VmFit *__restrict__ fits, int f, VmFit &sF, unsigned &sIter)
{
    const int *src = reinterpret_cast<const int *>(&fits[f]);
    int *dst = reinterpret_cast<int *>(&sF);
    for (int i = threadIdx.x; i < (int)(sizeof(VmFit) / 4); i += blockDim.x) dst[i] = __ldg(&src[i]);
    if (threadIdx.x == 0) {
        sIter = (unsigned)(fits[f].state->iter + 1);
        sFastOver = 0;
    }
    __syncthreads();
}

// A lane's running gradient sum for one site: consecutive targets of a lane
// mostly share their nearest site and bisector neighbour, so the sum reaches
// the fit's accumulators (section L of gradX) only when the site changes: one
// 64-bit reduction per component (integer sums modulo 2^64, so neither the
// grouping nor an intermediate wrap changes the result; the block bound
// below keeps the sums themselves in range).
struct RunSum {
    int site = -1;
    long long x = 0, y = 0;
};

__device__ __forceinline__ void run_flush(RunSum &r, unsigned long long *G)
{
    if (r.site >= 0) {
        if (r.x) atomicAdd(&G[2 * (size_t)r.site], (unsigned long long)r.x);
        if (r.y) atomicAdd(&G[2 * (size_t)r.site + 1], (unsigned long long)r.y);
    }
    r.site = -1;
    r.x = r.y = 0;
}

__device__ __forceinline__ void run_add(RunSum &r, int site, long long x, long long y, unsigned long long *G)
{
    if (site != r.site) {
        run_flush(r, G);
        r.site = site;
    }
    r.x += x;
    r.y += y;
}

// The loss kernel's fixed-point conversion of a gradient term. Its inline
// path takes terms that are an integer significand shifted by at most the
// fit's fastShift, so below 2^(fastShift + 24) <= 2^62 / T5: with every term
// there, no site sum can leave the int64 range. Every other term goes
// through the out-of-line conversion, which also raises the block's
// sFastOver when the term is that large or larger, so the check costs
// nothing on the common path.
__device__ __forceinline__ long long fx_term(float v, int e, int fastShift)
{
    unsigned u = __float_as_uint(v);
    int ex = (int)((u >> 23) & 0xFFu);
    int k = ex - 150 + e;
    if ((unsigned)(ex - 1) < 254u && (unsigned)k <= (unsigned)fastShift) {
        long long mag = (long long)((u & 0x7FFFFFu) | 0x800000u) << k;
        return (u >> 31) ? -mag : mag;
    }
    return fx_from_float_any(v, e, fastShift);
}

// A block that met a gradient term beyond the fit's fastShift flags the fit,
// once, for the exact recomputation.
__device__ __forceinline__ void flag_fit(const VmFit &F, int f, SlowQueue *queue)
{
    if (atomicExch(&F.state->needExact, 1) == 0) {
        int k = atomicAdd(&queue->nFlagged, 1);
        if (k < kMaxFlagged) queue->flagged[k] = f;
        else atomicOr(&F.state->errors, VM_KERR_CAPACITY);
    }
}

// One block takes a contiguous range of tiles (THREADS targets, or with WIN
// THREADS / 32 windows, each) of the fits' concatenated target order; within
// each fit's part of it, every warp walks
// its own contiguous run of windows, one per iteration. A window is 32
// targets in target order, or, with WIN (fits with a window list: small fits,
// whose pass is as long as its slowest warp), a cell-aligned run of at most
// 32. The lanes of an iteration are served in groups that share a grid cell
// (normally one group; always one with cell-aligned windows):
// the 5x5 cell block around the group's cell is staged once in shared memory
// (and kept while the warp stays in that cell), and distance bounds to the
// group's bounding box cut the candidates of both passes of loss_staged to
// the few sites some lane can need.
template <int THREADS, int MINB, bool WIN>
__global__ void __launch_bounds__(THREADS, MINB)
    k_loss(const VmFit *__restrict__ fits, const int *__restrict__ prefix, int nFits, int mode, SlowQueue *queue)
{
    constexpr int NW = THREADS / 32;
    constexpr int kGroups = 3; // cell groups per warp and iteration on the staged path
    __shared__ unsigned long long sLo[NW], sHi[NW];
    __shared__ int sCnt[NW], sSlow[NW];
    __shared__ WarpStage sStage[NW];
    __shared__ VmFit sF;
    __shared__ unsigned sIter;
    int totalTiles = prefix[nFits];
    long long t0 = (long long)blockIdx.x * totalTiles / gridDim.x;
    long long t1 = (long long)(blockIdx.x + 1) * totalTiles / gridDim.x;
    if (t0 >= t1) return;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    WarpStage &W = sStage[warp];
    const VmFit &F = sF;
    int f = find_fit(prefix, nFits, (int)t0);
    int stCell = -1, stFit = -1, stM2 = 0; // this warp's staged block
    for (long long t = t0; t < t1;) {
        while (t >= prefix[f + 1]) ++f;
        load_fit(fits, f, sF, sIter);
        long long segEnd = min(t1, (long long)prefix[f + 1]);
        bool active = F.active || mode == 1;
        // this fit's part of the block's range, then this warp's run of it:
        // targets (32 an iteration), or with WIN windows (one an iteration; a
        // tile is NW windows)
        int w0, w1;
        if constexpr (WIN) {
            int A = (int)(t - prefix[f]) * NW;
            int B = min((int)(segEnd - prefix[f]) * NW, F.nWindows);
            int per = B > A ? (B - A + NW - 1) / NW : 0;
            w0 = A + warp * per;
            w1 = min(w0 + per, B);
        } else {
            int A = (int)(t - prefix[f]) * THREADS;
            int B = min((int)(segEnd - prefix[f]) * THREADS, F.nTargets);
            int per = B > A ? (B - A + NW * 32 - 1) / (NW * 32) * 32 : 0;
            w0 = A + warp * per;
            w1 = min(w0 + per, B);
        }
        if (!active) w1 = w0;
        unsigned long long aLo = 0, aHi = 0;
        int aCnt = 0, aSlow = 0;
        unsigned long long *G = reinterpret_cast<unsigned long long *>(F.gradX);
        RunSum run0, runJ;
        for (int it = w0; it < w1; it += WIN ? 1 : 32) {
            int base = WIN ? F.twin[it] : it;
            int end = WIN ? F.twin[it + 1] : w1;
            int local = base + lane;
            bool valid = local < end;
            float2 p = make_float2(0.0f, 0.0f);
            bool take = false;
            int cx = 0, cy = 0;
            if (valid) {
                p = F.tpos[local];
                take = true;
                if (mode == 0) {
                    take = p.x >= F.bx0 && p.x <= F.bx1 && p.y >= F.by0 && p.y <= F.by1;
                    if (take && F.fraction < 1.0f)
                        take = rand01((unsigned)F.tslot[local], sIter, F.seed) < F.fraction;
                }
                cx = cell_coord(p.x, F.inv, F.gridW);
                cy = cell_coord(p.y, F.inv, F.gridH);
            }
            TgtOut o;
            int r = -1;
            bool pending = take; // still to be served by the staged path
            for (int g = 0; g < kGroups; ++g) {
                __syncwarp(); // every lane is done with the previous group's staging
                unsigned rem = __ballot_sync(kFull, pending);
                if (!rem) break;
                int leader = __ffs(rem) - 1;
                int lcx = __shfl_sync(kFull, cx, leader), lcy = __shfl_sync(kFull, cy, leader);
                bool mine = pending && cx == lcx && cy == lcy;
                int lcell = lcy * F.gridW + lcx;
                if (lcell != stCell || f != stFit) {
                    stM2 = stage_block(F, W, lcx, lcy);
                    stCell = lcell;
                    stFit = f;
                }
                int m2 = stM2;
                if (m2 > kStage) break; // the remaining lanes take the per-lane search
                float bx0 = warp_min(mine ? p.x : FLT_MAX), bx1 = warp_max(mine ? p.x : -FLT_MAX);
                float by0 = warp_min(mine ? p.y : FLT_MAX), by1 = warp_max(mine ? p.y : -FLT_MAX);
                int xlo = max(lcx - 2, 0), xhi = min(lcx + 2, F.gridW - 1);
                int ylo = max(lcy - 2, 0), yhi = min(lcy + 2, F.gridH - 1);
                // writes o only for this group's lanes
                float bdd = 0.0f;
                bool rankSure = false;
                int rg = loss_staged(F, W, mine, p, m2, bx0, bx1, by0, by1, xlo, xhi, ylo, yhi, o, bdd, rankSure);
                if (m2 > F.K && __any_sync(kFull, mine && rg > 0 && !rankSure)) {
                    // bj must rank below K among all sites; every closer site is staged
                    // (certified), and a site s is closer only if dmin(s) <= d2(p, bj).
                    // One warp vote settles it unless K staged sites are that near.
                    float lim = warp_max((mine && rg > 0) ? bdd : 0.0f);
                    int cnt = __popc(__ballot_sync(kFull, lane < m2 && W.dmin[lane] <= lim)) +
                              __popc(__ballot_sync(kFull, lane + 32 < m2 && W.dmin[lane + 32] <= lim));
                    if (cnt >= F.K && mine && rg > 0 && staged_rank(W, m2, p, bdd, o.j) >= F.K) rg = -1;
                }
                if (mine) {
                    r = rg;
                    pending = false;
                }
            }
            int used = 0;
            bool deferred = false;
            if (take) {
                if (pending) {
                    TgtOut ob; // its address goes to the out-of-line search; o stays in registers
                    r = loss_block(F, p, 1, F.K, ob);
                    if (r < 0) r = loss_block(F, p, 2, F.K, ob);
                    if (r > 0) o = ob;
                }
                if (r < 0) {
                    int q = atomicAdd(&queue->count, 1);
                    if (q < queue->capacity) queue->items[q] = make_int2(f, local); // capacity >= live targets
                    else atomicOr(&F.state->errors, VM_KERR_CAPACITY);
                    r = 0;
                    deferred = true;
                    aSlow += 1;
                }
                used = r;
            }
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
                if (mode == 0) {
                    int e = F.gradExp, fs = F.fastShift;
                    run_add(run0, o.i0, fx_term(o.g0x, e, fs), fx_term(o.g0y, e, fs), G);
                    run_add(runJ, o.j, fx_term(o.gjx, e, fs), fx_term(o.gjy, e, fs), G);
                }
            }
        }
        run_flush(run0, G);
        run_flush(runJ, G);
        // the loss, count and fallbacks of this fit: warp, block, then one atomic each
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
        if (threadIdx.x == 0 && active) {
            unsigned long long lo = 0, hi = 0;
            int cnt = 0, slow = 0;
            for (int w = 0; w < NW; ++w) {
                add128(lo, hi, sLo[w], sHi[w]);
                cnt += sCnt[w];
                slow += sSlow[w];
            }
            if (mode == 0 && sFastOver) flag_fit(F, f, queue);
            VmState *st = F.state;
            atomic_add128(&st->accLo, &st->accHi, lo, hi);
            if (cnt) atomicAdd(&st->accCount, cnt);
            if (slow) atomicAdd(&st->slowTotal, slow);
        }
        __syncthreads(); // sF is replaced next
        t = segEnd;
    }
}

// The deferred targets: exact ring search, one target per thread, with the
// loss and count added straight into the fit's accumulators and the gradient
// into its exact split words. In a step pass it also writes each fit's Adam
// schedule for the step, and recomputes the whole gradient of every fit whose
// fast-path bound failed (its deferred targets are then part of that).
// The body of k_loss_exact for thread `tid` of `stride` threads.
__device__ __forceinline__ void exact_pass(const VmFit *__restrict__ fits, int nFits, int mode, SlowQueue *queue,
                                           int tid, int stride)
{
    if (mode == 0)
        for (int f = tid; f < nFits; f += stride)
            if (fits[f].active) adam_schedule(fits[f]); // for the Adam kernel that follows
    int n = min(queue->count, queue->capacity);
    for (int q = tid; q < n; q += stride) {
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
        if (mode == 0 && !F.state->needExact) {
            int e = F.gradExp;
            unsigned long long *g = reinterpret_cast<unsigned long long *>(F.gradX);
            fxd_red(g, F.nSlots, o.j, fx_from_float(o.gjx, e), fx_from_float(o.gjy, e), &F.state->dUsed);
            fxd_red(g, F.nSlots, o.i0, fx_from_float(o.g0x, e), fx_from_float(o.g0y, e), &F.state->dUsed);
        }
    }
    if (mode != 0) return;
    int nf = min(queue->nFlagged, kMaxFlagged);
    for (int k = 0; k < nf; ++k) {
        const VmFit &F = fits[queue->flagged[k]];
        unsigned iter = (unsigned)(F.state->iter + 1);
        unsigned long long *g = reinterpret_cast<unsigned long long *>(F.gradX);
        int e = F.gradExp;
        for (int t = tid; t < F.nTargets; t += stride) {
            float2 p = F.tpos[t];
            bool take = p.x >= F.bx0 && p.x <= F.bx1 && p.y >= F.by0 && p.y <= F.by1;
            if (take && F.fraction < 1.0f) take = rand01((unsigned)F.tslot[t], iter, F.seed) < F.fraction;
            TgtOut o;
            if (!take || !loss_exact(F, p, o)) continue;
            fxd_red(g, F.nSlots, o.j, fx_from_float(o.gjx, e), fx_from_float(o.gjy, e), &F.state->dUsed);
            fxd_red(g, F.nSlots, o.i0, fx_from_float(o.g0x, e), fx_from_float(o.g0y, e), &F.state->dUsed);
        }
    }
}

__global__ void __launch_bounds__(128) k_loss_exact(const VmFit *__restrict__ fits, int nFits, int mode,
                                                    SlowQueue *queue)
{
    exact_pass(fits, nFits, mode, queue, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// The exact pass of one fit by one block (out of line: it is the rare path,
// and its registers stay out of the caller's).
static __device__ __noinline__ void exact_pass_block(const VmFit *__restrict__ fits, SlowQueue *queue)
{
    exact_pass(fits, 1, 0, queue, threadIdx.x, blockDim.x);
}

// A fit this small finishes its step in one block (k_small_grid).
constexpr int kSmallThreads = 1024;
constexpr int kSmallSlots = 4 * kSmallThreads;
constexpr int kSmallCells = 8 * kSmallThreads;

// The rest of a small fit's step in one block (k_loss_exact, k_adam_bin,
// k_scan_tiles, k_scan_apply and k_scatter for one fit of at most kSmallSlots
// slots and kSmallCells grid cells): the deferred targets and the Adam
// schedule, then Adam with the binning into shared-memory counts, their
// exclusive scan in place, the cell starts, the scatter and the publish. Ranks within a cell come from the shared atomics, in another order
// than the four-kernel path; nothing in the step depends on that order.
__global__ void __launch_bounds__(kSmallThreads) k_small_grid(const VmFit *__restrict__ fits, SlowQueue *queue)
{
    __shared__ int sStart[kSmallCells + 1];
    __shared__ int sWarp[kSmallThreads / 32];
    __shared__ int sTotal;
    constexpr int kPer = kSmallSlots / kSmallThreads;
    const VmFit &F = fits[0];
    int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int n = F.nSlots, cells = F.gridW * F.gridH;
    // the deferred targets and the schedule; their writes are visible to the
    // whole block after the barrier
    exact_pass_block(fits, queue);
    for (int c = tid; c <= cells; c += kSmallThreads) sStart[c] = 0;
    __syncthreads();
    if (tid == 0) {
        queue->count = 0;
        queue->nFlagged = 0;
    }
    // Adam and the binning
    int key[kPer], rank[kPer];
    float2 pos[kPer];
    if (F.active) {
        AdamStep a = adam_step(F);
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            int i = tid + k * kSmallThreads;
            key[k] = -1;
            if (i < n) {
                pos[k] = adam_slot(F, a, i);
                if (pos[k].x >= 0.0f) {
                    key[k] = cell_coord(pos[k].y, F.inv, F.gridH) * F.gridW + cell_coord(pos[k].x, F.inv, F.gridW);
                    rank[k] = atomicAdd(&sStart[key[k]], 1);
                }
            }
        }
    } else {
        // a fit left out of the step keeps its positions: re-bin them
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            int i = tid + k * kSmallThreads;
            key[k] = -1;
            if (i < n) {
                pos[k] = F.gen[i];
                if (pos[k].x >= 0.0f) {
                    key[k] = cell_coord(pos[k].y, F.inv, F.gridH) * F.gridW + cell_coord(pos[k].x, F.inv, F.gridW);
                    rank[k] = atomicAdd(&sStart[key[k]], 1);
                }
            }
        }
    }
    __syncthreads();
    // exclusive scan of the counts in place (8 cells a thread), total at [cells]
    int v[8], base = tid * 8, run = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        int x = base + k < cells ? sStart[base + k] : 0;
        v[k] = run;
        run += x;
    }
    int incl = run;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        int t = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl += t;
    }
    if (lane == 31) sWarp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = sWarp[lane], wi = w;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            int t = __shfl_up_sync(kFull, wi, off);
            if (lane >= off) wi += t;
        }
        sWarp[lane] = wi - w;
        if (lane == 31) sTotal = wi;
    }
    __syncthreads();
    int excl = incl - run + sWarp[warp];
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (base + k < cells) sStart[base + k] = excl + v[k];
    if (tid == 0) sStart[cells] = sTotal;
    __syncthreads();
    for (int c = tid; c <= cells; c += kSmallThreads) F.start[c] = sStart[c];
    // the slots' cell keys (exported with the grid) and the cell-sorted copy
#pragma unroll
    for (int k = 0; k < kPer; ++k)
        if (tid + k * kSmallThreads < n) F.key[tid + k * kSmallThreads] = key[k];
#pragma unroll
    for (int k = 0; k < kPer; ++k)
        if (key[k] >= 0) {
            int at = sStart[key[k]] + rank[k];
            F.sortedIdx[at] = tid + k * kSmallThreads;
            F.sortedPos[at] = pos[k];
        }
    if (tid == 0 && F.active) {
        // end of a step: publish the loss pass and advance the step counter
        VmState *st = F.state;
        st->loss = fxl_to_float(st->accLo, st->accHi, F.lossExp);
        st->count = st->accCount;
        st->iter += 1;
        st->accLo = 0;
        st->accHi = 0;
        st->accCount = 0;
        st->needExact = 0;
        st->dUsed = 0;
    }
}


} // namespace vmk

// ---------------------------------------------------------------------------
// launch wrappers (host)
// ---------------------------------------------------------------------------
using namespace vmk;

extern "C++" {

// Loss kernel variants (block size, min blocks per SM); all give the
// identical result.
struct LossVariant {
    int threads, minBlocks;
};
static const LossVariant kVariants[] = {{256, 4}, {256, 3}, {256, 2}, {128, 5},
                                        {128, 6}, {64, 16}, {64, 12}, {64, 10}};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

int vm_loss_variants() { return kNumVariants; }
int vm_loss_variant_threads(int v) { return kVariants[v < 0 || v >= kNumVariants ? 0 : v].threads; }

template <int T, int B> static void *loss_fn(bool win)
{
    return win ? (void *)k_loss<T, B, true> : (void *)k_loss<T, B, false>;
}

static void *variant_fn(int v, bool win)
{
    switch (v) {
    case 0: return loss_fn<256, 4>(win);
    case 1: return loss_fn<256, 3>(win);
    case 2: return loss_fn<256, 2>(win);
    case 3: return loss_fn<128, 5>(win);
    case 4: return loss_fn<128, 6>(win);
    case 5: return loss_fn<64, 16>(win);
    case 6: return loss_fn<64, 12>(win);
    default: return loss_fn<64, 10>(win);
    }
}

cudaError_t vm_launch_loss(const VmFit *fits, const int *tilePrefix, int nFits, int totalTiles, int mode,
                           int gridBlocks, int variant, int windowed, void *queue, cudaStream_t s)
{
    SlowQueue *q = static_cast<SlowQueue *>(queue);
    if (totalTiles > 0) {
        int g = gridBlocks < totalTiles ? gridBlocks : totalTiles;
        if (g < 1) g = 1;
        void *args[] = {(void *)&fits, (void *)&tilePrefix, (void *)&nFits, (void *)&mode, (void *)&q};
        cudaError_t e = cudaLaunchKernel(variant_fn(variant, windowed != 0), dim3(g),
                                         dim3(vm_loss_variant_threads(variant)), args, 0, s);
        if (e) return e;
    }
    // with no targets the step still needs its Adam schedule (k_loss_exact)
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    k_loss_exact<<<sms * 2, 128, 0, s>>>(fits, nFits, mode, q);
    return cudaGetLastError();
}

bool vm_small_grid_fits(int slots, int cells) { return slots <= kSmallSlots && cells <= kSmallCells; }

cudaError_t vm_launch_small_grid(const VmFit *fit, void *queue, cudaStream_t s)
{
    k_small_grid<<<1, kSmallThreads, 0, s>>>(fit, static_cast<SlowQueue *>(queue));
    return cudaGetLastError();
}

cudaError_t vm_launch_loss_fast(const VmFit *fits, const int *tilePrefix, int nFits, int totalTiles, int gridBlocks,
                                int variant, int windowed, void *queue, cudaStream_t s)
{
    if (totalTiles <= 0) return cudaSuccess;
    SlowQueue *q = static_cast<SlowQueue *>(queue);
    int mode = 0;
    int g = gridBlocks < totalTiles ? gridBlocks : totalTiles;
    if (g < 1) g = 1;
    void *args[] = {(void *)&fits, (void *)&tilePrefix, (void *)&nFits, (void *)&mode, (void *)&q};
    return cudaLaunchKernel(variant_fn(variant, windowed != 0), dim3(g), dim3(vm_loss_variant_threads(variant)), args, 0,
                            s);
}

int vm_loss_occupancy_blocks(int variant)
{
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, variant_fn(variant, false), vm_loss_variant_threads(variant), 0);
    if (per < 1) per = 1;
    return sms * per;
}

} // extern "C++"
