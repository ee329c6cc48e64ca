// Voronoi cell clipping for mesh extraction (reference voronoiCellKernel,
// voro_optimizer.cu:312-437).
//
// Per generator: the 32 nearest sites by ring search, then the domain box is
// clipped (Sutherland-Hodgman, the reference's vertex/edge-label bookkeeping)
// by the bisectors of those neighbours in kNN order until the security radius
// certifies the cell (|cj - ci|^2 > 4 max|v - ci|^2); an uncertified cell
// falls back to every generator in index order, as in the reference.
//
// Arithmetic: a new vertex is the reference's FP64 interpolation along the
// clipped edge, t = fa / (fa - fb) with fa, fb the edge ends' signed
// bisector values, each operation one IEEE rounding (built without FMA
// contraction), so every vertex is the reference's bit for bit. Vertices are
// kept in FP64 (and rounded to FP32). The inside/outside test of a vertex
// against a new bisector runs in FP32 with a rigorous error bound and is
// re-evaluated in FP64 only when the FP32 value lies inside that bound, which
// gives the FP64 test's decision. Centroid and output vertices use the FP64
// vertices, as the reference does.
#include "vm_device.cuh"
#include "vm_kernels.h"
#include "vm_knn.cuh"

namespace vmk {

constexpr int kMaxVerts = 24;
constexpr int kCellK = 32;

// A vertex's coordinates are stored as pairs, so that each is read and
// written as one vector access of the thread's local memory.
struct CellPoly {
    double2 v[kMaxVerts]; // FP64 vertex, relative to the site
    float2 f[kMaxVerts];  // the same rounded to FP32
    int lab[kMaxVerts];
    int n;
};

struct CellCtx {
    double cx, cy; // the cell's site, converted once
    float fx, fy;  // and as given
    double w, h;   // domain size
};

// a - b is exact in float (Sterbenz: same sign and within a factor of 2, or
// an operand zero), so it equals the exact difference rounded once, which is
// also the FP64 difference rounded to float.
__device__ __forceinline__ bool sub_exact(float a, float b)
{
    return a == 0.0f || b == 0.0f || (b > 0.0f ? (a >= 0.5f * b && a <= 2.0f * b) : (a <= 0.5f * b && a >= 2.0f * b));
}

// Clip P by the bisector of ci and site j (reference clipByBisector :320-351).
// Writes into Q; returns false on vertex overflow. *changed = 0 if no vertex was outside.
// When it cuts, r2 = r2max_f(Q), taken as the vertices are written.
//
// A vertex is outside the half-plane <x, r> <= |r|^2/2 (:322-325) when the
// FP32 value of <x, r> - |r|^2/2 exceeds its error bound, inside when it is
// below minus the bound; in between, the FP64 value decides. The FP64 offset
// and half-norm are formed only when a vertex needs them or the polygon is
// cut (the FP32 offset comes from the FP32 difference when that is exact).
__device__ bool clip(const CellCtx &c, const CellPoly &P, CellPoly &Q, int j, float2 cj, bool &changed, float &r2)
{
    double rx = 0.0, ry = 0.0, cc = 0.0;
    bool have64 = false;
    auto need64 = [&]() {
        if (!have64) {
            rx = (double)cj.x - c.cx;
            ry = (double)cj.y - c.cy;
            cc = 0.5 * (rx * rx + ry * ry);
            have64 = true;
        }
    };
    float rfx, rfy;
    if (sub_exact(cj.x, c.fx) && sub_exact(cj.y, c.fy)) {
        rfx = cj.x - c.fx;
        rfy = cj.y - c.fy;
    } else {
        need64();
        rfx = (float)rx;
        rfy = (float)ry;
    }
    float cf = 0.5f * (rfx * rfx + rfy * rfy);
    unsigned out = 0, band = 0;
    for (int k = 0; k < P.n; ++k) {
        const float2 q = P.f[k];
        float a = q.x * rfx, b = q.y * rfy;
        float f = a + b - cf;
        float bound = 1.9073486328125e-06f * (fabsf(a) + fabsf(b) + cf + fabsf(f)) + 1e-37f; // 2^-19
        if (f > bound) out |= 1u << k;
        else if (!(f < -bound)) band |= 1u << k;
    }
    if (band) {
        need64();
        for (unsigned m = band; m; m &= m - 1) {
            int k = __ffs(m) - 1;
            const double2 v = P.v[k];
            if (v.x * rx + v.y * ry - cc > 0.0) out |= 1u << k;
        }
    }
    if (!out) {
        changed = false;
        return true;
    }
    need64();
    changed = true;
    bool ok = true;
    Q.n = 0;
    float r = 0.0f;
    for (int k = 0; k < P.n; ++k) {
        int k1 = k + 1 == P.n ? 0 : k + 1;
        bool inA = !((out >> k) & 1u), inB = !((out >> k1) & 1u);
        if (inA) {
            if (Q.n < kMaxVerts) {
                const float2 q = P.f[k];
                Q.v[Q.n] = P.v[k];
                Q.f[Q.n] = q;
                Q.lab[Q.n] = P.lab[k];
                ++Q.n;
                r = fmaxf(r, q.x * q.x + q.y * q.y);
            } else ok = false;
        }
        if (inA != inB) {
            // the reference's interpolation (:337-343); fa and fb differ in sign
            const double2 va = P.v[k], vb = P.v[k1];
            const double ax = va.x, ay = va.y, bx = vb.x, by = vb.y;
            const double fa = ax * rx + ay * ry - cc, fb = bx * rx + by * ry - cc;
            const double t = fa / (fa - fb);
            const double x = ax + t * (bx - ax), y = ay + t * (by - ay);
            if (Q.n < kMaxVerts) {
                const float fx = (float)x, fy = (float)y;
                Q.v[Q.n] = make_double2(x, y);
                Q.f[Q.n] = make_float2(fx, fy);
                Q.lab[Q.n] = inA ? j : P.lab[k];
                ++Q.n;
                r = fmaxf(r, fx * fx + fy * fy);
            } else ok = false;
        }
    }
    r2 = r;
    return ok;
}

__device__ __forceinline__ float r2max_f(const CellPoly &P)
{
    float r = 0.0f;
    for (int k = 0; k < P.n; ++k) {
        const float2 q = P.f[k];
        r = fmaxf(r, q.x * q.x + q.y * q.y);
    }
    return r;
}

__device__ __forceinline__ double r2max_d(const CellPoly &P)
{
    double r = 0.0;
    for (int k = 0; k < P.n; ++k) {
        const double2 v = P.v[k];
        r = fmax(r, v.x * v.x + v.y * v.y);
    }
    return r;
}

// (double)dd > 4 * maxRadius2(P), decided in FP32 unless within its error band.
// r4 = 4 * r2max_f(P), kept by the caller while P is unchanged.
__device__ __forceinline__ bool beyond(float dd, const CellPoly &P, float r4)
{
    const float r = r4;
    if (dd > r * 1.0000038146972656f) return true;  // 1 + 2^-18
    if (dd < r * 0.9999961853027344f) return false; // 1 - 2^-18
    return (double)dd > 4.0 * r2max_d(P);
}

__device__ __forceinline__ bool occupied(const unsigned long long *masks, int tilesX, int tilesY, float invVoxel,
                                         float2 p)
{
    if (!masks) return false;
    float fx = floorf(p.x * invVoxel), fy = floorf(p.y * invVoxel);
    if (!(fx >= 0.0f) || !(fy >= 0.0f) || fx >= 2147483647.0f || fy >= 2147483647.0f) return false;
    int i = (int)fx, j = (int)fy;
    int tx = i >> 3, ty = j >> 3;
    if (tx >= tilesX || ty >= tilesY) return false;
    return (masks[(size_t)ty * tilesX + tx] >> (((j & 7) << 3) | (i & 7))) & 1ull;
}

__global__ void __launch_bounds__(128, 7) k_cells(const VmFit *__restrict__ fit, const unsigned long long *masks,
                                               int tilesX, int tilesY, float invVoxel, float2 *__restrict__ outVerts,
                                               int *__restrict__ outEdges, int *__restrict__ outCount,
                                               unsigned char *__restrict__ outInside, int *__restrict__ flags)
{
    const VmFit &F = *fit;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= F.nSlots) return;
    float2 ci = F.gen[i];
    if (ci.x < 0.0f) {
        outCount[i] = 0;
        outInside[i] = 0;
        return;
    }
    // the ring search keeps its top 32 in registers (every index a constant
    // of the unrolled insertion); the clip loops below index the list at run
    // time, which puts d2/idx in local memory, so they get one copy of it
    float d2[kCellK];
    int idx[kCellK];
    {
        float rd2[kCellK];
        int ridx[kCellK];
        knn_ring<kCellK>(F.start, F.sortedPos, F.sortedIdx, F.gridW, F.gridH, F.cell, F.inv, ci, rd2, ridx);
#pragma unroll
        for (int k = 0; k < kCellK; ++k) {
            d2[k] = rd2[k];
            idx[k] = ridx[k];
        }
    }

    CellCtx c;
    c.cx = (double)ci.x;
    c.cy = (double)ci.y;
    c.fx = ci.x;
    c.fy = ci.y;
    c.w = (double)F.width;
    c.h = (double)F.height;
    CellPoly buf[2];
    CellPoly *P = &buf[0], *Q = &buf[1];
    double x0 = -c.cx, y0 = -c.cy, x1 = c.w - c.cx, y1 = c.h - c.cy;
    P->v[0] = make_double2(x0, y0); P->lab[0] = -1;
    P->v[1] = make_double2(x1, y0); P->lab[1] = -2;
    P->v[2] = make_double2(x1, y1); P->lab[2] = -3;
    P->v[3] = make_double2(x0, y1); P->lab[3] = -4;
    for (int k = 0; k < 4; ++k) {
        P->f[k] = make_float2((float)P->v[k].x, (float)P->v[k].y);
    }
    P->n = 4;

    bool ok = true, certified = false;
    float r4 = 4.0f * r2max_f(*P); // refreshed after each cut
    for (int k = 0; k < kCellK; ++k) {
        int j = idx[k];
        if (j < 0) {
            certified = true; // every generator has been seen
            break;
        }
        if (j == i) continue;
        if (beyond(d2[k], *P, r4)) {
            certified = true;
            break;
        }
        bool changed;
        float r2;
        ok &= clip(c, *P, *Q, j, F.gen[j], changed, r2);
        if (changed) {
            CellPoly *t = P; P = Q; Q = t;
            r4 = 4.0f * r2;
        }
    }
    if (!certified && beyond(d2[kCellK - 1], *P, r4)) certified = true;
    if (!certified) {
        atomicAdd(&flags[0], 1);
        // The reference clips by every other generator in index order, skipping
        // those beyond the current security radius (:402-414). Only sites within
        // the radius at this point can cut the cell (r2max only shrinks), so they
        // are gathered from the hash grid, sorted by index and clipped in that
        // order -- the same sequence of cuts. Too many candidates: the full loop.
        constexpr int kGather = 256;
        int cand[kGather];
        int nc = 0;
        bool gathered = true;
        double R2 = 4.0 * r2max_d(*P);
        float R = (float)sqrt(R2) * 1.0001f + 1e-30f;
        int gx0 = cell_coord(ci.x - R, F.inv, F.gridW), gx1 = cell_coord(ci.x + R, F.inv, F.gridW);
        int gy0 = cell_coord(ci.y - R, F.inv, F.gridH), gy1 = cell_coord(ci.y + R, F.inv, F.gridH);
        if ((long long)(gx1 - gx0 + 1) * (gy1 - gy0 + 1) > 4096) gathered = false;
        for (int gy = gy0; gathered && gy <= gy1; ++gy) {
            int s0 = F.start[gy * F.gridW + gx0], s1 = F.start[gy * F.gridW + gx1 + 1];
            for (int s = s0; s < s1; ++s) {
                int j = F.sortedIdx[s];
                if (j == i) continue;
                bool seen = false;
                for (int k = 0; k < kCellK; ++k) seen |= idx[k] == j;
                if (seen) continue;
                float2 g = F.sortedPos[s];
                double rx = (double)g.x - c.cx, ry = (double)g.y - c.cy;
                if (rx * rx + ry * ry > R2) continue;
                if (nc == kGather) {
                    gathered = false;
                    break;
                }
                int k = nc++;
                while (k > 0 && cand[k - 1] > j) {
                    cand[k] = cand[k - 1];
                    --k;
                }
                cand[k] = j;
            }
        }
        if (gathered) {
            for (int q = 0; q < nc; ++q) {
                int j = cand[q];
                float2 g = F.gen[j];
                double rx = (double)g.x - c.cx, ry = (double)g.y - c.cy;
                if (rx * rx + ry * ry > 4.0 * r2max_d(*P)) continue;
                bool changed;
                float r2;
                ok &= clip(c, *P, *Q, j, g, changed, r2);
                if (changed) {
                    CellPoly *t = P; P = Q; Q = t;
                }
            }
        }
        for (int j = 0; !gathered && j < F.nSlots; ++j) {
            if (j == i) continue;
            float2 g = F.gen[j];
            if (g.x < 0.0f) continue;
            bool seen = false;
            for (int k = 0; k < kCellK; ++k) seen |= idx[k] == j;
            if (seen) continue;
            double rx = (double)g.x - c.cx, ry = (double)g.y - c.cy;
            if (rx * rx + ry * ry > 4.0 * r2max_d(*P)) continue;
            bool changed;
            float r2;
            ok &= clip(c, *P, *Q, j, g, changed, r2);
            if (changed) {
                CellPoly *t = P; P = Q; Q = t;
            }
        }
    }
    if (!ok) atomicAdd(&flags[1], 1);

    // centroid (shoelace) -> occupancy (reference :417-431); with no
    // occupancy every cell is outside and the centroid is not needed
    bool in = false;
    if (masks) {
        double area = 0.0, cx = 0.0, cy = 0.0;
        for (int k = 0; k < P->n; ++k) {
            int k1 = k + 1 == P->n ? 0 : k + 1;
            const double2 va = P->v[k], vb = P->v[k1];
            double ax = va.x, ay = va.y, bx = vb.x, by = vb.y;
            double cr = ax * by - bx * ay;
            area += cr;
            cx += (ax + bx) * cr;
            cy += (ay + by) * cr;
        }
        float2 centroid = ci;
        if (fabs(area) > 1e-12) {
            centroid.x += (float)(cx / (3.0 * area));
            centroid.y += (float)(cy / (3.0 * area));
        }
        in = occupied(masks, tilesX, tilesY, invVoxel, centroid);
    }
    outInside[i] = in ? 1 : 0;
    outCount[i] = P->n;
    for (int k = 0; k < P->n; ++k) {
        outVerts[(size_t)i * kMaxVerts + k] = make_float2((float)(c.cx + P->v[k].x), (float)(c.cy + P->v[k].y));
        outEdges[(size_t)i * kMaxVerts + k] = P->lab[k];
    }
}

// Cell i's vertices and edge labels from its fixed-size slot to the packed
// CSR position start[i] (start = exclusive scan of the counts).
__global__ void __launch_bounds__(256) k_compact_cells(const float2 *__restrict__ verts, const int *__restrict__ labels,
                                                       const int *__restrict__ start, int n, float2 *__restrict__ outV,
                                                       int *__restrict__ outL)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int b = start[i], c = start[i + 1] - b;
    for (int k = 0; k < c; ++k) {
        outV[b + k] = verts[(size_t)i * kMaxVerts + k];
        outL[b + k] = labels[(size_t)i * kMaxVerts + k];
    }
}

// ---------------------------------------------------------------------------
// Boundary assembly (reference voro_optimizer.cu:798-854) on the device.
// Boundary edges are emitted in the reference's loop order (cell, then edge
// within the cell); occurrence 2e / 2e+1 is edge e's first / second vertex.
// A vertex is the sorted generator triple of its cell corner (labels + 4,
// 21 bits each); vertices are numbered by first occurrence, as the
// reference's insertion-ordered map numbers them.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long triple_key(int a, int b, int c)
{
    unsigned long long v0 = (unsigned long long)(a + 4), v1 = (unsigned long long)(b + 4),
                       v2 = (unsigned long long)(c + 4);
    unsigned long long t;
    if (v0 > v1) { t = v0; v0 = v1; v1 = t; }
    if (v1 > v2) { t = v1; v1 = v2; v2 = t; }
    if (v0 > v1) { t = v0; v0 = v1; v1 = t; }
    return (v0 << 42) | (v1 << 21) | v2;
}

__device__ __forceinline__ bool boundary_edge(int l, const unsigned char *inside) { return !(l >= 0 && inside[l]); }

__global__ void k_bnd_count(int n, const int *__restrict__ start, const int *__restrict__ labels,
                            const unsigned char *__restrict__ inside, int *__restrict__ cnt)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int m = 0;
    if (inside[i])
        for (int k = start[i]; k < start[i + 1]; ++k) m += boundary_edge(labels[k], inside);
    cnt[i] = m;
}

// Open-addressing insert of a vertex key; returns its slot. The table is at
// least twice the number of occurrences, so a free slot is always reached.
__device__ __forceinline__ unsigned bnd_insert(unsigned long long *keys, unsigned mask, unsigned long long key)
{
    unsigned long long h = key;
    h ^= h >> 33; h *= 0xff51afd7ed558ccdULL; h ^= h >> 33; h *= 0xc4ceb9fe1a85ec53ULL; h ^= h >> 33;
    unsigned s = (unsigned)h & mask;
    for (unsigned probe = 0; probe <= mask; ++probe) {
        unsigned long long old = atomicCAS(&keys[s], ~0ull, key);
        if (old == ~0ull || old == key) return s;
        s = (s + 1) & mask;
    }
    return 0xffffffffu; // unreachable at half load
}

__global__ void k_bnd_emit(int n, const int *__restrict__ start, const int *__restrict__ labels,
                           const float2 *__restrict__ verts, const unsigned char *__restrict__ inside,
                           const int *__restrict__ eStart, unsigned long long *__restrict__ keys, unsigned mask,
                           int *__restrict__ minPos, unsigned *__restrict__ occSlot, float2 *__restrict__ occPt,
                           int *__restrict__ err)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !inside[i]) return;
    const int b = start[i], c = start[i + 1] - b;
    int e = eStart[i];
    for (int k = 0; k < c; ++k) {
        const int l = labels[b + k];
        if (!boundary_edge(l, inside)) continue;
        const int prev = labels[b + (k + c - 1) % c], next = labels[b + (k + 1) % c];
        const unsigned long long ka = triple_key(i, prev, l), kb = triple_key(i, l, next);
        const unsigned sa = bnd_insert(keys, mask, ka), sb = bnd_insert(keys, mask, kb);
        if (sa == 0xffffffffu || sb == 0xffffffffu) {
            atomicOr(err, 1);
            return;
        }
        atomicMin(&minPos[sa], 2 * e);
        atomicMin(&minPos[sb], 2 * e + 1);
        occSlot[2 * e] = sa;
        occSlot[2 * e + 1] = sb;
        occPt[2 * e] = verts[b + k];
        occPt[2 * e + 1] = verts[b + (k + 1) % c];
        ++e;
    }
}

__global__ void k_bnd_first(int occ, const unsigned *__restrict__ occSlot, const int *__restrict__ minPos,
                            int *__restrict__ first)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < occ) first[p] = minPos[occSlot[p]] == p;
}

// first[] now holds the exclusive scan of the first-occurrence flags
__global__ void k_bnd_number(int occ, const unsigned *__restrict__ occSlot, const int *__restrict__ minPos,
                             const int *__restrict__ first, const float2 *__restrict__ occPt, int *__restrict__ edges,
                             float2 *__restrict__ vertices)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= occ) return;
    const int f = minPos[occSlot[p]];
    edges[p] = first[f];
    if (f == p) vertices[first[p]] = occPt[p];
}

} // namespace vmk

cudaError_t vm_launch_boundary(int n, const int *start, const int *labels, const float2 *verts,
                               const unsigned char *inside, int *cnt, int phase, const int *eStart,
                               unsigned long long *keys, unsigned mask, int *minPos, unsigned *occSlot, float2 *occPt,
                               int occ, int *first, int *edges, float2 *vertices, int *err, cudaStream_t s)
{
    switch (phase) {
    case 0:
        if (n > 0) vmk::k_bnd_count<<<(n + 255) / 256, 256, 0, s>>>(n, start, labels, inside, cnt);
        break;
    case 1:
        if (n > 0)
            vmk::k_bnd_emit<<<(n + 255) / 256, 256, 0, s>>>(n, start, labels, verts, inside, eStart, keys, mask, minPos,
                                                            occSlot, occPt, err);
        break;
    case 2:
        if (occ > 0) vmk::k_bnd_first<<<(occ + 255) / 256, 256, 0, s>>>(occ, occSlot, minPos, first);
        break;
    default:
        if (occ > 0)
            vmk::k_bnd_number<<<(occ + 255) / 256, 256, 0, s>>>(occ, occSlot, minPos, first, occPt, edges, vertices);
        break;
    }
    return cudaGetLastError();
}

cudaError_t vm_launch_compact_cells(const float2 *verts, const int *labels, const int *start, int n, float2 *outV,
                                    int *outL, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    vmk::k_compact_cells<<<(n + 255) / 256, 256, 0, s>>>(verts, labels, start, n, outV, outL);
    return cudaGetLastError();
}

cudaError_t vm_launch_cells_n(const VmFit *fit, int nSlots, const unsigned long long *masks, int tilesX, int tilesY,
                              float invVoxel, float2 *outVerts, int *outEdges, int *outCount,
                              unsigned char *outInside, int *flags, cudaStream_t s)
{
    if (nSlots <= 0) return cudaSuccess;
    vmk::k_cells<<<(nSlots + 127) / 128, 128, 0, s>>>(fit, masks, tilesX, tilesY, invVoxel, outVerts, outEdges,
                                                      outCount, outInside, flags);
    return cudaGetLastError();
}
