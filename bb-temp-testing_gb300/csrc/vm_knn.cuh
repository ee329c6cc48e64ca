// Exact K-nearest-site query by square-ring search over the cell-sorted hash
// grid (reference voro_optimizer.cu:130-163), with the top-K kept in
// registers by a branch-free unrolled insertion and distance ties ordered by
// site index. The ring loop and its termination test (the K-th distance is
// within the distance from the query to the searched block's edge, or the
// block covers the grid) are the reference's.
#pragma once

#include "vm_device.cuh"

namespace vmk {

template <int K>
__device__ __forceinline__ void topk_insert(float (&d2)[K], int (&idx)[K], float dd, int id)
{
    if (!key_less(dd, id, d2[K - 1], idx[K - 1])) return;
#pragma unroll
    for (int k = K - 1; k >= 1; --k) {
        bool a = key_less(dd, id, d2[k - 1], idx[k - 1]);
        bool b = key_less(dd, id, d2[k], idx[k]);
        float nd = a ? d2[k - 1] : (b ? dd : d2[k]);
        int ni = a ? idx[k - 1] : (b ? id : idx[k]);
        d2[k] = nd;
        idx[k] = ni;
    }
    if (key_less(dd, id, d2[0], idx[0])) {
        d2[0] = dd;
        idx[0] = id;
    }
}

// Ring search around q's cell. pos/sid are the cell-sorted site arrays.
template <int K>
__device__ void knn_ring(const int *__restrict__ start, const float2 *__restrict__ pos, const int *__restrict__ sid,
                         int gw, int gh, float cell, float inv, float2 q, float (&d2)[K], int (&idx)[K])
{
#pragma unroll
    for (int k = 0; k < K; ++k) {
        d2[k] = FLT_MAX;
        idx[k] = -1;
    }
    int cx = cell_coord(q.x, inv, gw), cy = cell_coord(q.y, inv, gh);
    for (int ring = 0;; ++ring) {
        int x0 = cx - ring, x1 = cx + ring, y0 = cy - ring, y1 = cy + ring;
        int ya = max(y0, 0), yb = min(y1, gh - 1);
        for (int y = ya; y <= yb; ++y) {
            if (y == y0 || y == y1) {
                // full row of the ring: cells x0..x1 are one contiguous run
                int xa = max(x0, 0), xb = min(x1, gw - 1);
                if (xa > xb) continue;
                int s0 = __ldg(&start[y * gw + xa]), s1 = __ldg(&start[y * gw + xb + 1]);
                for (int s = s0; s < s1; ++s) {
                    float2 p = __ldg(&pos[s]);
                    float dx = p.x - q.x, dy = p.y - q.y;
                    topk_insert<K>(d2, idx, dx * dx + dy * dy, __ldg(&sid[s]));
                }
            } else {
                // interior row: only the two end cells belong to the ring
#pragma unroll
                for (int side = 0; side < 2; ++side) {
                    int x = side ? x1 : x0;
                    if (side && x1 == x0) break;
                    if (x < 0 || x >= gw) continue;
                    int s0 = __ldg(&start[y * gw + x]), s1 = __ldg(&start[y * gw + x + 1]);
                    for (int s = s0; s < s1; ++s) {
                        float2 p = __ldg(&pos[s]);
                        float dx = p.x - q.x, dy = p.y - q.y;
                        topk_insert<K>(d2, idx, dx * dx + dy * dy, __ldg(&sid[s]));
                    }
                }
            }
        }
        if (x0 <= 0 && y0 <= 0 && x1 >= gw - 1 && y1 >= gh - 1) break;
        float safe = fminf(fminf(q.x - (float)x0 * cell, (float)(x1 + 1) * cell - q.x),
                           fminf(q.y - (float)y0 * cell, (float)(y1 + 1) * cell - q.y));
        safe = fmaxf(safe, 0.0f);
        if (d2[K - 1] <= safe * safe) break;
    }
}

} // namespace vmk
