// C entry points around the reference's own Canvas (src/voromesh/canvas.cpp
// and src/voromesh/shape2d.cpp, compiled in place by build_ref.sh into
// oracle/_ref/libref_canvas.so). Test infrastructure: the pins in tests/ and
// the fixture generator in tests/golden/ read the reference state through
// these functions.
//
// The private members are opened for reading only (free list, surface map),
// so that the full state can be compared with the oracle's.
#include <cstdint>
#include <vector>

#define private public
#include "voromesh/canvas.h"
#undef private

using voromesh::Canvas;
using voromesh::Vec2;

extern "C" {

void *rc_canvas_create(float w, float h, float voxel) { return new Canvas(w, h, voxel); }

void rc_canvas_destroy(void *c) { delete static_cast<Canvas *>(c); }

void rc_canvas_rasterize(void *c, const float *xy, int n)
{
    std::vector<Vec2> poly((size_t)n);
    for (int k = 0; k < n; ++k) poly[k] = {xy[2 * k], xy[2 * k + 1]};
    static_cast<Canvas *>(c)->RasterizeShape(poly);
}

// counts: tx0 ty0 tx1 ty1 removed added flipped ndirty; dirty: up to cap entries
void rc_canvas_stamp(void *c, float cx, float cy, float r, int inside, int *counts, int *dirty, int cap)
{
    Canvas::Edit e = static_cast<Canvas *>(c)->StampDisc({cx, cy}, r, inside != 0);
    counts[0] = e.tx0; counts[1] = e.ty0; counts[2] = e.tx1; counts[3] = e.ty1;
    counts[4] = e.removed; counts[5] = e.added; counts[6] = e.flipped;
    counts[7] = (int)e.dirtySlots.size();
    for (int k = 0; k < (int)e.dirtySlots.size() && k < cap; ++k) dirty[k] = e.dirtySlots[k];
}

// counts: slots, free slots, surface voxels, surface tiles
void rc_canvas_counts(void *c, long long *counts)
{
    Canvas *cv = static_cast<Canvas *>(c);
    counts[0] = (long long)cv->mSlots.size();
    counts[1] = (long long)cv->mFreeSlots.size();
    counts[2] = (long long)cv->SurfaceCount();
    counts[3] = (long long)cv->SurfaceTileCount();
}

// Dense export in the oracle's layout (tiles x 64 voxels, tile-major).
void rc_canvas_get(void *c, float *slots, int *freeList, uint64_t *inside, uint64_t *smask, float *spt, int *sslot)
{
    Canvas *cv = static_cast<Canvas *>(c);
    size_t tiles = (size_t)cv->TilesX() * cv->TilesY();
    for (size_t s = 0; s < cv->mSlots.size(); ++s) {
        slots[2 * s] = cv->mSlots[s].x;
        slots[2 * s + 1] = cv->mSlots[s].y;
    }
    for (size_t s = 0; s < cv->mFreeSlots.size(); ++s) freeList[s] = cv->mFreeSlots[s];
    for (size_t t = 0; t < tiles; ++t) {
        inside[t] = cv->InsideMasks()[t];
        smask[t] = 0;
        for (int b = 0; b < 64; ++b) {
            spt[2 * (t * 64 + b)] = -1.0f;
            spt[2 * (t * 64 + b) + 1] = -1.0f;
            sslot[t * 64 + b] = -1;
        }
    }
    for (const auto &kv : cv->mSurface) {
        int tx = (int)(uint32_t)kv.first, ty = (int)(uint32_t)(kv.first >> 32);
        size_t t = (size_t)ty * cv->TilesX() + tx;
        const Canvas::SurfaceTile &st = kv.second;
        smask[t] = st.mask;
        for (int b = 0; b < 64; ++b) {
            if (!(st.mask >> b & 1)) continue;
            spt[2 * (t * 64 + b)] = st.points[b].x;
            spt[2 * (t * 64 + b) + 1] = st.points[b].y;
            sslot[t * 64 + b] = st.slots[b];
        }
    }
}

// voromesh::MakeHeart (src/voromesh/shape2d.cpp:7-24)
void rc_make_heart(float cx, float cy, float width, int segments, float *xy)
{
    std::vector<Vec2> p = voromesh::MakeHeart(cx, cy, width, segments);
    for (int k = 0; k < segments; ++k) {
        xy[2 * k] = p[k].x;
        xy[2 * k + 1] = p[k].y;
    }
}

} // extern "C"
