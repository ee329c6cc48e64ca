// voromesh::Canvas implemented over the cv_* C ABI (vm_capi.h): the canvas
// state lives on the GPU; TargetSlots() / InsideMasks() / IsSurface() read
// host mirrors that are brought up to date lazily. Errors follow the
// reference's convention for the GPU classes: message on stderr, exit(1).
#include "voromesh/canvas.h"
#include "voromesh/gb300_ext.h"
#include "voromesh/voro_optimizer.h"

#include <cstdio>
#include <cstdlib>

#include "gb300_access.h"
#include "vm_capi.h"

namespace {

void check(int rc, const char *what)
{
    if (rc == VM_OK) return;
    char msg[512];
    vm_last_error(msg, sizeof(msg));
    std::fprintf(stderr, "voromesh: %s failed: %s (%s)\n", what, vm_error_string(rc), msg);
    std::exit(1);
}

} // namespace

namespace voromesh {

struct Canvas::Device
{
    cv_canvas *h = nullptr;
    cv_info_t info{};
    // host mirrors; valid flags say whether they match the device
    mutable std::vector<Vec2>     slots;
    mutable std::vector<uint64_t> inside, surface;
    mutable bool slotsValid = true, insideValid = true, surfaceValid = true;
    // tile rectangle of occupancy changed since the mirror was last valid
    mutable int dtx0 = 0, dty0 = 0, dtx1 = 0, dty1 = 0;
    std::vector<float> values; // staging of an edit's dirty values
};

Canvas::Canvas(float width, float height, float voxelSize) : mDev(std::make_unique<Device>())
{
    check(cv_create(width, height, voxelSize, &mDev->h), "Canvas");
    check(cv_info(mDev->h, &mDev->info), "Canvas");
    mVoxelSize = mDev->info.voxelSize;
    mVoxelsX = mDev->info.voxelsX;
    mVoxelsY = mDev->info.voxelsY;
    mTilesX = mDev->info.tilesX;
    mTilesY = mDev->info.tilesY;
    mDev->inside.assign((size_t)mTilesX * mTilesY, 0);
    mDev->surface.assign((size_t)mTilesX * mTilesY, 0);
}

Canvas::~Canvas()
{
    if (mDev && mDev->h) cv_destroy(mDev->h);
}

void Canvas::RasterizeShape(const std::vector<Vec2> &polygon)
{
    check(cv_rasterize(mDev->h, reinterpret_cast<const float *>(polygon.data()), (int)polygon.size(), nullptr),
          "Canvas::RasterizeShape");
    check(cv_info(mDev->h, &mDev->info), "Canvas::RasterizeShape");
    mDev->slotsValid = mDev->insideValid = mDev->surfaceValid = false;
}

Canvas::Edit Canvas::StampDisc(Vec2 c, float radius, bool inside)
{
    Edit e;
    cv_edit ce{};
    check(cv_stamp_disc(mDev->h, c.x, c.y, radius, inside ? 1 : 0, &ce), "Canvas::StampDisc");
    check(cv_info(mDev->h, &mDev->info), "Canvas::StampDisc");
    e.tx0 = ce.tx0;
    e.ty0 = ce.ty0;
    e.tx1 = ce.tx1;
    e.ty1 = ce.ty1;
    e.removed = ce.removed;
    e.added = ce.added;
    e.flipped = ce.flipped;
    if (ce.ndirty > 0) {
        e.dirtySlots.resize((size_t)ce.ndirty);
        mDev->values.resize(2 * (size_t)ce.ndirty);
        check(cv_edit_dirty(mDev->h, e.dirtySlots.data(), mDev->values.data(), ce.ndirty), "Canvas::StampDisc");
        // the slot mirror follows the edit: every changed or new slot is dirty
        if (mDev->slotsValid) {
            mDev->slots.resize((size_t)mDev->info.numSlots, Vec2{-1.0f, -1.0f});
            for (int k = 0; k < ce.ndirty; ++k)
                mDev->slots[e.dirtySlots[k]] = Vec2{mDev->values[2 * k], mDev->values[2 * k + 1]};
        }
    }
    if (e.removed + e.added) mDev->surfaceValid = false;
    if (e.flipped && mDev->insideValid) {
        // only the edit's tiles are re-read, on the next access
        mDev->insideValid = false;
        mDev->dtx0 = e.tx0;
        mDev->dty0 = e.ty0;
        mDev->dtx1 = e.tx1;
        mDev->dty1 = e.ty1;
    } else if (e.flipped) {
        mDev->dtx0 = 0;
        mDev->dty0 = 0;
        mDev->dtx1 = mTilesX;
        mDev->dty1 = mTilesY;
    }
    return e;
}

const std::vector<Vec2> &Canvas::TargetSlots() const
{
    if (!mDev->slotsValid) {
        mDev->slots.resize((size_t)mDev->info.numSlots);
        check(cv_get_slots(mDev->h, reinterpret_cast<float *>(mDev->slots.data())), "Canvas::TargetSlots");
        mDev->slotsValid = true;
    }
    return mDev->slots;
}

const std::vector<uint64_t> &Canvas::InsideMasks() const
{
    if (!mDev->insideValid) {
        if (mDev->dtx1 > mDev->dtx0 && mDev->dty1 > mDev->dty0 &&
            (mDev->dtx1 - mDev->dtx0) * (mDev->dty1 - mDev->dty0) < mTilesX * mTilesY)
            check(cv_get_inside_rect(mDev->h, mDev->inside.data(), mDev->dtx0, mDev->dty0, mDev->dtx1, mDev->dty1),
                  "Canvas::InsideMasks");
        else
            check(cv_get_inside(mDev->h, mDev->inside.data()), "Canvas::InsideMasks");
        mDev->insideValid = true;
        mDev->dtx0 = mDev->dty0 = mDev->dtx1 = mDev->dty1 = 0;
    }
    return mDev->inside;
}

bool Canvas::IsInside(int i, int j) const
{
    const std::vector<uint64_t> &m = InsideMasks();
    return InDomain(i, j) &&
           (m[size_t(j >> kTileLog2) * mTilesX + (i >> kTileLog2)] >> (((j & 7) << kTileLog2) | (i & 7)) & 1);
}

bool Canvas::IsSurface(int i, int j) const
{
    if (!InDomain(i, j)) return false;
    if (!mDev->surfaceValid) {
        check(cv_get_surface(mDev->h, mDev->surface.data(), nullptr, nullptr), "Canvas::IsSurface");
        mDev->surfaceValid = true;
    }
    return mDev->surface[size_t(j >> kTileLog2) * mTilesX + (i >> kTileLog2)] >> (((j & 7) << kTileLog2) | (i & 7)) & 1;
}

cv_canvas *Gb300Access::handle(const Canvas &canvas) { return canvas.mDev->h; }

void SetTargetsFromCanvas(VoroOptimizer &opt, const Canvas &canvas)
{
    check(vm_set_targets_from_canvas(Gb300Access::handle(opt), Gb300Access::handle(canvas)), "SetTargetsFromCanvas");
    Gb300Access::refresh(opt);
}

void UpdateFromCanvas(VoroOptimizer &opt, const Canvas &canvas)
{
    check(vm_update_from_canvas(Gb300Access::handle(opt), Gb300Access::handle(canvas)), "UpdateFromCanvas");
    Gb300Access::refresh(opt);
}

size_t Canvas::SurfaceCount() const { return (size_t)mDev->info.surfaceCount; }

size_t Canvas::SurfaceTileCount() const { return (size_t)mDev->info.surfaceTiles; }

} // namespace voromesh
