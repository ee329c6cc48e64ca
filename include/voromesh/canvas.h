#pragma once

// ---------------------------------------------------------------------------
// canvas.h — voromesh::Canvas, the authoritative 2D shape, kept on the GPU.
//
// Same public declarations as the reference's include/voromesh/canvas.h:25-89
// (source-compatible, not link-compatible: the state lives in device memory
// behind a private handle). Voxel (i, j) covers [i, i+1) x [j, j+1) *
// voxelSize; voxels form 8x8 tiles and voxel (i, j) is bit
// (j & 7) * 8 + (i & 7) of its tile's word.
//   * Occupancy: dense row-major tile words, bit set = voxel centre inside.
//   * Surface: per surface voxel the mean of the boundary samples in it and
//     the target slot that mirrors it.
// TargetSlots() and InsideMasks() return host mirrors, refreshed from the
// device when an edit has changed them. Edits report the slots and tiles they
// changed. New rim voxels of a stamp take free slots in tile-major voxel
// order (the reference: std::unordered_map order), so slot indices may differ
// from the reference's by a relabelling; all values are the same.
// ---------------------------------------------------------------------------
#include "voromesh/shape2d.h"

#include <cstddef>
#include <cstdint>
#include <memory>
#include <vector>

namespace voromesh {

class Canvas
{
public:
    static constexpr int kTileLog2 = 3;
    static constexpr int kTileSize = 1 << kTileLog2; // voxels per tile side

    struct SurfaceTile
    {
        uint64_t mask = 0;
        Vec2     points[kTileSize * kTileSize];
        int      slots[kTileSize * kTileSize];
    };

    struct Edit
    {
        std::vector<int> dirtySlots;              // target slots whose value changed
        int tx0 = 0, ty0 = 0, tx1 = 0, ty1 = 0;   // occupancy tiles [tx0,tx1) x [ty0,ty1) rewritten
        int removed = 0, added = 0, flipped = 0;  // surface samples, occupancy voxels

        bool Changed() const { return removed + added + flipped > 0; }
    };

    Canvas(float width, float height, float voxelSize);
    ~Canvas();

    Canvas(const Canvas &)            = delete;
    Canvas &operator=(const Canvas &) = delete;

    /// Replaces the canvas with a closed polygon: its outline becomes the
    /// surface and its interior (by voxel centre) the occupancy.
    void RasterizeShape(const std::vector<Vec2> &polygon);

    /// Stamps a disc. Its interior becomes `inside` (false = carve, true =
    /// add), surface samples strictly inside it are deleted, and its rim
    /// becomes surface wherever it previously lay on the other side.
    Edit StampDisc(Vec2 center, float radius, bool inside);

    bool InDomain(int i, int j) const { return i >= 0 && j >= 0 && i < mVoxelsX && j < mVoxelsY; }
    bool IsInside(int i, int j) const;
    bool IsSurface(int i, int j) const;

    /// Host mirror of the GPU target array; {-1, -1} marks a free slot.
    const std::vector<Vec2>     &TargetSlots() const;
    const std::vector<uint64_t> &InsideMasks() const;

    int    TilesX() const { return mTilesX; }
    int    TilesY() const { return mTilesY; }
    float  VoxelSize() const { return mVoxelSize; }
    size_t SurfaceCount() const;
    size_t SurfaceTileCount() const;

private:
    struct Device;
    friend struct Gb300Access;

    float mVoxelSize;
    int   mVoxelsX, mVoxelsY, mTilesX, mTilesY;

    std::unique_ptr<Device> mDev;
};

} // namespace voromesh
