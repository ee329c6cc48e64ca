#pragma once

// ---------------------------------------------------------------------------
// voro_optimizer.h — 2D VoroMesh fitting and extraction on a GB300.
//
// Drop-in for the reference's include/voromesh/voro_optimizer.h:34-138: the
// same types, the same public methods with the same meaning, and the same
// private data members in the same order (the inline members read them), so
// code written against the reference compiles and links against
// libvoromesh_gb300.so unchanged. Only the contents of Device differ.
//
// Generators (Voronoi sites) are fitted to a target point cloud by VoroLoss —
// for a target p with nearest generator c0, the squared distance to the
// nearest bisector of (c0, cj) over its K nearest generators cj — with Adam
// and a MultiStepLR schedule; Extract() clips each generator's Voronoi cell
// to the domain and assembles the watertight boundary between cells of
// opposite occupancy. Slots with x < 0 are empty.
//
// The loss uses the reference's K = 12 nearest generators unless
// voromesh::SetDefaultLossNeighbours() (voromesh/gb300_ext.h) chose another
// K before the optimiser was constructed.
// ---------------------------------------------------------------------------
#include "voromesh/shape2d.h"

#include <array>
#include <cstdint>
#include <memory>
#include <vector>

namespace voromesh {

struct OptimizerParams
{
    int                iterations      = 400;   // schedule length of a global fit
    int                localIterations = 100;   // schedule length after a local edit
    float              lrPerSpacing    = 0.09f; // Adam learning rate in units of `spacing`
    float              sampleFraction  = 0.2f;  // fraction of targets drawn per step
    float              gamma           = 0.5f;  // MultiStepLR decay
    std::array<int, 4> milestones      = {80, 150, 200, 250}; // for `iterations` steps
    unsigned           seed            = 1;     // target subsampling
};

struct VoroMesh2D
{
    // Clipped Voronoi diagram: one convex polygon per generator slot.
    std::vector<Vec2>    generators;
    std::vector<uint8_t> inside;    // cell centroid inside the occupancy
    std::vector<int>     cellStart; // CSR offsets into cellVerts (generators + 1 entries)
    std::vector<Vec2>    cellVerts;

    // Boundary between inside and outside cells; vertices keyed by the
    // generator triple they are equidistant to.
    std::vector<Vec2>               vertices;
    std::vector<std::array<int, 2>> edges;

    bool  watertight    = false; // every boundary vertex has one in- and one out-edge
    int   loops         = 0;     // closed boundary curves
    int   unsafeCells   = 0;     // cells not certified by the 32 nearest (brute-force fallback)
    int   overflowCells = 0;     // cells over the 24-vertex budget
    float gpuMs         = 0.0f;  // hash grid + cell clipping + occupancy
    float hostMs        = 0.0f;  // download + boundary assembly
};

class VoroOptimizer
{
public:
    /// Domain [0,width] x [0,height]; `spacing` sizes the hash grid and the lr.
    VoroOptimizer(float width, float height, float spacing, const OptimizerParams &params = {});
    ~VoroOptimizer();

    VoroOptimizer(const VoroOptimizer &) = delete;
    VoroOptimizer &operator=(const VoroOptimizer &) = delete;

    void SetTargets(const std::vector<Vec2> &slots);
    void UpdateTargets(const std::vector<int> &dirty, const std::vector<Vec2> &slots);

    void SetOccupancy(const std::vector<uint64_t> &masks, int tilesX, int tilesY, float voxelSize);
    void UpdateOccupancy(const std::vector<uint64_t> &masks, int tx0, int ty0, int tx1, int ty1);

    void SetGenerators(const Vec2 *slots, int slotsW, int slotsH, float slotCellSize);
    void UpdateGenerators(const Vec2 *slots, int cx0, int cy0, int cx1, int cy1);

    void BeginSchedule(int iterations, int cx0, int cy0, int cx1, int cy1);
    void BeginSchedule(int iterations) { BeginSchedule(iterations, 0, 0, mSlotsW, mSlotsH); }

    /// Runs `iterations` steps; returns their GPU time in ms.
    float Step(int iterations);
    /// Runs the rest of the current schedule.
    float Optimize() { return Step(mScheduleLength - mIteration); }

    float LastBatchLoss() const { return mLastBatchLoss; }
    float EvaluateLoss();

    VoroMesh2D Extract();

    int                    Iteration() const { return mIteration; }
    int                    ScheduleLength() const { return mScheduleLength; }
    int                    NumSlots() const { return mSlotsW * mSlotsH; }
    const OptimizerParams &Params() const { return mParams; }

private:
    struct Device;
    friend struct Gb300Access; // canvas hand-off (gb300_ext.h); no effect on the layout

    void BuildGraph();
    void EnqueueBuildGrid();
    void EnqueueIteration();

    float           mWidth, mHeight, mSpacing;
    OptimizerParams mParams;
    int             mSlotsW = 0, mSlotsH = 0;
    int             mTargetCapacity = 0;
    int             mIteration = 0, mScheduleLength = 0;
    float           mLastBatchLoss = 0.0f;

    std::unique_ptr<Device> mDev;
};

} // namespace voromesh
