#pragma once

// ---------------------------------------------------------------------------
// gb300_ext.h — additions to the reference's C++ API (no counterpart there).
// ---------------------------------------------------------------------------

namespace voromesh {

class VoroOptimizer;
class Canvas;

/// Device-to-device hand-off from a canvas on the same GPU:
/// SetTargets(canvas.TargetSlots()) + SetOccupancy(canvas.InsideMasks(),
/// canvas.TilesX(), canvas.TilesY(), canvas.VoxelSize()).
void SetTargetsFromCanvas(VoroOptimizer &opt, const Canvas &canvas);
/// UpdateTargets(edit.dirtySlots, canvas.TargetSlots()) +
/// UpdateOccupancy(canvas.InsideMasks(), edit rectangle) for the canvas's
/// last StampDisc, without copying through the host.
void UpdateFromCanvas(VoroOptimizer &opt, const Canvas &canvas);

/// Number of nearest generators the VoroLoss of optimisers constructed from
/// now on considers (8, 12, 16, 24 or 32; the reference fixes it at 12).
/// Returns false for an unsupported value. Process-wide, not thread-safe.
bool SetDefaultLossNeighbours(int k);
int  DefaultLossNeighbours();

} // namespace voromesh
