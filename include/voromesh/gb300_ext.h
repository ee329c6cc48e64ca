#pragma once

// ---------------------------------------------------------------------------
// gb300_ext.h — additions to the reference's C++ API (no counterpart there).
// ---------------------------------------------------------------------------

namespace voromesh {

/// Number of nearest generators the VoroLoss of optimisers constructed from
/// now on considers (8, 12, 16, 24 or 32; the reference fixes it at 12).
/// Returns false for an unsupported value. Process-wide, not thread-safe.
bool SetDefaultLossNeighbours(int k);
int  DefaultLossNeighbours();

} // namespace voromesh
