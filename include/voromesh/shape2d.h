#pragma once

// ---------------------------------------------------------------------------
// shape2d.h — the 2D point type shared by the VoroMesh and Poisson APIs.
//
// Drop-in for the reference's include/voromesh/shape2d.h:10-14 (Vec2). The
// reference's MakeHeart demo shape (shape2d.h:21, a demo input) is not part
// of this library.
// ---------------------------------------------------------------------------

namespace voromesh {

/// An (x, y) point with the memory layout of CUDA's float2.
struct Vec2
{
    float x, y;
};

} // namespace voromesh
