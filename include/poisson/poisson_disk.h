#pragma once

// ---------------------------------------------------------------------------
// poisson_disk.h — Poisson-disk sampling by phase-grid dart throwing on a GB300.
//
// Drop-in for the reference's include/poisson/poisson_disk.h:13-62: same
// types, methods and private data members. Any rectangle of background-grid
// cells can be cleared and refilled while the samples around it stay fixed,
// so the whole set remains a valid Poisson-disk set.
// ---------------------------------------------------------------------------
#include <vector>

namespace poisson {

/// float2 layout; x < 0 marks an empty cell.
struct Sample
{
    float x, y;
};

class Sampler
{
public:
    Sampler(float width, float height, float radius, int trials = 30, unsigned seed = 1);
    ~Sampler();

    Sampler(const Sampler &) = delete;
    Sampler &operator=(const Sampler &) = delete;

    /// Clears cells [cx0,cx1) x [cy0,cy1) (clamped), throws `trials` rounds of
    /// darts into them and refreshes Cells() there. Returns GPU ms.
    float Resample(int cx0, int cy0, int cx1, int cy1);
    float ResampleAll() { return Resample(0, 0, mGridW, mGridH); }

    /// Host check: no two samples touching the region (plus the 2-cell
    /// conflict margin) are closer than the radius.
    bool Verify(int cx0, int cy0, int cx1, int cy1) const;
    bool VerifyAll() const { return Verify(0, 0, mGridW, mGridH); }

    /// Row-major host mirror of the grid, GridW() * GridH() cells.
    const std::vector<Sample> &Cells() const { return mCells; }

    float Width() const { return mWidth; }
    float Height() const { return mHeight; }
    float Radius() const { return mRadius; }
    float CellSize() const { return mCellSize; }
    int   GridW() const { return mGridW; }
    int   GridH() const { return mGridH; }
    int   Trials() const { return mTrials; }

private:
    float    mWidth, mHeight, mRadius, mCellSize;
    int      mGridW, mGridH, mTrials;
    unsigned mSeed;
    unsigned mRoundBase = 0; // advanced by `trials` per Resample

    void *mDeviceGrid = nullptr; // the library's sampler handle
    void *mStart = nullptr, *mStop = nullptr; // unused (kept for layout)

    std::vector<Sample> mCells;
};

} // namespace poisson
