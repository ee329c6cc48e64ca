// poisson::Sampler implemented over the C ABI (vm_capi.h). Errors print and
// exit(1) like the reference (src/poisson/poisson_disk.cu:32-40).
#include "poisson/poisson_disk.h"

#include <cstdio>
#include <cstdlib>

#include "vm_capi.h"

static_assert(sizeof(poisson::Sample) == 2 * sizeof(float), "Sample must mirror float2");

namespace {

void check(int rc, const char *what)
{
    if (rc == VM_OK) return;
    char msg[512];
    vm_last_error(msg, sizeof(msg));
    std::fprintf(stderr, "poisson: %s failed: %s (%s)\n", what, vm_error_string(rc), msg);
    std::exit(1);
}

} // namespace

namespace poisson {

Sampler::Sampler(float width, float height, float radius, int trials, unsigned seed)
    : mWidth(width), mHeight(height), mRadius(radius), mTrials(trials), mSeed(seed)
{
    pd_sampler *s = nullptr;
    check(pd_create(width, height, radius, trials, seed, &s), "Sampler");
    mDeviceGrid = s;
    pd_info_t info;
    check(pd_info(s, &info), "Sampler");
    mCellSize = info.cellSize;
    mGridW = info.gridW;
    mGridH = info.gridH;
    mRoundBase = info.roundBase;
    mCells.resize((size_t)mGridW * mGridH);
    check(pd_cells(s, reinterpret_cast<float *>(mCells.data())), "Sampler");
}

Sampler::~Sampler() { pd_destroy(static_cast<pd_sampler *>(mDeviceGrid)); }

float Sampler::Resample(int cx0, int cy0, int cx1, int cy1)
{
    pd_sampler *s = static_cast<pd_sampler *>(mDeviceGrid);
    float ms = 0.0f;
    check(pd_resample(s, cx0, cy0, cx1, cy1, &ms), "Resample");
    pd_info_t info;
    check(pd_info(s, &info), "Resample");
    mRoundBase = info.roundBase;
    check(pd_cells(s, reinterpret_cast<float *>(mCells.data())), "Resample");
    return ms;
}

bool Sampler::Verify(int cx0, int cy0, int cx1, int cy1) const
{
    int ok = 0;
    check(pd_verify(static_cast<pd_sampler *>(mDeviceGrid), cx0, cy0, cx1, cy1, &ok), "Verify");
    return ok != 0;
}

} // namespace poisson
