// voromesh::VoroOptimizer implemented over the C ABI (vm_capi.h).
//
// Error behaviour is the reference's (src/voromesh/voro_optimizer.cu:42-50):
// any failure prints a message to stderr and exits with status 1.
#include "voromesh/voro_optimizer.h"
#include "voromesh/gb300_ext.h"

#include <cstdio>
#include <cstdlib>

#include "gb300_access.h"
#include "vm_capi.h"

static_assert(sizeof(voromesh::Vec2) == 2 * sizeof(float), "Vec2 must mirror float2");

namespace {

int g_defaultLossK = 12;

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

bool SetDefaultLossNeighbours(int k)
{
    if (k != 8 && k != 12 && k != 16 && k != 24 && k != 32) return false;
    g_defaultLossK = k;
    return true;
}

int DefaultLossNeighbours() { return g_defaultLossK; }

struct VoroOptimizer::Device
{
    vm_optimizer *h = nullptr;
};

VoroOptimizer::VoroOptimizer(float width, float height, float spacing, const OptimizerParams &params)
    : mWidth(width), mHeight(height), mSpacing(spacing), mParams(params), mDev(std::make_unique<Device>())
{
    vm_params p;
    vm_params_default(&p);
    p.iterations = params.iterations;
    p.localIterations = params.localIterations;
    p.lrPerSpacing = params.lrPerSpacing;
    p.sampleFraction = params.sampleFraction;
    p.gamma = params.gamma;
    for (int k = 0; k < 4; ++k) p.milestones[k] = params.milestones[k];
    p.seed = params.seed;
    p.lossK = g_defaultLossK;
    check(vm_create(width, height, spacing, &p, &mDev->h), "VoroOptimizer");
}

VoroOptimizer::~VoroOptimizer()
{
    if (mDev) vm_destroy(mDev->h);
}

void VoroOptimizer::SetTargets(const std::vector<Vec2> &slots)
{
    check(vm_set_targets(mDev->h, reinterpret_cast<const float *>(slots.data()), (int)slots.size()), "SetTargets");
    vm_info_t info;
    check(vm_info(mDev->h, &info), "SetTargets");
    mTargetCapacity = info.targetCapacity;
}

void VoroOptimizer::UpdateTargets(const std::vector<int> &dirty, const std::vector<Vec2> &slots)
{
    check(vm_update_targets(mDev->h, dirty.data(), (int)dirty.size(), reinterpret_cast<const float *>(slots.data()),
                            (int)slots.size()),
          "UpdateTargets");
    vm_info_t info;
    check(vm_info(mDev->h, &info), "UpdateTargets");
    mTargetCapacity = info.targetCapacity;
}

void VoroOptimizer::SetOccupancy(const std::vector<uint64_t> &masks, int tilesX, int tilesY, float voxelSize)
{
    if (masks.size() < (size_t)tilesX * (size_t)tilesY) check(VM_ERR_ARG, "SetOccupancy");
    check(vm_set_occupancy(mDev->h, masks.data(), tilesX, tilesY, voxelSize), "SetOccupancy");
}

void VoroOptimizer::UpdateOccupancy(const std::vector<uint64_t> &masks, int tx0, int ty0, int tx1, int ty1)
{
    check(vm_update_occupancy(mDev->h, masks.data(), tx0, ty0, tx1, ty1), "UpdateOccupancy");
}

void VoroOptimizer::SetGenerators(const Vec2 *slots, int slotsW, int slotsH, float slotCellSize)
{
    check(vm_set_generators(mDev->h, reinterpret_cast<const float *>(slots), slotsW, slotsH, slotCellSize),
          "SetGenerators");
    mSlotsW = slotsW;
    mSlotsH = slotsH;
    mScheduleLength = mParams.iterations;
    mIteration = 0;
    mLastBatchLoss = 0.0f;
}

void VoroOptimizer::UpdateGenerators(const Vec2 *slots, int cx0, int cy0, int cx1, int cy1)
{
    check(vm_update_generators(mDev->h, reinterpret_cast<const float *>(slots), cx0, cy0, cx1, cy1),
          "UpdateGenerators");
}

void VoroOptimizer::BeginSchedule(int iterations, int cx0, int cy0, int cx1, int cy1)
{
    check(vm_begin_schedule(mDev->h, iterations, cx0, cy0, cx1, cy1), "BeginSchedule");
    mScheduleLength = iterations;
    mIteration = 0;
    mLastBatchLoss = 0.0f;
}

float VoroOptimizer::Step(int iterations)
{
    float ms = 0.0f;
    check(vm_step(mDev->h, iterations, &ms), "Step");
    vm_info_t info;
    check(vm_info(mDev->h, &info), "Step");
    mIteration = info.iteration;
    mLastBatchLoss = info.lastBatchLoss;
    return ms;
}

float VoroOptimizer::EvaluateLoss()
{
    float loss = 0.0f;
    check(vm_evaluate_loss(mDev->h, &loss), "EvaluateLoss");
    return loss;
}

VoroMesh2D VoroOptimizer::Extract()
{
    VoroMesh2D mesh;
    vm_mesh_info info;
    check(vm_extract(mDev->h, &info), "Extract");
    mesh.generators.resize(info.numGenerators);
    mesh.inside.resize(info.numGenerators);
    mesh.cellStart.resize(info.numGenerators > 0 ? info.numGenerators + 1 : 0);
    mesh.cellVerts.resize(info.numCellVerts);
    mesh.vertices.resize(info.numVertices);
    mesh.edges.resize(info.numEdges);
    check(vm_mesh_copy(mDev->h, reinterpret_cast<float *>(mesh.generators.data()), mesh.inside.data(),
                       mesh.cellStart.data(), reinterpret_cast<float *>(mesh.cellVerts.data()),
                       reinterpret_cast<float *>(mesh.vertices.data()), reinterpret_cast<int *>(mesh.edges.data()),
                       nullptr),
          "Extract");
    mesh.watertight = info.watertight != 0;
    mesh.loops = info.loops;
    mesh.unsafeCells = info.unsafeCells;
    mesh.overflowCells = info.overflowCells;
    mesh.gpuMs = info.gpuMs;
    mesh.hostMs = info.hostMs;
    return mesh;
}

vm_optimizer *Gb300Access::handle(VoroOptimizer &opt) { return opt.mDev->h; }

void Gb300Access::refresh(VoroOptimizer &opt)
{
    vm_info_t info;
    check(vm_info(opt.mDev->h, &info), "VoroOptimizer");
    opt.mTargetCapacity = info.targetCapacity;
}

// The step graph, grid build and iteration are enqueued inside the library;
// these private members only keep the reference's class declaration intact.
void VoroOptimizer::BuildGraph() {}
void VoroOptimizer::EnqueueBuildGrid() {}
void VoroOptimizer::EnqueueIteration() {}

} // namespace voromesh
