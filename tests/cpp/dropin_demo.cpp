// A caller written against the reference's C++ API (include/voromesh,
// include/poisson), as its demos use it (apps/voromesh_demo.cpp:94-181,
// apps/poisson_demo.cpp:122-148): sampler fill and verify, a global fit, a
// local edit (UpdateTargets, UpdateOccupancy, region Resample,
// UpdateGenerators, BeginSchedule on a rectangle) and Extract. It compiles
// unchanged against this library's headers and links libvoromesh_gb300.so.
//
// usage: dropin_demo <in.bin> <out.bin>
//   in:  int32 nGen, nTgt; float32 gen[nGen][2], tgt[nTgt][2]
//   out: float32 loss after the global fit, loss after the edit; int32
//        samples, verified, watertight, loops, boundary edges; float32
//        generators[nGen][2] after the edit
#include "poisson/poisson_disk.h"
#include "voromesh/gb300_ext.h"
#include "voromesh/voro_optimizer.h"

#include <cstdint>
#include <cstdio>
#include <vector>

using voromesh::Vec2;

int main(int argc, char **argv)
{
    if (argc != 3) return 2;
    FILE *in = std::fopen(argv[1], "rb");
    if (!in) return 2;
    int32_t nGen = 0, nTgt = 0;
    if (std::fread(&nGen, 4, 1, in) != 1 || std::fread(&nTgt, 4, 1, in) != 1) return 2;
    std::vector<Vec2> gen(nGen), tgt(nTgt);
    if (std::fread(gen.data(), sizeof(Vec2), nGen, in) != (size_t)nGen ||
        std::fread(tgt.data(), sizeof(Vec2), nTgt, in) != (size_t)nTgt)
        return 2;
    std::fclose(in);

    // Poisson sampler: fill, verify
    poisson::Sampler sampler(1.0f, 1.0f, 0.02f, 30, 1);
    sampler.ResampleAll();
    int samples = 0;
    for (const poisson::Sample &s : sampler.Cells()) samples += s.x >= 0.0f;
    int verified = sampler.VerifyAll() ? 1 : 0;

    // global fit: every target each step, the reference's default K = 12
    voromesh::SetDefaultLossNeighbours(12);
    voromesh::OptimizerParams params;
    params.iterations = 60;
    params.localIterations = 20;
    params.sampleFraction = 1.0f;
    voromesh::VoroOptimizer opt(2.0f, 2.0f, 0.05f, params);
    opt.SetTargets(tgt);
    // occupancy: a disc of radius 0.6 around the centre, 8x8-voxel tiles of 0.025
    const float voxel = 0.025f;
    const int tiles = 10; // 80 voxels = 2.0
    std::vector<uint64_t> masks(tiles * tiles, 0);
    for (int j = 0; j < tiles * 8; ++j)
        for (int i = 0; i < tiles * 8; ++i) {
            float x = (i + 0.5f) * voxel - 1.0f, y = (j + 0.5f) * voxel - 1.0f;
            if (x * x + y * y < 0.36f) masks[(j >> 3) * tiles + (i >> 3)] |= 1ull << (((j & 7) << 3) | (i & 7));
        }
    opt.SetOccupancy(masks, tiles, tiles, voxel);
    opt.SetGenerators(gen.data(), nGen, 1, 2.0f);
    opt.BeginSchedule(params.iterations);
    opt.Optimize();
    float loss0 = opt.EvaluateLoss();

    // local edit: move the targets of the first 64 slots, refit a rectangle of slots
    std::vector<int> dirty;
    std::vector<Vec2> slots = tgt;
    for (int k = 0; k < 64 && k < nTgt; ++k) {
        slots[k].x = slots[k].x * 0.98f + 0.02f;
        dirty.push_back(k);
    }
    opt.UpdateTargets(dirty, slots);
    opt.UpdateOccupancy(masks, 0, 0, tiles, tiles);
    sampler.Resample(0, 0, 10, 10);
    std::vector<Vec2> moved = gen; // the full slot array; the rectangle is read from it
    for (int k = 0; k < 256 && k < nGen; ++k) moved[k].x = moved[k].x < 0.0f ? moved[k].x : moved[k].x * 0.999f;
    opt.UpdateGenerators(moved.data(), 0, 0, 256, 1);
    opt.BeginSchedule(params.localIterations, 0, 0, 256, 1);
    opt.Optimize();
    float loss1 = opt.EvaluateLoss();

    voromesh::VoroMesh2D mesh = opt.Extract();
    FILE *out = std::fopen(argv[2], "wb");
    if (!out) return 3;
    int32_t ints[5] = {samples, verified, mesh.watertight ? 1 : 0, mesh.loops, (int32_t)mesh.edges.size()};
    std::fwrite(&loss0, 4, 1, out);
    std::fwrite(&loss1, 4, 1, out);
    std::fwrite(ints, 4, 5, out);
    std::fwrite(mesh.generators.data(), sizeof(Vec2), mesh.generators.size(), out);
    std::fclose(out);
    std::printf("samples %d verified %d loss %.6g -> %.6g watertight %d loops %d edges %d\n", samples, verified,
                (double)loss0, (double)loss1, ints[2], ints[3], ints[4]);
    return 0;
}
