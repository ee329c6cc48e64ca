// A caller of the reference's Canvas API (include/voromesh/canvas.h) in the
// editor's order (apps/voromesh_demo.cpp:103-125): RasterizeShape, then
// StampDisc edits, each handed to an optimiser. Compiles unchanged against
// this library's headers; the hand-off uses gb300_ext.h where the editor
// passes host arrays.
//
// usage: canvas_demo <in.bin> <out.bin>
//   in:  int32 nPoly, nStamps; float32 poly[nPoly][2]; float32 stamps[nStamps][4] (cx, cy, r, inside)
//   out: per stamp int32 tx0 ty0 tx1 ty1 removed added flipped ndirty, then its dirty slots;
//        then int32 nSlots, float32 slots[nSlots][2]; int32 nTiles, uint64 masks[nTiles];
//        int32 surfaceCount, surfaceTiles, IsInside(100,100), IsSurface of the first slot's voxel;
//        float32 the optimiser's EvaluateLoss after the hand-offs
#include "voromesh/canvas.h"
#include "voromesh/gb300_ext.h"
#include "voromesh/voro_optimizer.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

using voromesh::Vec2;

int main(int argc, char **argv)
{
    if (argc != 3) return 2;
    FILE *in = std::fopen(argv[1], "rb");
    if (!in) return 2;
    int32_t nPoly = 0, nStamps = 0;
    if (std::fread(&nPoly, 4, 1, in) != 1 || std::fread(&nStamps, 4, 1, in) != 1) return 2;
    std::vector<Vec2> poly(nPoly);
    std::vector<float> stamps(4 * (size_t)nStamps);
    if (std::fread(poly.data(), sizeof(Vec2), nPoly, in) != (size_t)nPoly ||
        std::fread(stamps.data(), sizeof(float), stamps.size(), in) != stamps.size())
        return 2;
    std::fclose(in);
    FILE *out = std::fopen(argv[2], "wb");
    if (!out) return 2;

    voromesh::Canvas canvas(256.0f, 256.0f, 1.0f);
    canvas.RasterizeShape(poly);
    voromesh::OptimizerParams params;
    params.sampleFraction = 1.0f;
    voromesh::VoroOptimizer opt(256.0f, 256.0f, 8.0f, params);
    voromesh::SetTargetsFromCanvas(opt, canvas);
    std::vector<Vec2> gens;
    for (int j = 0; j < 32; ++j)
        for (int i = 0; i < 32; ++i) gens.push_back({(i + 0.5f) * 8.0f, (j + 0.5f) * 8.0f});
    opt.SetGenerators(gens.data(), 32, 32, 8.0f);
    opt.BeginSchedule(20);
    opt.Optimize();

    for (int k = 0; k < nStamps; ++k) {
        const float *s = &stamps[4 * (size_t)k];
        voromesh::Canvas::Edit e = canvas.StampDisc({s[0], s[1]}, s[2], s[3] != 0.0f);
        int32_t head[8] = {e.tx0, e.ty0, e.tx1, e.ty1, e.removed, e.added, e.flipped, (int32_t)e.dirtySlots.size()};
        std::fwrite(head, 4, 8, out);
        std::fwrite(e.dirtySlots.data(), 4, e.dirtySlots.size(), out);
        if (e.Changed()) {
            voromesh::UpdateFromCanvas(opt, canvas);
            opt.BeginSchedule(5);
            opt.Optimize();
        }
    }
    const std::vector<Vec2> &slots = canvas.TargetSlots();
    int32_t ns = (int32_t)slots.size();
    std::fwrite(&ns, 4, 1, out);
    std::fwrite(slots.data(), sizeof(Vec2), slots.size(), out);
    const std::vector<uint64_t> &masks = canvas.InsideMasks();
    int32_t nt = (int32_t)masks.size();
    std::fwrite(&nt, 4, 1, out);
    std::fwrite(masks.data(), 8, masks.size(), out);
    int32_t tail[4] = {(int32_t)canvas.SurfaceCount(), (int32_t)canvas.SurfaceTileCount(), canvas.IsInside(100, 100),
                       0};
    for (const Vec2 &p : slots)
        if (p.x >= 0.0f) {
            tail[3] = canvas.IsSurface((int)std::floor(p.x), (int)std::floor(p.y));
            break;
        }
    std::fwrite(tail, 4, 4, out);
    float loss = opt.EvaluateLoss();
    std::fwrite(&loss, 4, 1, out);
    std::fclose(out);
    return 0;
}
