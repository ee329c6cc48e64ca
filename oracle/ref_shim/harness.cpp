// Host entry points around the reference's own kernels (compiled from the
// reference sources by build_ref.sh; that script places the kernel sections
// in namespaces k12 / k16 (kLossK = 12 / 16) and pd before this file).
//
// Each entry point runs one kernel over all of its threads in index order,
// which is a legal schedule of the reference's launch: the bin kernel's
// atomic ranks then come out in slot order and every float atomic is applied
// in thread order. The host orchestration between kernels (grid build order,
// step sequence) is driven from tests/golden/make_golden.py.
#include <vector>

namespace {

template <class G> G make_grid(const int *start, const int *idx, const float *pos, int w, int h, float cell)
{
    G g;
    g.start = start;
    g.idx = idx;
    g.pos = reinterpret_cast<const float2 *>(pos);
    g.w = w;
    g.h = h;
    g.cellSize = cell;
    return g;
}

void one_thread(unsigned i)
{
    blockIdx.x = i; blockIdx.y = 0; blockIdx.z = 0;
    threadIdx.x = 0; threadIdx.y = 0; threadIdx.z = 0;
    blockDim.x = 1; blockDim.y = 1; blockDim.z = 1;
}

template <class RP> void fill_rp(RP &rp, const float *f, const int *iv)
{
    // f: lr gamma beta1 beta2 eps width height bx0 by0 bx1 by1
    // iv: milestones[4] slotsW cx0 cy0 cx1 cy1
    rp.lr = f[0]; rp.gamma = f[1]; rp.beta1 = f[2]; rp.beta2 = f[3]; rp.eps = f[4];
    rp.width = f[5]; rp.height = f[6];
    rp.bx0 = f[7]; rp.by0 = f[8]; rp.bx1 = f[9]; rp.by1 = f[10];
    for (int k = 0; k < 4; ++k) rp.milestones[k] = iv[k];
    rp.slotsW = iv[4]; rp.cx0 = iv[5]; rp.cy0 = iv[6]; rp.cx1 = iv[7]; rp.cy1 = iv[8];
}

} // namespace

extern "C" {

// binKernel -> exclusive scan of counts -> scatterKernel (voro_optimizer.cu:689-700)
void ref_build_grid(const float *gen, int n, int gw, int gh, float cell, int *start, int *sortedIdx,
                    float *sortedPos, int *genCell)
{
    int cells = gw * gh + 1;
    std::vector<int> counts(cells, 0), rank(n > 0 ? n : 1, 0);
    k12::HashGrid g = make_grid<k12::HashGrid>(start, sortedIdx, sortedPos, gw, gh, cell);
    const float2 *gp = reinterpret_cast<const float2 *>(gen);
    for (int i = 0; i < n; ++i) { one_thread(i); k12::binKernel(gp, n, g, counts.data(), genCell, rank.data()); }
    int run = 0;
    for (int c = 0; c < cells; ++c) { start[c] = run; run += counts[c]; }
    for (int i = 0; i < n; ++i) {
        one_thread(i);
        k12::scatterKernel(gp, n, genCell, rank.data(), start, sortedIdx, reinterpret_cast<float2 *>(sortedPos));
    }
}

// knn<K> (voro_optimizer.cu:130-163) for each query
void ref_knn(int K, const int *start, const int *sidx, const float *spos, int gw, int gh, float cell,
             const float *queries, int nq, int *outIdx, float *outD2)
{
    k12::HashGrid g = make_grid<k12::HashGrid>(start, sidx, spos, gw, gh, cell);
    for (int i = 0; i < nq; ++i) {
        float2 q = make_float2(queries[2 * i], queries[2 * i + 1]);
        int *I = outIdx + (size_t)i * K;
        float *D = outD2 + (size_t)i * K;
        switch (K) {
        case 12: k12::knn<12>(g, q, I, D); break;
        case 16: k12::knn<16>(g, q, I, D); break;
        case 32: k12::knn<32>(g, q, I, D); break;
        default: break;
        }
    }
}

// vorolossKernel (voro_optimizer.cu:199-266) over all targets. state: iter,count (int) and loss (float).
// rpf/rpi NULL -> rp = nullptr (EvaluateLoss). grad NULL -> loss only.
void ref_loss(int K, const float *targets, int numTargets, const int *start, const int *sidx, const float *spos,
              int gw, int gh, float cell, const float *gen, float *grad, int *stateInt, float *stateLoss,
              const float *rpf, const int *rpi, float fraction, unsigned seed)
{
    const float2 *tp = reinterpret_cast<const float2 *>(targets);
    const float2 *gp = reinterpret_cast<const float2 *>(gen);
    float2 *gr = reinterpret_cast<float2 *>(grad);
    if (K == 12) {
        k12::HashGrid g = make_grid<k12::HashGrid>(start, sidx, spos, gw, gh, cell);
        k12::IterState st{stateInt[0], stateInt[1], *stateLoss};
        k12::RunParams rp;
        if (rpf) fill_rp(rp, rpf, rpi);
        for (int i = 0; i < numTargets; ++i) {
            one_thread(i);
            k12::vorolossKernel(tp, numTargets, g, gp, gr, &st, rpf ? &rp : nullptr, fraction, seed);
        }
        stateInt[0] = st.iter; stateInt[1] = st.count; *stateLoss = st.loss;
    } else {
        k16::HashGrid g = make_grid<k16::HashGrid>(start, sidx, spos, gw, gh, cell);
        k16::IterState st{stateInt[0], stateInt[1], *stateLoss};
        k16::RunParams rp;
        if (rpf) fill_rp(rp, rpf, rpi);
        for (int i = 0; i < numTargets; ++i) {
            one_thread(i);
            k16::vorolossKernel(tp, numTargets, g, gp, gr, &st, rpf ? &rp : nullptr, fraction, seed);
        }
        stateInt[0] = st.iter; stateInt[1] = st.count; *stateLoss = st.loss;
    }
}

// adamKernel (voro_optimizer.cu:271-301)
void ref_adam(float *gen, float *m, float *v, float *grad, int n, int iter, int count, const float *rpf,
              const int *rpi)
{
    k12::IterState st{iter, count, 0.0f};
    k12::RunParams rp;
    fill_rp(rp, rpf, rpi);
    for (int i = 0; i < n; ++i) {
        one_thread(i);
        k12::adamKernel(reinterpret_cast<float2 *>(gen), reinterpret_cast<float2 *>(m), reinterpret_cast<float2 *>(v),
                        reinterpret_cast<float2 *>(grad), n, &st, &rp);
    }
}

// voronoiCellKernel (voro_optimizer.cu:361-437)
void ref_cells(const int *start, const int *sidx, const float *spos, int gw, int gh, float cell, const float *gen,
               int n, float width, float height, const unsigned long long *masks, int tilesX, int tilesY,
               float invVoxel, float *outVerts, int *outEdges, int *outCount, unsigned char *outInside, int *flags)
{
    k12::HashGrid g = make_grid<k12::HashGrid>(start, sidx, spos, gw, gh, cell);
    k12::Occupancy occ{masks, tilesX, tilesY, invVoxel};
    flags[0] = flags[1] = 0;
    for (int i = 0; i < n; ++i) {
        one_thread(i);
        k12::voronoiCellKernel(g, reinterpret_cast<const float2 *>(gen), n, width, height, occ,
                               reinterpret_cast<float2 *>(outVerts), outEdges, outCount, outInside, flags);
    }
}

// Sampler::Resample body (poisson_disk.cu:141-164): clearRegionKernel + trials x 9 dartPhaseKernel launches
void ref_poisson_resample(float *grid, float width, float height, float radius, float cellSize, int gridW, int gridH,
                          unsigned seed, int x0, int y0, int x1, int y1, int trials, unsigned roundBase)
{
    pd::Region rg{x0, y0, x1, y1};
    pd::Params p{width, height, radius, cellSize, gridW, gridH, seed};
    float2 *gp = reinterpret_cast<float2 *>(grid);
    int rw = x1 - x0, rh = y1 - y0;
    if (rw <= 0 || rh <= 0) return;
    for (int cy = 0; cy < rh; ++cy)
        for (int cx = 0; cx < rw; ++cx) {
            blockIdx.x = cx; blockIdx.y = cy; threadIdx.x = threadIdx.y = 0; blockDim.x = blockDim.y = 1;
            pd::clearRegionKernel(gp, gridW, rg);
        }
    int threadsX = (rw + 2) / 3, threadsY = (rh + 2) / 3;
    for (int round = 0; round < trials; ++round)
        for (int py = 0; py < 3; ++py)
            for (int px = 0; px < 3; ++px)
                for (int ty = 0; ty < threadsY; ++ty)
                    for (int tx = 0; tx < threadsX; ++tx) {
                        blockIdx.x = tx; blockIdx.y = ty; threadIdx.x = threadIdx.y = 0;
                        blockDim.x = blockDim.y = 1;
                        pd::dartPhaseKernel(gp, p, rg, px, py, roundBase + (unsigned)round);
                    }
}

// Sampler constructor arithmetic (poisson_disk.cu:119-125)
void ref_poisson_dims(float width, float height, float radius, float *cellSize, int *gridW, int *gridH)
{
    *cellSize = radius / sqrtf(2.0f);
    *gridW = (int)ceilf(width / *cellSize);
    *gridH = (int)ceilf(height / *cellSize);
}

} // extern "C"
