// Host runtime of the single-fit optimiser and the Poisson sampler behind the
// C ABI (include/vm_capi.h). Each function mirrors one method of the
// reference's VoroOptimizer / Sampler (src/voromesh/voro_optimizer.cu:512-858,
// src/poisson/poisson_disk.cu:119-199); the device work is the batch-native
// kernels of vm_step.cu / vm_extract.cu / vm_poisson.cu run on a batch of one.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "vm_capi.h"
#include "vm_device.cuh"
#include "vm_host.h"
#include "vm_kernels.h"

namespace vmh {

thread_local std::string g_lastError;

NvtxRange::NvtxRange(const char *name) { nvtxRangePushA(name); }
NvtxRange::~NvtxRange() { nvtxRangePop(); }

int fail(int code, const std::string &msg)
{
    g_lastError = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what)
{
    int code = e == cudaErrorMemoryAllocation ? VM_ERR_OOM
               : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? VM_ERR_NODEVICE
                                                                              : VM_ERR_CUDA;
    return fail(code, std::string(what) + ": " + cudaGetErrorString(e));
}

int floor_log2f(float h)
{
    int e = 0;
    std::frexp(h, &e);
    return e - 1;
}

// Watertightness and loop count of the boundary (reference
// voro_optimizer.cu:836-854) from its edges: watertight when every vertex
// has exactly one outgoing and one incoming edge; loops = cycles then.
void boundary_topology(MeshHost &mesh)
{
    size_t nv = mesh.vertices.size(), ne = mesh.edges.size() / 2;
    std::vector<int> nxt(nv, -1), inDeg(nv, 0);
    mesh.watertight = true;
    mesh.loops = 0;
    for (size_t e = 0; e < ne; ++e) {
        int a = mesh.edges[2 * e], b = mesh.edges[2 * e + 1];
        if (nxt[a] != -1) mesh.watertight = false;
        nxt[a] = b;
        ++inDeg[b];
    }
    for (size_t v = 0; v < nv; ++v)
        if (nxt[v] == -1 || inDeg[v] != 1) mesh.watertight = false;
    if (mesh.watertight) {
        std::vector<uint8_t> seen(nv, 0);
        for (size_t v = 0; v < nv; ++v) {
            if (seen[v]) continue;
            ++mesh.loops;
            for (int w = (int)v; !seen[w]; w = nxt[w]) seen[w] = 1;
        }
    }
}

} // namespace vmh

using namespace vmh;

// ===========================================================================
// optimiser handle
// ===========================================================================
struct vm_optimizer {
    float width = 0, height = 0, spacing = 0;
    vm_params params{};
    int gridW = 0, gridH = 0, cells = 0, tiles = 0;
    int slotsW = 0, slotsH = 0;
    float slotCellSize = 0;
    int targetCapacity = 0, liveTargets = 0;
    int iteration = 0, scheduleLength = 0;
    float lastBatchLoss = 0;
    bool gridValid = false;
    bool gridCanonical = false; // each cell's run sorted by slot (needed only when exported)
    int lossGrid = 0;
    int lossTile = 256;    // targets per loss tile (= its block size)
    int lossVariant = 3;   // loss kernel variant in use
    int lossForced = -1;   // variant chosen by the caller (vm_set_loss_variant), -1 = automatic
    bool tunePending = false; // the autotuner still has to pick the variant
    VmState *pinnedState = nullptr; // host staging of the state read after each Step

    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaGraphExec_t graph = nullptr;

    DevBuf<float2> gen, m, v, sortedPos, traw, tpos, stageVals, qbuf, cellVerts;
    DevBuf<long long> gradX;
    DevBuf<int> key, rank, counts, start, sortedIdx, tkey, trank, tslot, stageSlots, kIdx, cellEdges,
        cellCount, flags, dbgI0, dbgJ;
    DevBuf<float> kD2, dbgLoss;
    DevBuf<unsigned char> inside;
    DevBuf<unsigned long long> occ;
    DevBuf<VmState> state;
    DevBuf<VmFit> dFit;
    DevBuf<VmPointSet> dSites, dTargets, dCsrSet;
    DevBuf<int> cellStartD, csrLabels, dCsrPre; // extraction: cells packed in CSR order
    DevBuf<unsigned long long> tileState, ttileState, csrTileState; // scan tile words (vm_launch_scan)
    DevBuf<int> bndCnt, bndPartial, bndErr, bndMin, bndFirst, bndEdges; // boundary assembly
    DevBuf<unsigned long long> bndKeys;
    DevBuf<unsigned> bndSlot;
    DevBuf<float2> bndPt, bndVerts;
    DevBuf<float2> meshGen;          // the last Extract's generators
    DevBuf<unsigned char> meshInside; // and occupancy flags
    DevBuf<float2> csrVerts;
    DevBuf<int> dPre; // [0, siteBlocks, 0, tiles, 0, lossTiles, 0, targetBlocks]
    DevBuf<int> dTPre; // [0, targetBlocks, 0, targetKeyTiles]
    DevBuf<int> tcounts, tstart; // target sort by sub-cell (only while sorting)
    DevBuf<char> queue;  // deferred-target queue header
    DevBuf<int2> qitems; // its items
    std::vector<cudaEvent_t> timing; // vm_step_timed events
    int tilesX = 0, tilesY = 0;
    float invVoxel = 0;
    VmFit fit{};
    MeshHost mesh;
    long long exactTotal = 0;
    int block5Max = 0;          // most live targets in any 5x5 block of cells (sets the split shift)
    DevBuf<int> block5Buf;
    // the loss windows of a small fit (nWindows > 0): cell-aligned runs of at
    // most 32 targets (vm_launch_target_windows)
    int nWindows = 0;
    DevBuf<int> twin;
    DevBuf<int> winCounts, winStart; // the window counts and their scan
    DevBuf<unsigned long long> winState;
    DevBuf<VmPointSet> dWinSet;
    DevBuf<int> dWinPre;
    int winPre[2] = {0, 0}; // host copy of dWinPre (read by an async copy)

    int numSlots() const { return slotsW * slotsH; }
};

namespace {

// Loss tiles of the fit: targets per tile = the variant's block size, or with
// a window list block size / 32 windows per tile.
int loss_tiles(const vm_optimizer *h)
{
    if (h->nWindows > 0) {
        int nw = h->lossTile / 32;
        return (h->nWindows + nw - 1) / nw;
    }
    return (h->liveTargets + h->lossTile - 1) / h->lossTile;
}

int upload_tables(vm_optimizer *h)
{
    VmFit &F = h->fit;
    int n = h->numSlots();
    F.nSlots = n;
    F.slotsW = h->slotsW;
    F.slotsH = h->slotsH;
    F.gridW = h->gridW;
    F.gridH = h->gridH;
    F.cell = h->spacing;
    F.inv = 1.0f / h->spacing;
    F.width = h->width;
    F.height = h->height;
    F.K = h->params.lossK;
    F.fraction = h->params.sampleFraction;
    F.seed = h->params.seed;
    F.gradExp = 40 - floor_log2f(h->spacing);
    F.lossExp = 64 - 2 * floor_log2f(h->spacing);
    F.nTargets = h->liveTargets;
    F.active = 1;
    F.fastShift = vm_fast_shift(h->block5Max);
    F.twin = h->nWindows > 0 ? h->twin.p : nullptr;
    F.nWindows = h->nWindows;
    F.gen = h->gen.p; F.m = h->m.p; F.v = h->v.p; F.gradX = h->gradX.p;
    F.key = h->key.p; F.rank = h->rank.p; F.counts = h->counts.p; F.start = h->start.p; F.tileState = h->tileState.p;
    F.sortedIdx = h->sortedIdx.p; F.sortedPos = h->sortedPos.p;
    F.tpos = h->tpos.p; F.tslot = h->tslot.p;
    F.state = h->state.p;
    VmPointSet S{};
    S.pts = h->gen.p; S.n = n; S.gridW = h->gridW; S.gridH = h->gridH; S.inv = F.inv;
    S.key = h->key.p; S.rank = h->rank.p; S.counts = h->counts.p; S.start = h->start.p; S.tileState = h->tileState.p;
    S.outPos = h->sortedPos.p; S.outIdx = h->sortedIdx.p; S.canonical = 1; S.useIndexOrder = 1;
    int pre[8] = {0, (n + 255) / 256, 0, h->tiles, 0, loss_tiles(h), 0, (h->targetCapacity + 255) / 256};
    cudaError_t e;
    if ((e = cudaMemcpyAsync(h->dFit.p, &F, sizeof(VmFit), cudaMemcpyHostToDevice, h->stream))) return cuda_fail(e, "upload fit");
    if ((e = cudaMemcpyAsync(h->dSites.p, &S, sizeof(S), cudaMemcpyHostToDevice, h->stream))) return cuda_fail(e, "upload sites");
    if ((e = cudaMemcpyAsync(h->dPre.p, pre, sizeof(pre), cudaMemcpyHostToDevice, h->stream))) return cuda_fail(e, "upload prefix");
    // the tables live in pageable memory on the host: finish before they change
    if ((e = cudaStreamSynchronize(h->stream))) return cuda_fail(e, "upload sync");
    return VM_OK;
}

void drop_graph(vm_optimizer *h)
{
    if (h->graph) cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
}

void set_loss_variant(vm_optimizer *h, int v)
{
    h->lossVariant = v;
    h->lossTile = vm_loss_variant_threads(v);
    h->lossGrid = vm_loss_occupancy_blocks(v);
}

// Loss kernel variant: the caller's choice, else VM_LOSS_VARIANT, else the
// autotuner's choice for this fit size (made at the first step; until then
// 64-thread tiles for small fits and 256-thread tiles otherwise).
void choose_loss_variant(vm_optimizer *h, int sms)
{
    int v = h->lossForced;
    if (v < 0) {
        const char *env = std::getenv("VM_LOSS_VARIANT");
        if (env && *env) v = std::atoi(env);
    }
    h->tunePending = v < 0 || v >= vm_loss_variants();
    if (h->tunePending) v = h->liveTargets < 256 * 4 * sms ? 5 : 1;
    set_loss_variant(h, v);
}

// The autotuner: per device and power-of-two bucket of live targets, the loss
// variant with the shortest measured pass, kept for the process.
std::mutex g_tuneMu;
constexpr int kTuneDevices = 16;
int g_tuned[kTuneDevices][64]; // [device][bucket] -> variant, -1 = not yet timed
bool g_tunedInit = false;

int tune_bucket(int live)
{
    int b = 0;
    while (b < 62 && (2LL << b) <= live) ++b;
    return b;
}

int read_state(vm_optimizer *h, VmState &st);

// Times every variant on this fit (5 loss passes each, after one untimed
// pass, in two sweeps) and keeps the fastest. The passes leave the generators and moments
// alone; the gradient accumulators and the state are restored afterwards.
int autotune_loss_variant(vm_optimizer *h)
{
    h->tunePending = false;
    int bucket = tune_bucket(h->liveTargets);
    int dev = 0;
    cudaGetDevice(&dev);
    dev = std::min(std::max(dev, 0), kTuneDevices - 1); // devices past the table share its last row
    {
        std::lock_guard<std::mutex> lk(g_tuneMu);
        if (!g_tunedInit) {
            for (auto &row : g_tuned)
                for (int &t : row) t = -1;
            g_tunedInit = true;
        }
        if (g_tuned[dev][bucket] >= 0) {
            set_loss_variant(h, g_tuned[dev][bucket]);
            return upload_tables(h);
        }
    }
    VmState saved;
    int rc;
    if ((rc = read_state(h, saved))) return rc;
    int nv = vm_loss_variants();
    std::vector<float> score(nv, 1e30f);
    cudaError_t e;
    for (int round = 0; round < 2; ++round) // the better of two sweeps, against noise and warm-up
        for (int v = 0; v < nv; ++v) {
            set_loss_variant(h, v);
            if ((rc = upload_tables(h))) return rc;
            int lossTiles = loss_tiles(h);
            float ms = 0.0f;
            for (int k = 0; k < 6; ++k) {
                if (k == 1 && (e = cudaEventRecord(h->ev0, h->stream))) return cuda_fail(e, "tune event");
                if ((e = vm_launch_loss(h->dFit.p, h->dPre.p + 4, 1, lossTiles, 0, h->lossGrid, v, h->nWindows > 0,
                                        h->queue.p,
                                        h->stream)) ||
                    (e = vm_launch_finalize(h->dFit.p, 1, h->queue.p, h->stream)))
                    return cuda_fail(e, "tune pass");
            }
            if ((e = cudaEventRecord(h->ev1, h->stream)) || (e = cudaEventSynchronize(h->ev1)) ||
                (e = cudaEventElapsedTime(&ms, h->ev0, h->ev1)))
                return cuda_fail(e, "tune timing");
            score[v] = std::min(score[v], ms);
        }
    int best = (int)(std::min_element(score.begin(), score.end()) - score.begin());
    if ((e = cudaMemsetAsync(h->gradX.p, 0, sizeof(long long) * kGradWords * (size_t)h->numSlots(), h->stream)) ||
        (e = cudaMemcpyAsync(h->state.p, &saved, sizeof(VmState), cudaMemcpyHostToDevice, h->stream)) ||
        (e = cudaStreamSynchronize(h->stream)))
        return cuda_fail(e, "tune restore");
    {
        std::lock_guard<std::mutex> lk(g_tuneMu);
        g_tuned[dev][bucket] = best;
    }
    set_loss_variant(h, best);
    return upload_tables(h);
}

int enqueue_build_grid(vm_optimizer *h)
{
    int n = h->numSlots();
    cudaError_t e;
    if ((e = vm_launch_bin(h->dSites.p, h->dPre.p + 0, 1, (n + 255) / 256, 1, h->stream))) return cuda_fail(e, "bin");
    if ((e = vm_launch_scan(h->dSites.p, h->dPre.p + 2, 1, h->tiles, h->stream))) return cuda_fail(e, "scan");
    if ((e = vm_launch_scatter(h->dSites.p, h->dPre.p + 0, 1, (n + 255) / 256, nullptr, h->stream)))
        return cuda_fail(e, "scatter");
    h->gridCanonical = false;
    return VM_OK;
}

int ensure_grid(vm_optimizer *h)
{
    if (h->gridValid) return VM_OK;
    int rc = enqueue_build_grid(h);
    if (rc) return rc;
    h->gridValid = true;
    return VM_OK;
}

int enqueue_step(vm_optimizer *h)
{
    int n = h->numSlots();
    cudaError_t e;
    int lossTiles = loss_tiles(h);
    if (vm_small_grid_fits(n, h->cells)) {
        // the loss fast path, then the rest of the step in one block
        if ((e = vm_launch_loss_fast(h->dFit.p, h->dPre.p + 4, 1, lossTiles, h->lossGrid, h->lossVariant,
                                     h->nWindows > 0, h->queue.p, h->stream)) ||
            (e = vm_launch_small_grid(h->dFit.p, h->queue.p, h->stream)))
            return cuda_fail(e, "small step");
        return VM_OK;
    }
    if ((e = vm_launch_loss(h->dFit.p, h->dPre.p + 4, 1, lossTiles, 0, h->lossGrid, h->lossVariant, h->nWindows > 0,
                            h->queue.p, h->stream)))
        return cuda_fail(e, "loss");
    if ((e = vm_launch_adam_bin(h->dFit.p, h->dPre.p + 0, 1, (n + 255) / 256, h->queue.p, h->stream)))
        return cuda_fail(e, "adam");
    if ((e = vm_launch_scan(h->dSites.p, h->dPre.p + 2, 1, h->tiles, h->stream))) return cuda_fail(e, "scan");
    if ((e = vm_launch_scatter(h->dSites.p, h->dPre.p + 0, 1, (n + 255) / 256, h->dFit.p, h->stream)))
        return cuda_fail(e, "scatter");
    return VM_OK;
}

int ensure_graph(vm_optimizer *h)
{
    if (h->graph) return VM_OK;
    cudaGraph_t g;
    cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
    if (e) return cuda_fail(e, "begin capture");
    int rc = enqueue_step(h);
    e = cudaStreamEndCapture(h->stream, &g);
    if (e) return rc ? rc : cuda_fail(e, "end capture");
    if (rc) {
        cudaGraphDestroy(g);
        return rc;
    }
    e = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (e) return cuda_fail(e, "graph instantiate");
    return VM_OK;
}

// Error bits a kernel raised in the fit's state (VM_KERR_*), as a status.
int kernel_status(int bits)
{
    if (!bits) return VM_OK;
    return fail(VM_ERR_CUDA, std::string("kernel error bits 0x") + std::to_string(bits) +
                                 ((bits & VM_KERR_CAPACITY) ? " (deferred-target queue full)" : ""));
}

int read_state(vm_optimizer *h, VmState &st)
{
    // through a pinned staging copy: one direct DMA per Step
    VmState *dst = h->pinnedState ? h->pinnedState : &st;
    cudaError_t e = cudaMemcpyAsync(dst, h->state.p, sizeof(VmState), cudaMemcpyDeviceToHost, h->stream);
    if (!e) e = cudaStreamSynchronize(h->stream);
    if (e) return cuda_fail(e, "read state");
    if (dst != &st) st = *dst;
    return VM_OK;
}

// log2 of the sub-cells per cell side in the target order: 4x4 sub-cells keep
// each warp's 32 targets in a small box (tight distance bounds in the loss),
// within 2^27 sort keys. VM_TARGET_SUB overrides it (0-3).
int target_sub(const vm_optimizer *h)
{
    int sub = 2;
    const char *env = std::getenv("VM_TARGET_SUB");
    if (env && *env) sub = std::min(std::max(std::atoi(env), 0), 3);
    while (sub > 0 && ((long long)h->cells << (2 * sub)) > (1LL << 27)) --sub;
    return sub;
}

// A fit with fewer live targets than this is latency-bound: its loss pass
// lasts as long as its slowest warp, so it gets cell-aligned windows (one grid
// cell per warp iteration, instead of up to three for 32 consecutive targets).
// Larger fits are throughput-bound and keep windows of 32 targets, which
// need fewer iterations.
constexpr int kWindowedTargets = 1 << 19;

// Enqueues the loss windows of the sorted targets (vm_launch_target_windows)
// for at most `live` live targets, from the target sort's key starts
// (h->tstart); their number lands in *nWin once the stream has reached it.
int enqueue_windows(vm_optimizer *h, int sub, int live, int *nWin)
{
    int cells = h->cells, tiles = (cells + kScanTile - 1) / kScanTile;
    int rc;
    if ((rc = h->winCounts.reserve((size_t)cells + 1)) || (rc = h->winStart.reserve((size_t)cells + 1)) ||
        (rc = zeroed_tile_state(h->winState, tiles, h->stream)) ||
        (rc = h->twin.reserve((size_t)live / 32 + std::min(cells, live) + 1)) || (rc = h->dWinSet.reserve(1)) ||
        (rc = h->dWinPre.reserve(2)))
        return rc;
    VmPointSet W{};
    W.gridW = cells;
    W.gridH = 1;
    W.counts = h->winCounts.p;
    W.start = h->winStart.p;
    W.tileState = h->winState.p;
    h->winPre[0] = 0;
    h->winPre[1] = tiles;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(h->dWinSet.p, &W, sizeof(W), cudaMemcpyHostToDevice, h->stream)) ||
        (e = cudaMemcpyAsync(h->dWinPre.p, h->winPre, sizeof(h->winPre), cudaMemcpyHostToDevice, h->stream)) ||
        (e = vm_launch_target_windows(h->tstart.p, cells, sub, h->dWinSet.p, h->dWinPre.p, tiles, h->winCounts.p,
                                      h->winStart.p, h->twin.p, h->stream)) ||
        (e = cudaMemcpyAsync(nWin, h->winStart.p + cells, sizeof(int), cudaMemcpyDeviceToHost, h->stream)))
        return cuda_fail(e, "loss windows");
    return VM_OK;
}

// Targets in (cell, sub-cell) order, the order the loss pass walks them. The
// key arrays exist only during the sort.
int sort_targets(vm_optimizer *h)
{
    cudaError_t e;
    int rc;
    int sub = target_sub(h);
    long long keys = (long long)h->cells << (2 * sub);
    int keyTiles = (int)((keys + kScanTile - 1) / kScanTile);
    int tb = (h->targetCapacity + 255) / 256;
    if ((rc = h->tcounts.alloc(keys + 1)) || (rc = h->tstart.alloc(keys + 1)) ||
        (rc = zeroed_tile_state(h->ttileState, keyTiles, h->stream)))
        return rc;
    VmPointSet T{};
    T.pts = h->traw.p; T.n = h->targetCapacity; T.gridW = h->gridW; T.gridH = h->gridH; T.inv = 1.0f / h->spacing;
    T.key = h->tkey.p; T.rank = h->trank.p; T.counts = h->tcounts.p; T.start = h->tstart.p;
    T.tileState = h->ttileState.p; T.outPos = h->tpos.p; T.outIdx = h->tslot.p; T.canonical = 0; T.useIndexOrder = 1;
    T.sub = sub;
    int pre[4] = {0, tb, 0, keyTiles};
    if ((e = cudaMemsetAsync(h->tcounts.p, 0, sizeof(int) * (size_t)(keys + 1), h->stream)) ||
        (e = cudaMemcpyAsync(h->dTargets.p, &T, sizeof(T), cudaMemcpyHostToDevice, h->stream)) ||
        (e = cudaMemcpyAsync(h->dTPre.p, pre, sizeof(pre), cudaMemcpyHostToDevice, h->stream)))
        return cuda_fail(e, "target sort tables");
    if ((e = vm_launch_bin(h->dTargets.p, h->dTPre.p, 1, tb, 0, h->stream))) return cuda_fail(e, "target bin");
    if ((e = vm_launch_scan(h->dTargets.p, h->dTPre.p + 2, 1, keyTiles, h->stream))) return cuda_fail(e, "target scan");
    if ((e = vm_launch_scatter(h->dTargets.p, h->dTPre.p, 1, tb, nullptr, h->stream)))
        return cuda_fail(e, "target scatter");
    int live = 0, b5 = 0;
    if ((rc = h->block5Buf.reserve(1))) return rc;
    if ((e = vm_launch_block5_max(h->tstart.p, h->gridW, h->gridH, sub, h->block5Buf.p, h->stream)))
        return cuda_fail(e, "target block counts");
    if ((e = cudaMemcpyAsync(&live, h->tstart.p + keys, sizeof(int), cudaMemcpyDeviceToHost, h->stream)) ||
        (e = cudaMemcpyAsync(&b5, h->block5Buf.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream)))
        return cuda_fail(e, "live targets");
    // a small fit's loss windows, in the same pass when every target slot
    // would still make it a small fit
    int nWin = 0;
    bool windowsQueued = h->targetCapacity < kWindowedTargets;
    if (windowsQueued && (rc = enqueue_windows(h, sub, h->targetCapacity, &nWin))) return rc;
    // the tables above live on the host stack
    if ((e = cudaStreamSynchronize(h->stream))) return cuda_fail(e, "target sort");
    if (live > 0 && live < kWindowedTargets && !windowsQueued) {
        if ((rc = enqueue_windows(h, sub, live, &nWin))) return rc;
        if ((e = cudaStreamSynchronize(h->stream))) return cuda_fail(e, "loss windows");
    }
    if (!(live > 0 && live < kWindowedTargets)) nWin = 0;
    h->tcounts.release();
    h->tstart.release();
    h->ttileState.release();
    if (live != h->liveTargets || nWin != h->nWindows) drop_graph(h);
    h->liveTargets = live;
    h->nWindows = nWin;
    h->block5Max = b5;
    int qcap = std::max(live, 1); // every live target fits: the loss never overflows the queue
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    choose_loss_variant(h, sms);
    if ((rc = h->qitems.reserve(qcap))) return rc;
    if ((e = vm_queue_init(h->queue.p, h->qitems.p, qcap, h->stream))) return cuda_fail(e, "queue");
    return upload_tables(h);
}

} // namespace

extern "C" {

const char *vm_error_string(int code)
{
    switch (code) {
    case VM_OK: return "ok";
    case VM_ERR_ARG: return "invalid argument";
    case VM_ERR_OOM: return "out of memory";
    case VM_ERR_CUDA: return "CUDA error";
    case VM_ERR_STATE: return "invalid state";
    case VM_ERR_BUDGET: return "over memory budget";
    case VM_ERR_TIMEOUT: return "timeout";
    case VM_ERR_UNSUPPORTED: return "unsupported parameter";
    case VM_ERR_NODEVICE: return "no CUDA device";
    default: return "unknown error";
    }
}

int vm_last_error(char *buf, int len)
{
    if (!buf || len <= 0) return VM_ERR_ARG;
    std::snprintf(buf, (size_t)len, "%s", g_lastError.c_str());
    return VM_OK;
}

int vm_version(int *major, int *minor, int *sm)
{
    if (major) *major = 1;
    if (minor) *minor = 0;
    if (sm) *sm = 103;
    return VM_OK;
}

void vm_params_default(vm_params *p)
{
    if (!p) return;
    p->iterations = 400;
    p->localIterations = 100;
    p->lrPerSpacing = 0.09f;
    p->sampleFraction = 0.2f;
    p->gamma = 0.5f;
    p->milestones[0] = 80;
    p->milestones[1] = 150;
    p->milestones[2] = 200;
    p->milestones[3] = 250;
    p->seed = 1;
    p->lossK = 12;
}

int vm_create(float width, float height, float spacing, const vm_params *params, vm_optimizer **out)
{
    if (!out) return fail(VM_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (!(width > 0.0f) || !(height > 0.0f) || !(spacing > 0.0f)) return fail(VM_ERR_ARG, "width, height and spacing must be > 0");
    vm_params p;
    vm_params_default(&p);
    if (params) p = *params;
    if (p.lossK != 8 && p.lossK != 12 && p.lossK != 16 && p.lossK != 24 && p.lossK != 32)
        return fail(VM_ERR_UNSUPPORTED, "lossK must be 8, 12, 16, 24 or 32");
    // hash grid: ceil(w / spacing) x ceil(h / spacing) (reference voro_optimizer.cu:520-521)
    double gw = std::ceil(width / spacing), gh = std::ceil(height / spacing);
    if (gw * gh > 1.5e9) return fail(VM_ERR_ARG, "hash grid too large");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return cuda_fail(e, "cudaGetDevice");
    vm_optimizer *h = new vm_optimizer();
    h->width = width;
    h->height = height;
    h->spacing = spacing;
    h->params = p;
    h->gridW = std::max(1, (int)std::ceil(width / spacing));
    h->gridH = std::max(1, (int)std::ceil(height / spacing));
    h->cells = h->gridW * h->gridH;
    h->tiles = (h->cells + kScanTile - 1) / kScanTile;
    int rc = VM_OK;
    if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) || (e = cudaEventCreate(&h->ev0)) ||
        (e = cudaEventCreate(&h->ev1)))
        rc = cuda_fail(e, "stream/event");
    if (!rc) rc = h->counts.alloc(h->cells + 1);
    if (!rc) rc = h->start.alloc(h->cells + 1);
    if (!rc) rc = zeroed_tile_state(h->tileState, h->tiles, h->stream);
    if (!rc) rc = h->state.alloc(1);
    if (!rc) rc = h->dFit.alloc(1);
    if (!rc) rc = h->dSites.alloc(1);
    if (!rc) rc = h->dTargets.alloc(1);
    if (!rc) rc = h->dPre.alloc(8);
    if (!rc) rc = h->dTPre.alloc(4);
    if (!rc) rc = h->flags.alloc(2);
    if (!rc) rc = h->queue.alloc(vm_queue_bytes());
    if (!rc && (e = vm_queue_init(h->queue.p, nullptr, 0, h->stream))) rc = cuda_fail(e, "queue");
    if (!rc && (e = cudaMemset(h->counts.p, 0, sizeof(int) * (h->cells + 1)))) rc = cuda_fail(e, "memset");
    if (!rc && (e = cudaMemset(h->state.p, 0, sizeof(VmState)))) rc = cuda_fail(e, "memset");
    if (!rc && cudaMallocHost((void **)&h->pinnedState, sizeof(VmState)) != cudaSuccess) {
        h->pinnedState = nullptr; // pageable reads still work
        cudaGetLastError();
    }
    if (!rc) h->lossGrid = vm_loss_occupancy_blocks(h->lossVariant);
    if (!rc) rc = upload_tables(h);
    if (rc) {
        vm_destroy(h);
        return rc;
    }
    *out = h;
    return VM_OK;
}

int vm_destroy(vm_optimizer *h)
{
    if (!h) return VM_OK;
    drop_graph(h);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    for (cudaEvent_t ev : h->timing) cudaEventDestroy(ev);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->pinnedState) cudaFreeHost(h->pinnedState);
    delete h; // DevBuf members free their memory
    return VM_OK;
}

static int set_targets_from(vm_optimizer *h, const void *xy, int n, cudaMemcpyKind kind)
{
    int cap = std::max(n, 1);
    int rc;
    if (cap != h->targetCapacity) {
        drop_graph(h);
        h->targetCapacity = cap;
        if ((rc = h->traw.alloc(cap)) || (rc = h->tkey.alloc(cap)) || (rc = h->trank.alloc(cap)) ||
            (rc = h->tpos.alloc(cap)) || (rc = h->tslot.alloc(cap)))
            return rc;
    }
    cudaError_t e;
    // NaN padding fails every x >= 0 test (reference voro_optimizer.cu:558)
    if ((e = cudaMemsetAsync(h->traw.p, 0xFF, sizeof(float2) * cap, h->stream))) return cuda_fail(e, "memset targets");
    if (n > 0 && (e = cudaMemcpyAsync(h->traw.p, xy, sizeof(float2) * (size_t)n, kind, h->stream)))
        return cuda_fail(e, "upload targets");
    if ((rc = upload_tables(h))) return rc;
    return sort_targets(h);
}

int vm_set_targets(vm_optimizer *h, const float *xy, int n)
{
    vmh::NvtxRange range("vm_set_targets");
    if (!h || n < 0 || (n > 0 && !xy)) return fail(VM_ERR_ARG, "vm_set_targets: bad arguments");
    return set_targets_from(h, xy, n, cudaMemcpyHostToDevice);
}

int vm_update_targets(vm_optimizer *h, const int *dirty, int ndirty, const float *slots, int nslots)
{
    vmh::NvtxRange range("vm_update_targets");
    if (!h || ndirty < 0 || nslots < 0) return fail(VM_ERR_ARG, "vm_update_targets: bad arguments");
    if (ndirty == 0) return VM_OK;
    if (!dirty || !slots) return fail(VM_ERR_ARG, "vm_update_targets: NULL buffer");
    if (nslots > h->targetCapacity) {
        // grow with slack and re-upload everything (reference :566-571)
        size_t cap = std::max((size_t)nslots * 3 / 2, (size_t)nslots + 64);
        std::vector<float> padded(2 * cap, -1.0f);
        std::memcpy(padded.data(), slots, sizeof(float) * 2 * (size_t)nslots);
        return vm_set_targets(h, padded.data(), (int)cap);
    }
    std::vector<float2> values((size_t)ndirty);
    for (int k = 0; k < ndirty; ++k) {
        int s = dirty[k];
        if (s < 0 || s >= nslots) return fail(VM_ERR_ARG, "vm_update_targets: dirty slot out of range");
        values[k] = make_float2(slots[2 * (size_t)s], slots[2 * (size_t)s + 1]);
    }
    int rc;
    if ((rc = h->stageSlots.reserve(ndirty)) || (rc = h->stageVals.reserve(ndirty))) return rc;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(h->stageSlots.p, dirty, sizeof(int) * ndirty, cudaMemcpyHostToDevice, h->stream)) ||
        (e = cudaMemcpyAsync(h->stageVals.p, values.data(), sizeof(float2) * ndirty, cudaMemcpyHostToDevice,
                             h->stream)) ||
        (e = vm_launch_scatter_targets(h->traw.p, h->stageSlots.p, h->stageVals.p, ndirty, h->stream)))
        return cuda_fail(e, "update targets");
    return sort_targets(h);
}

int vm_set_occupancy(vm_optimizer *h, const uint64_t *masks, int tilesX, int tilesY, float voxelSize)
{
    if (!h || tilesX < 0 || tilesY < 0 || !(voxelSize > 0.0f)) return fail(VM_ERR_ARG, "vm_set_occupancy: bad arguments");
    size_t n = (size_t)tilesX * tilesY;
    if (n && !masks) return fail(VM_ERR_ARG, "vm_set_occupancy: NULL masks");
    int rc;
    if (tilesX != h->tilesX || tilesY != h->tilesY) {
        h->tilesX = tilesX;
        h->tilesY = tilesY;
        if ((rc = h->occ.alloc(n))) return rc;
    }
    h->invVoxel = 1.0f / voxelSize;
    cudaError_t e;
    if (n && (e = cudaMemcpyAsync(h->occ.p, masks, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, h->stream)))
        return cuda_fail(e, "upload occupancy");
    if ((e = cudaStreamSynchronize(h->stream))) return cuda_fail(e, "occupancy");
    return VM_OK;
}

int vm_update_occupancy(vm_optimizer *h, const uint64_t *masks, int tx0, int ty0, int tx1, int ty1)
{
    if (!h) return fail(VM_ERR_ARG, "NULL handle");
    tx0 = std::max(tx0, 0), ty0 = std::max(ty0, 0);
    tx1 = std::min(tx1, h->tilesX), ty1 = std::min(ty1, h->tilesY);
    if (tx0 >= tx1 || ty0 >= ty1) return VM_OK;
    if (!masks) return fail(VM_ERR_ARG, "NULL masks");
    size_t pitch = (size_t)h->tilesX * sizeof(uint64_t);
    size_t off = (size_t)ty0 * h->tilesX + tx0;
    cudaError_t e = cudaMemcpy2DAsync(h->occ.p + off, pitch, masks + off, pitch, (tx1 - tx0) * sizeof(uint64_t),
                                      ty1 - ty0, cudaMemcpyHostToDevice, h->stream);
    if (!e) e = cudaStreamSynchronize(h->stream);
    if (e) return cuda_fail(e, "update occupancy");
    return VM_OK;
}

int vm_set_generators(vm_optimizer *h, const float *xy, int slotsW, int slotsH, float slotCellSize)
{
    vmh::NvtxRange range("vm_set_generators");
    if (!h || slotsW < 0 || slotsH < 0) return fail(VM_ERR_ARG, "vm_set_generators: bad arguments");
    long long n64 = (long long)slotsW * slotsH;
    if (n64 > 0x7FFFFFFF / kMaxCellVerts) return fail(VM_ERR_ARG, "too many generator slots");
    int n = (int)n64;
    if (n > 0 && !xy) return fail(VM_ERR_ARG, "vm_set_generators: NULL slots");
    int rc;
    if (slotsW != h->slotsW || slotsH != h->slotsH) {
        drop_graph(h);
        h->slotsW = slotsW;
        h->slotsH = slotsH;
        if ((rc = h->gen.alloc(n)) || (rc = h->m.alloc(n)) || (rc = h->v.alloc(n)) || (rc = h->gradX.alloc(kGradWords * (size_t)n)) ||
            (rc = h->key.alloc(n)) || (rc = h->rank.alloc(n)) || (rc = h->sortedIdx.alloc(n)) ||
            (rc = h->sortedPos.alloc(n)))
            return rc;
        h->cellVerts.release();
        h->cellEdges.release();
        h->cellCount.release();
        h->inside.release();
    }
    h->slotCellSize = slotCellSize;
    cudaError_t e;
    if (n > 0) {
        if ((e = cudaMemcpyAsync(h->gen.p, xy, sizeof(float2) * (size_t)n, cudaMemcpyHostToDevice, h->stream)) ||
            (e = cudaMemsetAsync(h->gradX.p, 0, sizeof(long long) * kGradWords * (size_t)n, h->stream)))
            return cuda_fail(e, "upload generators");
    }
    h->gridValid = false;
    if ((rc = upload_tables(h))) return rc;
    return vm_begin_schedule(h, h->params.iterations, 0, 0, h->slotsW, h->slotsH);
}

int vm_update_generators(vm_optimizer *h, const float *xy, int cx0, int cy0, int cx1, int cy1)
{
    if (!h) return fail(VM_ERR_ARG, "NULL handle");
    cx0 = std::max(cx0, 0), cy0 = std::max(cy0, 0);
    cx1 = std::min(cx1, h->slotsW), cy1 = std::min(cy1, h->slotsH);
    if (cx0 >= cx1 || cy0 >= cy1) return VM_OK;
    if (!xy) return fail(VM_ERR_ARG, "NULL slots");
    size_t pitch = (size_t)h->slotsW * sizeof(float2);
    size_t off = (size_t)cy0 * h->slotsW + cx0;
    cudaError_t e = cudaMemcpy2DAsync(h->gen.p + off, pitch, reinterpret_cast<const float2 *>(xy) + off, pitch,
                                      (cx1 - cx0) * sizeof(float2), cy1 - cy0, cudaMemcpyHostToDevice, h->stream);
    if (!e) e = cudaStreamSynchronize(h->stream);
    if (e) return cuda_fail(e, "update generators");
    h->gridValid = false;
    return VM_OK;
}

int vm_begin_schedule(vm_optimizer *h, int iterations, int cx0, int cy0, int cx1, int cy1)
{
    vmh::NvtxRange range("vm_begin_schedule");
    if (!h) return fail(VM_ERR_ARG, "NULL handle");
    cx0 = std::max(cx0, 0), cy0 = std::max(cy0, 0);
    cx1 = std::min(cx1, h->slotsW), cy1 = std::min(cy1, h->slotsH);
    VmFit &F = h->fit;
    // RunParams (reference voro_optimizer.cu:658-675)
    F.lr = h->params.lrPerSpacing * h->spacing;
    F.gamma = h->params.gamma;
    F.beta1 = 0.9f;
    F.beta2 = 0.999f;
    F.eps = 1e-8f;
    for (int k = 0; k < 4; ++k)
        F.milestones[k] = h->params.iterations != 0
                              ? (int)std::lround(double(h->params.milestones[k]) * iterations / h->params.iterations)
                              : h->params.milestones[k];
    F.cx0 = cx0; F.cy0 = cy0; F.cx1 = cx1; F.cy1 = cy1;
    float margin = 2.0f * h->spacing;
    F.bx0 = (float)cx0 * h->slotCellSize - margin;
    F.by0 = (float)cy0 * h->slotCellSize - margin;
    F.bx1 = (float)cx1 * h->slotCellSize + margin;
    F.by1 = (float)cy1 * h->slotCellSize + margin;
    cudaError_t e;
    if (cx0 < cx1 && cy0 < cy1) {
        size_t pitch = (size_t)h->slotsW * sizeof(float2);
        size_t off = (size_t)cy0 * h->slotsW + cx0;
        if ((e = cudaMemset2DAsync(h->m.p + off, pitch, 0, (cx1 - cx0) * sizeof(float2), cy1 - cy0, h->stream)) ||
            (e = cudaMemset2DAsync(h->v.p + off, pitch, 0, (cx1 - cx0) * sizeof(float2), cy1 - cy0, h->stream)))
            return cuda_fail(e, "reset moments");
    }
    if ((e = cudaMemsetAsync(h->state.p, 0, sizeof(VmState), h->stream))) return cuda_fail(e, "reset state");
    h->scheduleLength = iterations;
    h->iteration = 0;
    h->lastBatchLoss = 0.0f;
    return upload_tables(h);
}

int vm_step(vm_optimizer *h, int iterations, float *gpuMs)
{
    vmh::NvtxRange range("vm_step");
    if (!h) return fail(VM_ERR_ARG, "NULL handle");
    if (gpuMs) *gpuMs = 0.0f;
    if (iterations <= 0 || h->numSlots() == 0 || h->targetCapacity == 0) return VM_OK;
    int rc;
    if ((rc = ensure_grid(h))) return rc;
    if (h->tunePending) {
        drop_graph(h);
        if ((rc = autotune_loss_variant(h))) return rc;
    }
    if ((rc = ensure_graph(h))) return rc;
    cudaError_t e;
    if ((e = cudaEventRecord(h->ev0, h->stream))) return cuda_fail(e, "event");
    h->gridCanonical = false; // the steps rebuild the grid
    for (int k = 0; k < iterations; ++k)
        if ((e = cudaGraphLaunch(h->graph, h->stream))) return cuda_fail(e, "graph launch");
    if ((e = cudaEventRecord(h->ev1, h->stream))) return cuda_fail(e, "event");
    VmState st;
    if ((rc = read_state(h, st)) || (rc = kernel_status(st.errors))) return rc;
    h->iteration = st.iter;
    h->lastBatchLoss = st.count > 0 ? st.loss / (float)st.count : 0.0f;
    h->exactTotal = st.slowTotal;
    float ms = 0.0f;
    if ((e = cudaEventElapsedTime(&ms, h->ev0, h->ev1))) return cuda_fail(e, "elapsed");
    if (gpuMs) *gpuMs = ms;
    return VM_OK;
}

int vm_step_timed(vm_optimizer *h, int iterations, float *stageMs)
{
    vmh::NvtxRange range("vm_step_timed");
    if (!h || !stageMs || iterations < 0) return fail(VM_ERR_ARG, "bad arguments");
    for (int k = 0; k < 4; ++k) stageMs[k] = 0.0f;
    if (iterations == 0 || h->numSlots() == 0 || h->targetCapacity == 0) return VM_OK;
    int rc;
    if ((rc = ensure_grid(h))) return rc;
    size_t need = (size_t)iterations * 5;
    cudaError_t e;
    while (h->timing.size() < need) {
        cudaEvent_t ev;
        if ((e = cudaEventCreate(&ev))) return cuda_fail(e, "event");
        h->timing.push_back(ev);
    }
    int n = h->numSlots();
    int lossTiles = loss_tiles(h);
    h->gridCanonical = false; // the steps rebuild the grid
    for (int k = 0; k < iterations; ++k) {
        cudaEvent_t *ev = &h->timing[(size_t)k * 5];
        if ((e = cudaEventRecord(ev[0], h->stream)) ||
            (e = vm_launch_loss(h->dFit.p, h->dPre.p + 4, 1, lossTiles, 0, h->lossGrid, h->lossVariant,
                                h->nWindows > 0, h->queue.p, h->stream)) ||
            (e = cudaEventRecord(ev[1], h->stream)) ||
            (e = vm_launch_adam_bin(h->dFit.p, h->dPre.p + 0, 1, (n + 255) / 256, h->queue.p, h->stream)) ||
            (e = cudaEventRecord(ev[2], h->stream)) ||
            (e = vm_launch_scan(h->dSites.p, h->dPre.p + 2, 1, h->tiles, h->stream)) ||
            (e = cudaEventRecord(ev[3], h->stream)) ||
            (e = vm_launch_scatter(h->dSites.p, h->dPre.p + 0, 1, (n + 255) / 256, h->dFit.p, h->stream)) ||
            (e = cudaEventRecord(ev[4], h->stream)))
            return cuda_fail(e, "timed step");
    }
    VmState st;
    if ((rc = read_state(h, st)) || (rc = kernel_status(st.errors))) return rc;
    h->iteration = st.iter;
    h->lastBatchLoss = st.count > 0 ? st.loss / (float)st.count : 0.0f;
    h->exactTotal = st.slowTotal;
    for (int k = 0; k < iterations; ++k) {
        cudaEvent_t *ev = &h->timing[(size_t)k * 5];
        for (int j = 0; j < 4; ++j) {
            float ms = 0.0f;
            if ((e = cudaEventElapsedTime(&ms, ev[j], ev[j + 1]))) return cuda_fail(e, "elapsed");
            stageMs[j] += ms / iterations;
        }
    }
    return VM_OK;
}

int vm_set_loss_variant(vm_optimizer *h, int variant)
{
    if (!h || variant < -1 || variant >= vm_loss_variants()) return fail(VM_ERR_ARG, "bad loss variant");
    h->lossForced = variant;
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    choose_loss_variant(h, sms);
    drop_graph(h);
    return upload_tables(h);
}

int vm_get_loss_variant(vm_optimizer *h, int *variant, int *count)
{
    if (!h) return fail(VM_ERR_ARG, "NULL handle");
    if (variant) *variant = h->lossVariant;
    if (count) *count = vm_loss_variants();
    return VM_OK;
}

int vm_evaluate_loss(vm_optimizer *h, float *loss)
{
    vmh::NvtxRange range("vm_evaluate_loss");
    if (!h || !loss) return fail(VM_ERR_ARG, "bad arguments");
    *loss = 0.0f;
    if (h->numSlots() == 0 || h->targetCapacity == 0) return VM_OK;
    int rc;
    if ((rc = ensure_grid(h))) return rc;
    cudaError_t e;
    int lossTiles = loss_tiles(h);
    if ((e = vm_launch_loss(h->dFit.p, h->dPre.p + 4, 1, lossTiles, 1, h->lossGrid, h->lossVariant, h->nWindows > 0,
                            h->queue.p, h->stream)) ||
        (e = vm_launch_finalize(h->dFit.p, 1, h->queue.p, h->stream)))
        return cuda_fail(e, "evaluate loss");
    VmState st;
    if ((rc = read_state(h, st)) || (rc = kernel_status(st.errors))) return rc;
    *loss = st.count > 0 ? st.loss / (float)st.count : 0.0f;
    return VM_OK;
}

int vm_info(vm_optimizer *h, vm_info_t *out)
{
    if (!h || !out) return fail(VM_ERR_ARG, "bad arguments");
    out->iteration = h->iteration;
    out->scheduleLength = h->scheduleLength;
    out->numSlots = h->numSlots();
    out->targetCapacity = h->targetCapacity;
    out->liveTargets = h->liveTargets;
    out->gridW = h->gridW;
    out->gridH = h->gridH;
    out->lastBatchLoss = h->lastBatchLoss;
    out->exactTargets = h->exactTotal;
    return VM_OK;
}

int vm_get_generators(vm_optimizer *h, float *xy)
{
    if (!h || !xy) return fail(VM_ERR_ARG, "bad arguments");
    int n = h->numSlots();
    if (!n) return VM_OK;
    cudaError_t e = cudaMemcpyAsync(xy, h->gen.p, sizeof(float2) * (size_t)n, cudaMemcpyDeviceToHost, h->stream);
    if (!e) e = cudaStreamSynchronize(h->stream);
    if (e) return cuda_fail(e, "read generators");
    return VM_OK;
}

int vm_get_moments(vm_optimizer *h, float *m, float *v)
{
    if (!h) return fail(VM_ERR_ARG, "NULL handle");
    int n = h->numSlots();
    cudaError_t e = cudaSuccess;
    if (n && m) e = cudaMemcpyAsync(m, h->m.p, sizeof(float2) * (size_t)n, cudaMemcpyDeviceToHost, h->stream);
    if (!e && n && v) e = cudaMemcpyAsync(v, h->v.p, sizeof(float2) * (size_t)n, cudaMemcpyDeviceToHost, h->stream);
    if (!e) e = cudaStreamSynchronize(h->stream);
    if (e) return cuda_fail(e, "read moments");
    return VM_OK;
}

int vm_get_grid(vm_optimizer *h, int *start, int *sortedIdx, float *sortedPos, int *genCell)
{
    if (!h) return fail(VM_ERR_ARG, "NULL handle");
    int rc;
    if (h->numSlots() == 0) return VM_OK;
    if ((rc = ensure_grid(h))) return rc;
    cudaError_t e;
    if (!h->gridCanonical) {
        // the step leaves each cell's run in arrival order (nothing in the step
        // depends on it); the exported grid is in ascending slot order
        if ((e = vm_launch_canonical(h->dSites.p, h->dPre.p + 2, 1, h->tiles, h->stream)))
            return cuda_fail(e, "canonical");
        h->gridCanonical = true;
    }
    int live = 0;
    e = cudaMemcpyAsync(&live, h->start.p + h->cells, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
    if (!e) e = cudaStreamSynchronize(h->stream);
    if (!e && start) e = cudaMemcpyAsync(start, h->start.p, sizeof(int) * (size_t)(h->cells + 1), cudaMemcpyDeviceToHost, h->stream);
    if (!e && sortedIdx) e = cudaMemcpyAsync(sortedIdx, h->sortedIdx.p, sizeof(int) * (size_t)live, cudaMemcpyDeviceToHost, h->stream);
    if (!e && sortedPos) e = cudaMemcpyAsync(sortedPos, h->sortedPos.p, sizeof(float2) * (size_t)live, cudaMemcpyDeviceToHost, h->stream);
    if (!e && genCell) e = cudaMemcpyAsync(genCell, h->key.p, sizeof(int) * (size_t)h->numSlots(), cudaMemcpyDeviceToHost, h->stream);
    if (!e) e = cudaStreamSynchronize(h->stream);
    if (e) return cuda_fail(e, "read grid");
    return VM_OK;
}

int vm_knn(vm_optimizer *h, const float *queries, int nq, int K, int *idx, float *d2)
{
    if (!h || nq < 0 || (nq > 0 && (!queries || !idx || !d2))) return fail(VM_ERR_ARG, "vm_knn: bad arguments");
    if (K != 8 && K != 12 && K != 16 && K != 24 && K != 32) return fail(VM_ERR_UNSUPPORTED, "K must be 8, 12, 16, 24 or 32");
    if (nq == 0) return VM_OK;
    if (h->numSlots() == 0) return fail(VM_ERR_STATE, "no generators");
    int rc;
    if ((rc = ensure_grid(h))) return rc;
    if ((rc = h->qbuf.reserve(nq)) || (rc = h->kIdx.reserve((size_t)nq * K)) || (rc = h->kD2.reserve((size_t)nq * K)))
        return rc;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(h->qbuf.p, queries, sizeof(float2) * (size_t)nq, cudaMemcpyHostToDevice, h->stream)) ||
        (e = vm_launch_knn(h->dFit.p, h->qbuf.p, nq, K, h->kIdx.p, h->kD2.p, h->stream)) ||
        (e = cudaMemcpyAsync(idx, h->kIdx.p, sizeof(int) * (size_t)nq * K, cudaMemcpyDeviceToHost, h->stream)) ||
        (e = cudaMemcpyAsync(d2, h->kD2.p, sizeof(float) * (size_t)nq * K, cudaMemcpyDeviceToHost, h->stream)) ||
        (e = cudaStreamSynchronize(h->stream)))
        return cuda_fail(e, "knn");
    return VM_OK;
}

int vm_probe(vm_optimizer *h, int mode, int *i0, int *j, float *loss, float *grad, int *count, float *lossSum)
{
    if (!h || (mode != 0 && mode != 1)) return fail(VM_ERR_ARG, "vm_probe: bad arguments");
    int n = h->numSlots();
    if (n == 0 || h->targetCapacity == 0) return fail(VM_ERR_STATE, "no generators or targets");
    int rc;
    if ((rc = ensure_grid(h))) return rc;
    int live = h->liveTargets;
    if ((rc = h->dbgI0.reserve(std::max(live, 1))) || (rc = h->dbgJ.reserve(std::max(live, 1))) ||
        (rc = h->dbgLoss.reserve(std::max(live, 1))))
        return rc;
    VmFit saved = h->fit;
    h->fit.dbgI0 = h->dbgI0.p;
    h->fit.dbgJ = h->dbgJ.p;
    h->fit.dbgLoss = h->dbgLoss.p;
    if ((rc = upload_tables(h))) return rc;
    cudaError_t e;
    int lossTiles = loss_tiles(h);
    if ((e = vm_launch_loss(h->dFit.p, h->dPre.p + 4, 1, lossTiles, mode, h->lossGrid, h->lossVariant, h->nWindows > 0,
                            h->queue.p, h->stream)) ||
        (e = vm_launch_finalize(h->dFit.p, 1, h->queue.p, h->stream))) {
        h->fit = saved;
        upload_tables(h);
        return cuda_fail(e, "probe");
    }
    std::vector<int> hi0(live), hj(live), slot(live);
    std::vector<float> hl(live);
    std::vector<long long> g(grad ? kGradWords * (size_t)n : 0);
    VmState st;
    if (live > 0) {
        if ((e = cudaMemcpyAsync(hi0.data(), h->dbgI0.p, sizeof(int) * live, cudaMemcpyDeviceToHost, h->stream)) ||
            (e = cudaMemcpyAsync(hj.data(), h->dbgJ.p, sizeof(int) * live, cudaMemcpyDeviceToHost, h->stream)) ||
            (e = cudaMemcpyAsync(hl.data(), h->dbgLoss.p, sizeof(float) * live, cudaMemcpyDeviceToHost, h->stream)) ||
            (e = cudaMemcpyAsync(slot.data(), h->tslot.p, sizeof(int) * live, cudaMemcpyDeviceToHost, h->stream)))
            return cuda_fail(e, "probe read");
    }
    if (grad && (e = cudaMemcpyAsync(g.data(), h->gradX.p, sizeof(long long) * kGradWords * n, cudaMemcpyDeviceToHost,
                                     h->stream)))
        return cuda_fail(e, "probe grad");
    if ((e = cudaMemsetAsync(h->gradX.p, 0, sizeof(long long) * kGradWords * (size_t)n, h->stream)))
        return cuda_fail(e, "probe clear");
    if ((rc = read_state(h, st))) return rc;
    // the pass's gradient flags were read above; clear them with the words
    if ((e = cudaMemsetAsync(&h->state.p->needExact, 0, 2 * sizeof(int), h->stream))) return cuda_fail(e, "probe flags");
    h->fit = saved;
    if ((rc = upload_tables(h))) return rc;
    int cap = h->targetCapacity;
    if (i0) std::fill(i0, i0 + cap, -1);
    if (j) std::fill(j, j + cap, -1);
    if (loss) std::fill(loss, loss + cap, 0.0f);
    for (int t = 0; t < live; ++t) {
        int s = slot[t];
        if (s < 0 || s >= cap) continue;
        if (i0) i0[s] = hi0[t];
        if (j) j[s] = hj[t];
        if (loss) loss[s] = hl[t];
    }
    if (grad) {
        // sections L, DL, DH of 2 words per slot; L is void when the pass redid the gradient exactly
        const long long *L = g.data(), *DL = L + 2 * (size_t)n, *DH = DL + 2 * (size_t)n;
        for (size_t k = 0; k < 2 * (size_t)n; ++k)
            grad[k] = vmk::fx_site_to_float(L[k], !st.needExact, (unsigned long long)DL[k], DH[k], h->fit.gradExp);
    }
    if (count) *count = st.count;
    if (lossSum) *lossSum = st.loss;
    return VM_OK;
}

int vm_extract(vm_optimizer *h, vm_mesh_info *info)
{
    vmh::NvtxRange range("vm_extract");
    if (!h || !info) return fail(VM_ERR_ARG, "bad arguments");
    std::memset(info, 0, sizeof(*info));
    h->mesh = MeshHost();
    int n = h->numSlots();
    if (n == 0) return VM_OK;
    // boundary vertex keys hold three 21-bit fields (label + 4), as in the
    // reference (voro_optimizer.cu:809-815): larger meshes would merge vertices
    if (n > (1 << 21) - 4) return fail(VM_ERR_UNSUPPORTED, "vm_extract: more than 2^21 - 4 generator slots");
    int rc;
    if ((rc = h->cellVerts.reserve((size_t)n * kMaxCellVerts)) || (rc = h->cellEdges.reserve((size_t)n * kMaxCellVerts)) ||
        (rc = h->cellCount.reserve(n)) || (rc = h->inside.reserve(n)))
        return rc;
    cudaError_t e;
    if ((e = cudaEventRecord(h->ev0, h->stream))) return cuda_fail(e, "event");
    if ((rc = ensure_grid(h))) return rc;
    if ((e = cudaMemsetAsync(h->flags.p, 0, 2 * sizeof(int), h->stream)) ||
        (e = vm_launch_cells_n(h->dFit.p, n, h->occ.p, h->tilesX, h->tilesY, h->invVoxel, h->cellVerts.p,
                               h->cellEdges.p, h->cellCount.p, h->inside.p, h->flags.p, h->stream)) ||
        (e = cudaEventRecord(h->ev1, h->stream)) || (e = cudaEventSynchronize(h->ev1)))
        return cuda_fail(e, "extract");
    cudaEventElapsedTime(&h->mesh.gpuMs, h->ev0, h->ev1);
    auto t0 = std::chrono::steady_clock::now();
    // pack the cells in CSR order on the device (scan of the counts, then a
    // gather), so only the used vertex slots cross to the host
    int tiles = (n + kScanTile - 1) / kScanTile;
    VmPointSet C{};
    C.gridW = n;
    C.gridH = 1;
    C.counts = h->cellCount.p;
    int pre[2] = {0, tiles};
    if ((rc = h->cellStartD.reserve((size_t)n + 1)) || (rc = zeroed_tile_state(h->csrTileState, tiles, h->stream)) ||
        (rc = h->dCsrSet.reserve(1)) || (rc = h->dCsrPre.reserve(2)))
        return rc;
    C.start = h->cellStartD.p;
    C.tileState = h->csrTileState.p;
    int total = 0, flags[2], nBnd = 0, nVert = 0;
    if ((e = cudaMemcpyAsync(h->dCsrSet.p, &C, sizeof(C), cudaMemcpyHostToDevice, h->stream)) ||
        (e = cudaMemcpyAsync(h->dCsrPre.p, pre, sizeof(pre), cudaMemcpyHostToDevice, h->stream)) ||
        (e = vm_launch_scan(h->dCsrSet.p, h->dCsrPre.p, 1, tiles, h->stream)) ||
        (e = cudaMemcpyAsync(&total, h->cellStartD.p + n, sizeof(int), cudaMemcpyDeviceToHost, h->stream)) ||
        (e = cudaStreamSynchronize(h->stream)))
        return cuda_fail(e, "extract pack");
    if ((rc = h->csrVerts.reserve(std::max(total, 1))) || (rc = h->csrLabels.reserve(std::max(total, 1)))) return rc;
    if ((e = vm_launch_compact_cells(h->cellVerts.p, h->cellEdges.p, h->cellStartD.p, n, h->csrVerts.p,
                                     h->csrLabels.p, h->stream)))
        return cuda_fail(e, "extract pack");
    // boundary assembly on the device (reference voro_optimizer.cu:798-835):
    // boundary edges in cell order, vertices numbered by first occurrence
    if ((rc = h->bndCnt.reserve((size_t)n + 1)) || (rc = h->bndPartial.reserve((size_t)vm_scan_partials(n + 1))) ||
        (rc = h->bndErr.reserve(1)))
        return rc;
    if ((e = cudaMemsetAsync(h->bndErr.p, 0, sizeof(int), h->stream)) ||
        (e = vm_launch_boundary(n, h->cellStartD.p, h->csrLabels.p, h->csrVerts.p, h->inside.p, h->bndCnt.p, 0, nullptr,
                                nullptr, 0, nullptr, nullptr, nullptr, 0, nullptr, nullptr, nullptr, nullptr,
                                h->stream)) ||
        (e = vm_scan_ex(h->bndCnt.p, h->bndCnt.p, n, h->bndPartial.p, h->stream)) ||
        (e = cudaMemcpyAsync(&nBnd, h->bndCnt.p + n, sizeof(int), cudaMemcpyDeviceToHost, h->stream)) ||
        (e = cudaStreamSynchronize(h->stream)))
        return cuda_fail(e, "boundary count");
    const int occ = 2 * nBnd;
    if (occ > 0) {
        size_t cap = 64;
        while (cap < 2 * (size_t)occ) cap <<= 1;
        if ((rc = h->bndKeys.reserve(cap)) || (rc = h->bndMin.reserve(cap)) || (rc = h->bndSlot.reserve(occ)) ||
            (rc = h->bndPt.reserve(occ)) || (rc = h->bndFirst.reserve((size_t)occ + 1)) ||
            (rc = h->bndEdges.reserve(occ)) || (rc = h->bndVerts.reserve(occ)) ||
            (rc = h->bndPartial.reserve((size_t)vm_scan_partials(occ + 1))))
            return rc;
        unsigned mask = (unsigned)(cap - 1);
        if ((e = cudaMemsetAsync(h->bndKeys.p, 0xFF, cap * sizeof(unsigned long long), h->stream)) ||
            (e = cudaMemsetAsync(h->bndMin.p, 0x7F, cap * sizeof(int), h->stream)) ||
            (e = vm_launch_boundary(n, h->cellStartD.p, h->csrLabels.p, h->csrVerts.p, h->inside.p, nullptr, 1,
                                    h->bndCnt.p, h->bndKeys.p, mask, h->bndMin.p, h->bndSlot.p, h->bndPt.p, occ,
                                    nullptr, nullptr, nullptr, h->bndErr.p, h->stream)) ||
            (e = vm_launch_boundary(n, nullptr, nullptr, nullptr, nullptr, nullptr, 2, nullptr, nullptr, mask,
                                    h->bndMin.p, h->bndSlot.p, nullptr, occ, h->bndFirst.p, nullptr, nullptr, nullptr,
                                    h->stream)) ||
            (e = vm_scan_ex(h->bndFirst.p, h->bndFirst.p, occ, h->bndPartial.p, h->stream)) ||
            (e = vm_launch_boundary(n, nullptr, nullptr, nullptr, nullptr, nullptr, 3, nullptr, nullptr, mask,
                                    h->bndMin.p, h->bndSlot.p, h->bndPt.p, occ, h->bndFirst.p, h->bndEdges.p,
                                    h->bndVerts.p, nullptr, h->stream)) ||
            (e = cudaMemcpyAsync(&nVert, h->bndFirst.p + occ, sizeof(int), cudaMemcpyDeviceToHost, h->stream)) ||
            (e = cudaStreamSynchronize(h->stream)))
            return cuda_fail(e, "boundary assembly");
    }
    // the cells stay on the device until vm_mesh_copy copies them straight
    // into the caller's arrays (one copy); the generators and occupancy
    // flags are snapshotted, since a Step or SetGenerators changes them
    MeshHost &M = h->mesh;
    if ((rc = h->meshGen.reserve(n)) || (rc = h->meshInside.reserve(n))) return rc;
    if ((e = cudaMemcpyAsync(h->meshGen.p, h->gen.p, sizeof(float2) * n, cudaMemcpyDeviceToDevice, h->stream)) ||
        (e = cudaMemcpyAsync(h->meshInside.p, h->inside.p, n, cudaMemcpyDeviceToDevice, h->stream)) ||
        (e = cudaMemcpyAsync(flags, h->flags.p, sizeof(flags), cudaMemcpyDeviceToHost, h->stream)))
        return cuda_fail(e, "extract read");
    M.numGenerators = n;
    M.numCellVerts = total;
    M.edges.resize((size_t)occ);
    M.vertices.resize((size_t)nVert);
    int bndErr = 0;
    if ((occ && (e = cudaMemcpyAsync(M.edges.data(), h->bndEdges.p, sizeof(int) * (size_t)occ, cudaMemcpyDeviceToHost,
                                     h->stream))) ||
        (nVert && (e = cudaMemcpyAsync(M.vertices.data(), h->bndVerts.p, sizeof(float2) * (size_t)nVert,
                                       cudaMemcpyDeviceToHost, h->stream))) ||
        (e = cudaMemcpyAsync(&bndErr, h->bndErr.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream)) ||
        (e = cudaStreamSynchronize(h->stream)))
        return cuda_fail(e, "extract read");
    if (bndErr) return fail(VM_ERR_CUDA, "boundary assembly: vertex table full");
    M.unsafeCells = flags[0];
    M.overflowCells = flags[1];
    boundary_topology(M);
    M.hostMs = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    info->numGenerators = n;
    info->numCellVerts = total;
    info->numVertices = (int)M.vertices.size();
    info->numEdges = (int)(M.edges.size() / 2);
    info->watertight = M.watertight ? 1 : 0;
    info->loops = M.loops;
    info->unsafeCells = M.unsafeCells;
    info->overflowCells = M.overflowCells;
    info->gpuMs = M.gpuMs;
    info->hostMs = M.hostMs;
    return VM_OK;
}

int vm_mesh_copy(vm_optimizer *h, float *generators, uint8_t *inside, int *cellStart, float *cellVerts, float *vertices,
                 int *edges, int *cellLabels)
{
    vmh::NvtxRange range("vm_mesh_copy");
    if (!h) return fail(VM_ERR_ARG, "NULL handle");
    const MeshHost &M = h->mesh;
    const size_t n = (size_t)M.numGenerators, total = (size_t)M.numCellVerts;
    cudaError_t e = cudaSuccess;
    if (n) {
        if (!e && generators) e = cudaMemcpyAsync(generators, h->meshGen.p, sizeof(float2) * n, cudaMemcpyDeviceToHost, h->stream);
        if (!e && inside) e = cudaMemcpyAsync(inside, h->meshInside.p, n, cudaMemcpyDeviceToHost, h->stream);
        if (!e && cellStart)
            e = cudaMemcpyAsync(cellStart, h->cellStartD.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, h->stream);
    }
    if (total) {
        if (!e && cellVerts)
            e = cudaMemcpyAsync(cellVerts, h->csrVerts.p, sizeof(float2) * total, cudaMemcpyDeviceToHost, h->stream);
        if (!e && cellLabels)
            e = cudaMemcpyAsync(cellLabels, h->csrLabels.p, sizeof(int) * total, cudaMemcpyDeviceToHost, h->stream);
    }
    if (vertices) std::memcpy(vertices, M.vertices.data(), sizeof(float2) * M.vertices.size());
    if (edges) std::memcpy(edges, M.edges.data(), sizeof(int) * M.edges.size());
    if (!e) e = cudaStreamSynchronize(h->stream);
    return e ? cuda_fail(e, "vm_mesh_copy") : VM_OK;
}

// ===========================================================================
// checkpoint / resume
// ===========================================================================
int vm_checkpoint(vm_optimizer *h, vm_checkpoint_info *info, float *gen, float *m, float *v)
{
    if (!h || !info) return fail(VM_ERR_ARG, "vm_checkpoint: bad arguments");
    vmh::NvtxRange range("vm_checkpoint");
    info->slotsW = h->slotsW;
    info->slotsH = h->slotsH;
    info->slotCellSize = h->slotCellSize;
    info->scheduleLength = h->scheduleLength;
    info->iteration = h->iteration;
    info->cx0 = h->fit.cx0;
    info->cy0 = h->fit.cy0;
    info->cx1 = h->fit.cx1;
    info->cy1 = h->fit.cy1;
    info->lastBatchLoss = h->lastBatchLoss;
    size_t bytes = sizeof(float2) * (size_t)h->numSlots();
    cudaError_t e = cudaSuccess;
    if (bytes && gen) e = cudaMemcpyAsync(gen, h->gen.p, bytes, cudaMemcpyDeviceToHost, h->stream);
    if (!e && bytes && m) e = cudaMemcpyAsync(m, h->m.p, bytes, cudaMemcpyDeviceToHost, h->stream);
    if (!e && bytes && v) e = cudaMemcpyAsync(v, h->v.p, bytes, cudaMemcpyDeviceToHost, h->stream);
    if (!e) e = cudaStreamSynchronize(h->stream);
    return e ? cuda_fail(e, "vm_checkpoint") : VM_OK;
}

int vm_restore(vm_optimizer *h, const vm_checkpoint_info *info, const float *gen, const float *m, const float *v)
{
    if (!h || !info || info->iteration < 0 || info->scheduleLength < 0 ||
        ((long long)info->slotsW * info->slotsH > 0 && (!gen || !m || !v)))
        return fail(VM_ERR_ARG, "vm_restore: bad arguments");
    vmh::NvtxRange range("vm_restore");
    int rc;
    if ((rc = vm_set_generators(h, gen, info->slotsW, info->slotsH, info->slotCellSize)) ||
        (rc = vm_begin_schedule(h, info->scheduleLength, info->cx0, info->cy0, info->cx1, info->cy1)))
        return rc;
    size_t bytes = sizeof(float2) * (size_t)h->numSlots();
    cudaError_t e = cudaSuccess;
    if (bytes) {
        e = cudaMemcpyAsync(h->m.p, m, bytes, cudaMemcpyHostToDevice, h->stream);
        if (!e) e = cudaMemcpyAsync(h->v.p, v, bytes, cudaMemcpyHostToDevice, h->stream);
    }
    // the step counter drives the learning-rate milestones, the bias
    // corrections and the subsample mask of the next steps
    int iter = info->iteration;
    if (!e) e = cudaMemcpyAsync(&h->state.p->iter, &iter, sizeof(int), cudaMemcpyHostToDevice, h->stream);
    if (!e) e = cudaStreamSynchronize(h->stream);
    if (e) return cuda_fail(e, "vm_restore");
    h->iteration = info->iteration;
    h->lastBatchLoss = info->lastBatchLoss;
    return VM_OK;
}

// ===========================================================================
// canvas hand-off (device to device)
// ===========================================================================
int vm_set_targets_from_canvas(vm_optimizer *h, cv_canvas *c)
{
    vmh::NvtxRange range("vm_set_targets_from_canvas");
    if (!h || !c) return fail(VM_ERR_ARG, "vm_set_targets_from_canvas: NULL handle");
    CanvasView v{};
    int rc;
    if ((rc = canvas_view(c, &v))) return rc;
    // SetTargets(canvas.TargetSlots()) (voro_optimizer.cu:549-560)
    if ((rc = set_targets_from(h, v.slots, v.nslots, cudaMemcpyDeviceToDevice))) return rc;
    // SetOccupancy(InsideMasks(), TilesX(), TilesY(), VoxelSize()) (:589-600)
    size_t n = (size_t)v.tilesX * v.tilesY;
    if (v.tilesX != h->tilesX || v.tilesY != h->tilesY) {
        h->tilesX = v.tilesX;
        h->tilesY = v.tilesY;
        if ((rc = h->occ.alloc(n))) return rc;
    }
    h->invVoxel = 1.0f / v.voxelSize;
    cudaError_t e;
    if (n && (e = cudaMemcpyAsync(h->occ.p, v.inside, sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, h->stream)))
        return cuda_fail(e, "canvas occupancy");
    if ((e = cudaStreamSynchronize(h->stream))) return cuda_fail(e, "canvas occupancy");
    return VM_OK;
}

int vm_update_from_canvas(vm_optimizer *h, cv_canvas *c)
{
    vmh::NvtxRange range("vm_update_from_canvas");
    if (!h || !c) return fail(VM_ERR_ARG, "vm_update_from_canvas: NULL handle");
    CanvasView v{};
    int rc;
    cudaError_t e;
    if ((rc = canvas_view(c, &v))) return rc;
    // UpdateTargets(edit.dirtySlots, TargetSlots()) (voro_optimizer.cu:562-587)
    if (v.ndirty > 0) {
        if (v.nslots > h->targetCapacity) {
            // grow with slack: the slot array, then {-1, -1} slots (:566-571)
            size_t cap = std::max((size_t)v.nslots * 3 / 2, (size_t)v.nslots + 64);
            drop_graph(h);
            h->targetCapacity = (int)cap;
            if ((rc = h->traw.alloc(cap)) || (rc = h->tkey.alloc(cap)) || (rc = h->trank.alloc(cap)) ||
                (rc = h->tpos.alloc(cap)) || (rc = h->tslot.alloc(cap)))
                return rc;
            if ((e = cudaMemcpyAsync(h->traw.p, v.slots, sizeof(float2) * (size_t)v.nslots, cudaMemcpyDeviceToDevice,
                                     h->stream)) ||
                (e = canvas_fill_empty(h->traw.p + v.nslots, cap - (size_t)v.nslots, h->stream)))
                return cuda_fail(e, "canvas targets");
            if ((rc = upload_tables(h))) return rc;
        } else if ((e = vm_launch_scatter_targets(h->traw.p, v.dirty, v.dirtyValues, v.ndirty, h->stream))) {
            return cuda_fail(e, "canvas targets");
        }
        if ((rc = sort_targets(h))) return rc;
    }
    // UpdateOccupancy(InsideMasks(), edit tile rectangle) (:602-611)
    if (v.tilesX != h->tilesX || v.tilesY != h->tilesY)
        return fail(VM_ERR_STATE, "vm_update_from_canvas: occupancy grid differs from the canvas (SetOccupancy first)");
    int tx0 = std::max(v.tx0, 0), ty0 = std::max(v.ty0, 0);
    int tx1 = std::min(v.tx1, h->tilesX), ty1 = std::min(v.ty1, h->tilesY);
    if ((e = canvas_copy_rect(v.inside, h->occ.p, h->tilesX, tx0, ty0, tx1, ty1, h->stream)) ||
        (e = cudaStreamSynchronize(h->stream)))
        return cuda_fail(e, "canvas occupancy");
    return VM_OK;
}

// ===========================================================================
// Poisson sampler
// ===========================================================================
} // extern "C"

namespace {
// Pinned staging of pd_resample_many's job table and packed regions (shared
// by every sampler of the process; calls take turns).
std::mutex g_pdStageMu;
char *g_pdStage = nullptr;
size_t g_pdStageCap = 0;
} // namespace

struct pd_sampler {
    float width, height, radius, cellSize;
    int gridW, gridH, trials;
    unsigned seed, roundBase = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    DevBuf<float2> grid;
    std::vector<float2> cells;
};

extern "C" {

int pd_create(float width, float height, float radius, int trials, unsigned seed, pd_sampler **out)
{
    if (!out) return fail(VM_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (!(width > 0.0f) || !(height > 0.0f) || !(radius > 0.0f) || trials < 0)
        return fail(VM_ERR_ARG, "width, height, radius must be > 0 and trials >= 0");
    pd_sampler *s = new pd_sampler();
    s->width = width;
    s->height = height;
    s->radius = radius;
    // Sampler::Sampler (reference poisson_disk.cu:120-125)
    s->cellSize = radius / sqrtf(2.0f);
    double gw = std::ceil((double)(width / s->cellSize)), gh = std::ceil((double)(height / s->cellSize));
    if (gw * gh > 2.0e9) {
        delete s;
        return fail(VM_ERR_ARG, "sampler grid too large");
    }
    s->gridW = (int)ceilf(width / s->cellSize);
    s->gridH = (int)ceilf(height / s->cellSize);
    s->trials = trials;
    s->seed = seed;
    size_t nCells = (size_t)s->gridW * s->gridH;
    s->cells.assign(nCells, make_float2(-1.0f, -1.0f));
    cudaError_t e;
    int rc = VM_OK;
    if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) || (e = cudaEventCreate(&s->ev0)) ||
        (e = cudaEventCreate(&s->ev1)))
        rc = cuda_fail(e, "sampler stream");
    if (!rc) rc = s->grid.alloc(nCells);
    if (!rc) rc = pd_resample(s, 0, 0, s->gridW, s->gridH, nullptr);
    if (rc) {
        pd_destroy(s);
        return rc;
    }
    *out = s;
    return VM_OK;
}

int pd_destroy(pd_sampler *s)
{
    if (!s) return VM_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return VM_OK;
}

int pd_resample(pd_sampler *s, int cx0, int cy0, int cx1, int cy1, float *gpuMs)
{
    vmh::NvtxRange range("pd_resample");
    if (!s) return fail(VM_ERR_ARG, "NULL sampler");
    if (gpuMs) *gpuMs = 0.0f;
    int x0 = std::max(cx0, 0), y0 = std::max(cy0, 0), x1 = std::min(cx1, s->gridW), y1 = std::min(cy1, s->gridH);
    if (x0 >= x1 || y0 >= y1) return VM_OK;
    PdParams p{s->width, s->height, s->radius, s->cellSize, s->gridW, s->gridH, s->seed};
    // phases as programmatic dependent launches unless VM_PD_PDL=0 (same samples)
    const char *env = std::getenv("VM_PD_PDL");
    const bool pdl = !(env && std::atoi(env) == 0);
    cudaError_t e;
    if ((e = cudaEventRecord(s->ev0, s->stream)) ||
        (e = pd_launch_resample(s->grid.p, p, x0, y0, x1, y1, s->trials, s->roundBase, s->stream, pdl)) ||
        (e = cudaEventRecord(s->ev1, s->stream)))
        return cuda_fail(e, "resample");
    s->roundBase += (unsigned)s->trials;
    size_t pitch = (size_t)s->gridW * sizeof(float2);
    size_t off = (size_t)y0 * s->gridW + x0;
    if ((e = cudaMemcpy2DAsync(s->cells.data() + off, pitch, s->grid.p + off, pitch, (x1 - x0) * sizeof(float2), y1 - y0,
                               cudaMemcpyDeviceToHost, s->stream)) ||
        (e = cudaStreamSynchronize(s->stream)))
        return cuda_fail(e, "resample read");
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    if (gpuMs) *gpuMs = ms;
    return VM_OK;
}

int pd_resample_many(pd_sampler *const *samplers, const int *regions, int n, float *gpuMs)
{
    vmh::NvtxRange range("pd_resample_many");
    if (gpuMs) *gpuMs = 0.0f;
    if (n < 0 || (n && (!samplers || !regions))) return fail(VM_ERR_ARG, "pd_resample_many: bad arguments");
    for (int i = 0; i < n; ++i) {
        if (!samplers[i]) return fail(VM_ERR_ARG, "pd_resample_many: NULL sampler");
        for (int k = 0; k < i; ++k)
            if (samplers[k] == samplers[i]) return fail(VM_ERR_ARG, "pd_resample_many: a sampler appears twice");
    }
    cudaError_t e;
    std::vector<PdJob> jobs;
    std::vector<int> jobOf;
    float total = 0.0f;
    for (int i = 0; i < n; ++i) {
        pd_sampler *s = samplers[i];
        const int *r = regions + 4 * (size_t)i;
        int x0 = std::max(r[0], 0), y0 = std::max(r[1], 0), x1 = std::min(r[2], s->gridW), y1 = std::min(r[3], s->gridH);
        if (x0 >= x1 || y0 >= y1) continue;
        if (!pd_small_region(x0, y0, x1, y1)) { // a large region: its own launches
            float ms = 0.0f;
            int rc = pd_resample(s, x0, y0, x1, y1, &ms);
            if (rc) return rc;
            total += ms;
            continue;
        }
        // the sampler's own stream must be done with its grid (usually it is idle)
        e = cudaStreamQuery(s->stream);
        if (e == cudaErrorNotReady) e = cudaStreamSynchronize(s->stream);
        if (e) return cuda_fail(e, "pd_resample_many sync");
        PdParams p{s->width, s->height, s->radius, s->cellSize, s->gridW, s->gridH, s->seed};
        jobs.push_back(PdJob{s->grid.p, p, x0, y0, x1, y1, s->trials, s->roundBase});
        jobOf.push_back(i);
    }
    if (!jobs.empty()) {
        pd_sampler *s0 = samplers[jobOf[0]];
        cudaStream_t st = s0->stream;
        // the regions come back packed: one device-to-host copy for all of them
        int nj = (int)jobs.size();
        size_t stageBytes = 0;
        for (const PdJob &j : jobs) stageBytes = std::max(stageBytes, pd_stage_bytes(j.x0, j.y0, j.x1, j.y1));
        std::vector<int> offsets(nj + 1, 0);
        for (int k = 0; k < nj; ++k)
            offsets[k + 1] = offsets[k] + (jobs[k].x1 - jobs[k].x0) * (jobs[k].y1 - jobs[k].y0);
        size_t jobBytes = sizeof(PdJob) * nj, offBytes = sizeof(int) * (size_t)(nj + 1);
        size_t cellBytes = sizeof(float2) * (size_t)offsets[nj];
        size_t offAt = (jobBytes + 255) & ~(size_t)255, cellAt = offAt + ((offBytes + 255) & ~(size_t)255);
        std::lock_guard<std::mutex> lk(g_pdStageMu);
        if (g_pdStageCap < cellAt + cellBytes) {
            if (g_pdStage) cudaFreeHost(g_pdStage);
            g_pdStage = nullptr;
            g_pdStageCap = 0;
            size_t cap = std::max(cellAt + cellBytes, (size_t)1 << 20);
            if ((e = cudaMallocHost((void **)&g_pdStage, cap))) return cuda_fail(e, "pd_resample_many staging");
            g_pdStageCap = cap;
        }
        std::memcpy(g_pdStage, jobs.data(), jobBytes);
        std::memcpy(g_pdStage + offAt, offsets.data(), offBytes);
        char *dBuf = nullptr;
        if ((e = cudaMallocAsync((void **)&dBuf, cellAt + cellBytes, st))) return cuda_fail(e, "pd_resample_many jobs");
        PdJob *dJobs = reinterpret_cast<PdJob *>(dBuf);
        const int *dOff = reinterpret_cast<const int *>(dBuf + offAt);
        float2 *dCells = reinterpret_cast<float2 *>(dBuf + cellAt);
        if ((e = cudaMemcpyAsync(dBuf, g_pdStage, cellAt, cudaMemcpyHostToDevice, st)) ||
            (e = cudaEventRecord(s0->ev0, st)) || (e = pd_launch_resample_many(dJobs, nj, stageBytes, st)) ||
            (e = cudaEventRecord(s0->ev1, st)) || (e = pd_launch_gather_regions(dJobs, dOff, nj, dCells, st)) ||
            (e = cudaMemcpyAsync(g_pdStage + cellAt, dCells, cellBytes, cudaMemcpyDeviceToHost, st))) {
            cudaFreeAsync(dBuf, st);
            cudaStreamSynchronize(st);
            return cuda_fail(e, "pd_resample_many");
        }
        cudaFreeAsync(dBuf, st);
        if ((e = cudaStreamSynchronize(st))) return cuda_fail(e, "pd_resample_many read");
        const float2 *packed = reinterpret_cast<const float2 *>(g_pdStage + cellAt);
        for (int k = 0; k < nj; ++k) {
            pd_sampler *s = samplers[jobOf[k]];
            const PdJob &j = jobs[k];
            s->roundBase += (unsigned)s->trials;
            int w = j.x1 - j.x0;
            for (int y = j.y0; y < j.y1; ++y)
                std::memcpy(s->cells.data() + (size_t)y * s->gridW + j.x0, packed + offsets[k] + (y - j.y0) * w,
                            sizeof(float2) * w);
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, s0->ev0, s0->ev1);
        total += ms;
    }
    if (gpuMs) *gpuMs = total;
    return VM_OK;
}

int pd_info(pd_sampler *s, pd_info_t *out)
{
    if (!s || !out) return fail(VM_ERR_ARG, "bad arguments");
    out->width = s->width;
    out->height = s->height;
    out->radius = s->radius;
    out->cellSize = s->cellSize;
    out->gridW = s->gridW;
    out->gridH = s->gridH;
    out->trials = s->trials;
    out->seed = s->seed;
    out->roundBase = s->roundBase;
    return VM_OK;
}

int pd_cells(pd_sampler *s, float *xy)
{
    if (!s || !xy) return fail(VM_ERR_ARG, "bad arguments");
    std::memcpy(xy, s->cells.data(), sizeof(float2) * s->cells.size());
    return VM_OK;
}

// Sampler::Verify (reference poisson_disk.cu:179-199)
int pd_verify(pd_sampler *s, int cx0, int cy0, int cx1, int cy1, int *ok)
{
    if (!s || !ok) return fail(VM_ERR_ARG, "bad arguments");
    float r2 = s->radius * s->radius;
    int W = s->gridW, H = s->gridH;
    int vx0 = std::max(cx0 - 2, 0), vx1 = std::min(cx1 + 2, W);
    int vy0 = std::max(cy0 - 2, 0), vy1 = std::min(cy1 + 2, H);
    *ok = 1;
    for (int cy = vy0; cy < vy1; ++cy)
        for (int cx = vx0; cx < vx1; ++cx) {
            float2 a = s->cells[(size_t)cy * W + cx];
            if (a.x < 0) continue;
            for (int ny = std::max(cy - 2, 0); ny <= std::min(cy + 2, H - 1); ++ny)
                for (int nx = std::max(cx - 2, 0); nx <= std::min(cx + 2, W - 1); ++nx) {
                    if (nx == cx && ny == cy) continue;
                    float2 b = s->cells[(size_t)ny * W + nx];
                    if (b.x < 0) continue;
                    float dx = a.x - b.x, dy = a.y - b.y;
                    if (dx * dx + dy * dy < r2) {
                        *ok = 0;
                        return VM_OK;
                    }
                }
        }
    return VM_OK;
}

int pd_count(pd_sampler *s, long long *n)
{
    if (!s || !n) return fail(VM_ERR_ARG, "bad arguments");
    long long c = 0;
    for (const float2 &p : s->cells) c += p.x >= 0.0f;
    *n = c;
    return VM_OK;
}

} // extern "C"
