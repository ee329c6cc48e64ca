// Batched fits and the serving loop (C ABI vmb_* / vms_*).
//
// The reference runs one fit per VoroOptimizer, one after another
// (apps/voromesh_demo.cpp:103-156). Here any number of independent fits of
// uneven sizes live in one device arena and step together: each stage of a
// step is one launch over the packed table of all live fits (VmFit /
// VmPointSet rows, block-prefix tables mapping blocks to fits), so small fits
// no longer pay a launch train each and large ones fill the GPU.
//
// Results are independent of the company a fit keeps: every per-fit sum is an
// exact fixed-point sum and every fit's state is its own, so a fit stepped in
// a batch produces bit-for-bit the generators it produces alone.
//
// The arena doubles as the HBM budget: a fit is admitted only when all of its
// buffers fit in the arena's free space (VM_ERR_BUDGET otherwise).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <thread>
#include <vector>

#include "vm_capi.h"
#include "vm_host.h"
#include "vm_kernels.h"

using namespace vmh;

namespace {

constexpr size_t kAlign = 256;
size_t aligned(size_t b) { return (b + kAlign - 1) / kAlign * kAlign; }

// First-fit device sub-allocator over one cudaMalloc, with coalescing.
struct Arena {
    char *base = nullptr;
    size_t cap = 0;
    std::map<size_t, size_t> free_; // offset -> size
    ~Arena()
    {
        if (base) cudaFree(base);
    }
    int init(size_t bytes)
    {
        bytes = aligned(bytes);
        cudaError_t e = cudaMalloc(&base, bytes);
        if (e) {
            base = nullptr;
            return cuda_fail(e, "arena cudaMalloc");
        }
        cap = bytes;
        free_[0] = bytes;
        return VM_OK;
    }
    bool alloc(size_t bytes, size_t *off)
    {
        bytes = aligned(std::max<size_t>(bytes, 1));
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            *off = it->first;
            size_t rest = it->second - bytes, at = it->first + bytes;
            free_.erase(it);
            if (rest) free_[at] = rest;
            return true;
        }
        return false;
    }
    void release(size_t off, size_t bytes)
    {
        bytes = aligned(std::max<size_t>(bytes, 1));
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t freeBytes() const
    {
        size_t s = 0;
        for (auto &kv : free_) s += kv.second;
        return s;
    }
};

struct BFit {
    bool live = false, done = false;
    float width = 0, height = 0, spacing = 0, slotCellSize = 0;
    vm_params params{};
    int slotsW = 0, slotsH = 0, n = 0, gridW = 0, gridH = 0, cells = 0, tiles = 0, cap = 0, liveTargets = 0;
    std::vector<std::pair<size_t, size_t>> blocks; // arena (offset, bytes)
    VmFit desc{};
    VmPointSet sites{}, tset{};
    float2 *traw = nullptr;
    // the live-target and 5x5-block counts are on their way to the host
    // (hcounts); desc.nTargets, desc.fastShift and liveTargets wait for them
    bool countsPending = false;
};

int fail_budget(const char *what) { return fail(VM_ERR_BUDGET, what); }

} // namespace

struct vmb_batch {
    Arena arena;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr; // one step of the current fit set (captured after each table rebuild)
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int maxFits = 0;
    std::vector<BFit> fits;          // by fit id
    DevBuf<VmState> states;          // by fit id
    std::vector<int> order;          // fit ids in the current tables
    DevBuf<VmFit> dFits, dOneFit;
    DevBuf<VmPointSet> dSites, dOneSet;
    DevBuf<int> dPre, dOnePre;       // [sitePre | scanPre | lossPre], single-set prefixes
    DevBuf<char> queue;
    DevBuf<int2> qitems;
    int siteBlocks = 0, scanTiles = 0, lossTiles = 0;
    int lossVariant = 1, lossTile = 256, lossGrid = 0;
    bool dirty = true;
    std::vector<VmState> hostStates;
    DevBuf<int> block5Buf; // a fit's largest 5x5-block target count, read back at vmb_add_fit
    int *hcounts = nullptr; // pinned, per fit id: live targets, largest 5x5-block count
    // pinned staging of host-to-device copies (a copy from pageable memory
    // would first wait for the stream); reused from its start after a sync
    char *hstage = nullptr;
    size_t hstageCap = 0, hstageUsed = 0;
};

namespace {

// Copies `bytes` from `src` into the pinned staging buffer and enqueues their
// copy to `dst` on the batch stream. The staged bytes stay untouched until
// the next stream sync (staging_done), so nothing waits here.
cudaError_t stage_copy(vmb_batch *b, void *dst, const void *src, size_t bytes)
{
    if (!bytes) return cudaSuccess;
    size_t room = (bytes + 255) & ~(size_t)255;
    if (b->hstageUsed + room > b->hstageCap) {
        // earlier staged copies may still be reading the buffer
        cudaError_t e = cudaStreamSynchronize(b->stream);
        if (e) return e;
        b->hstageUsed = 0;
        if (room > b->hstageCap) {
            if (b->hstage) cudaFreeHost(b->hstage);
            b->hstage = nullptr;
            b->hstageCap = 0;
            size_t cap = std::max(room, (size_t)1 << 22);
            if ((e = cudaMallocHost((void **)&b->hstage, cap))) return e;
            b->hstageCap = cap;
        }
    }
    char *p = b->hstage + b->hstageUsed;
    std::memcpy(p, src, bytes);
    b->hstageUsed += room;
    return cudaMemcpyAsync(dst, p, bytes, cudaMemcpyHostToDevice, b->stream);
}

// After a sync of the batch stream every staged copy has been read.
void staging_done(vmb_batch *b) { b->hstageUsed = 0; }

// Completes the fits added since the last sync: one stream sync for all of
// them, then their live-target counts and fast-path shifts from hcounts.
int resolve_counts(vmb_batch *b)
{
    bool any = false;
    for (const BFit &f : b->fits) any |= f.live && f.countsPending;
    if (!any) return VM_OK;
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e) return cuda_fail(e, "batch live targets");
    staging_done(b);
    for (int id = 0; id < (int)b->fits.size(); ++id) {
        BFit &f = b->fits[id];
        if (!f.live || !f.countsPending) continue;
        f.liveTargets = b->hcounts[2 * id];
        f.desc.nTargets = f.liveTargets;
        f.desc.fastShift = vm_fast_shift(b->hcounts[2 * id + 1]);
        f.countsPending = false;
    }
    return VM_OK;
}

int single_set_build(vmb_batch *b, const VmPointSet &S, int emptyIsNegative, int canonical)
{
    VmPointSet T = S;
    T.canonical = canonical;
    int blocks = (T.n + 255) / 256;
    long long keys = (long long)T.gridW * T.gridH << (2 * T.sub);
    int tiles = (int)((keys + kScanTile - 1) / kScanTile);
    int pre[4] = {0, blocks, 0, tiles};
    cudaError_t e;
    if ((e = stage_copy(b, b->dOneSet.p, &T, sizeof(T))) || (e = stage_copy(b, b->dOnePre.p, pre, sizeof(pre))) ||
        (e = vm_launch_bin(b->dOneSet.p, b->dOnePre.p, 1, blocks, emptyIsNegative, b->stream)) ||
        (e = vm_launch_scan(b->dOneSet.p, b->dOnePre.p + 2, 1, tiles, b->stream)) ||
        (e = vm_launch_scatter(b->dOneSet.p, b->dOnePre.p, 1, blocks, nullptr, b->stream)))
        return cuda_fail(e, "batch grid build");
    return VM_OK;
}

int rebuild_tables(vmb_batch *b)
{
    int rc0 = resolve_counts(b);
    if (rc0) return rc0;
    b->order.clear();
    for (int id = 0; id < (int)b->fits.size(); ++id)
        if (b->fits[id].live && !b->fits[id].done) b->order.push_back(id);
    int nf = (int)b->order.size();
    std::vector<VmFit> F(nf);
    std::vector<VmPointSet> S(nf);
    std::vector<int> pre(3 * (nf + 1), 0);
    long long totalLive = 0;
    for (int k = 0; k < nf; ++k) {
        BFit &f = b->fits[b->order[k]];
        F[k] = f.desc;
        S[k] = f.sites;
        pre[k + 1] = pre[k] + (f.n + 255) / 256;
        pre[(nf + 1) + k + 1] = pre[(nf + 1) + k] + f.tiles;
        pre[2 * (nf + 1) + k + 1] = pre[2 * (nf + 1) + k] + (f.liveTargets + b->lossTile - 1) / b->lossTile;
        totalLive += f.liveTargets;
    }
    b->siteBlocks = pre[nf];
    b->scanTiles = pre[(nf + 1) + nf];
    b->lossTiles = pre[2 * (nf + 1) + nf];
    int rc;
    if ((rc = b->dFits.reserve(std::max(nf, 1))) || (rc = b->dSites.reserve(std::max(nf, 1))) ||
        (rc = b->dPre.reserve(pre.size())))
        return rc;
    int qcap = (int)std::max<long long>(totalLive, 1);
    if ((size_t)qcap > b->qitems.n) {
        if ((rc = b->qitems.alloc((size_t)qcap + qcap / 2))) return rc;
    }
    cudaError_t e;
    if ((nf && ((e = cudaMemcpyAsync(b->dFits.p, F.data(), sizeof(VmFit) * nf, cudaMemcpyHostToDevice, b->stream)) ||
                (e = cudaMemcpyAsync(b->dSites.p, S.data(), sizeof(VmPointSet) * nf, cudaMemcpyHostToDevice,
                                     b->stream)))) ||
        (e = cudaMemcpyAsync(b->dPre.p, pre.data(), sizeof(int) * pre.size(), cudaMemcpyHostToDevice, b->stream)) ||
        (e = vm_queue_init(b->queue.p, b->qitems.p, (int)b->qitems.n, b->stream)) ||
        (e = cudaStreamSynchronize(b->stream)))
        return cuda_fail(e, "batch tables");
    staging_done(b);
    b->dirty = false;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    return VM_OK;
}

int enqueue_batch_step(vmb_batch *b)
{
    int nf = (int)b->order.size();
    if (!nf) return VM_OK;
    int *sitePre = b->dPre.p, *scanPre = b->dPre.p + (nf + 1), *lossPre = b->dPre.p + 2 * (nf + 1);
    cudaError_t e;
    if ((e = vm_launch_loss(b->dFits.p, lossPre, nf, b->lossTiles, 0, b->lossGrid, b->lossVariant, 0, b->queue.p,
                            b->stream)) ||
        (e = vm_launch_adam_bin(b->dFits.p, sitePre, nf, b->siteBlocks, b->queue.p, b->stream)) ||
        (e = vm_launch_scan(b->dSites.p, scanPre, nf, b->scanTiles, b->stream)) ||
        (e = vm_launch_scatter(b->dSites.p, sitePre, nf, b->siteBlocks, b->dFits.p, b->stream)))
        return cuda_fail(e, "batch step");
    return VM_OK;
}

// The step of the current fit set as a CUDA graph (captured once per table
// rebuild, replayed every step).
int ensure_batch_graph(vmb_batch *b)
{
    if (b->graph) return VM_OK;
    cudaGraph_t g;
    cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (e) return cuda_fail(e, "batch capture");
    int rc = enqueue_batch_step(b);
    e = cudaStreamEndCapture(b->stream, &g);
    if (e) return rc ? rc : cuda_fail(e, "batch capture");
    if (rc) {
        cudaGraphDestroy(g);
        return rc;
    }
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    return e ? cuda_fail(e, "batch graph") : VM_OK;
}

int read_states(vmb_batch *b)
{
    b->hostStates.resize(b->fits.size());
    if (b->fits.empty()) return VM_OK;
    cudaError_t e = cudaMemcpyAsync(b->hostStates.data(), b->states.p, sizeof(VmState) * b->fits.size(),
                                    cudaMemcpyDeviceToHost, b->stream);
    if (!e) e = cudaStreamSynchronize(b->stream);
    if (e) return cuda_fail(e, "batch states");
    for (size_t k = 0; k < b->fits.size(); ++k)
        if (b->fits[k].live && b->hostStates[k].errors)
            return fail(VM_ERR_CUDA, "kernel error bits 0x" + std::to_string(b->hostStates[k].errors) + " in fit " +
                                         std::to_string(k));
    return VM_OK;
}

void release_fit(vmb_batch *b, BFit &f)
{
    for (auto &bl : f.blocks) b->arena.release(bl.first, bl.second);
    f.blocks.clear();
    f.live = false;
    f.done = false;
}

} // namespace

extern "C" {

int vmb_create(size_t arenaBytes, int maxFits, int lossVariant, vmb_batch **out)
{
    if (!out || maxFits < 1 || arenaBytes < (1u << 20)) return fail(VM_ERR_ARG, "vmb_create: bad arguments");
    *out = nullptr;
    vmb_batch *b = new vmb_batch();
    b->maxFits = maxFits;
    int rc = VM_OK;
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) || (e = cudaEventCreate(&b->ev0)) ||
        (e = cudaEventCreate(&b->ev1)))
        rc = cuda_fail(e, "batch stream");
    if (!rc) rc = b->arena.init(arenaBytes);
    if (!rc) rc = b->states.alloc(maxFits);
    if (!rc) rc = b->queue.alloc(vm_queue_bytes());
    if (!rc) rc = b->dOneFit.alloc(1);
    if (!rc) rc = b->dOneSet.alloc(1);
    if (!rc) rc = b->dOnePre.alloc(4);
    if (!rc && (e = cudaMallocHost((void **)&b->hcounts, sizeof(int) * 2 * (size_t)maxFits))) {
        b->hcounts = nullptr;
        rc = cuda_fail(e, "batch counts");
    }
    if (!rc && (e = cudaMemset(b->states.p, 0, sizeof(VmState) * maxFits))) rc = cuda_fail(e, "states");
    if (!rc) {
        b->lossVariant = (lossVariant >= 0 && lossVariant < vm_loss_variants()) ? lossVariant : 1;
        b->lossTile = vm_loss_variant_threads(b->lossVariant);
        b->lossGrid = vm_loss_occupancy_blocks(b->lossVariant);
        b->fits.reserve(maxFits);
    }
    if (rc) {
        vmb_destroy(b);
        return rc;
    }
    *out = b;
    return VM_OK;
}

int vmb_destroy(vmb_batch *b)
{
    if (!b) return VM_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    if (b->hstage) cudaFreeHost(b->hstage);
    if (b->hcounts) cudaFreeHost(b->hcounts);
    delete b;
    return VM_OK;
}

size_t vmb_fit_bytes(int slotsW, int slotsH, int nTargets, float width, float height, float spacing)
{
    if (slotsW < 0 || slotsH < 0 || nTargets < 0 || !(spacing > 0.0f)) return 0;
    size_t n = (size_t)slotsW * slotsH, cap = std::max(nTargets, 1);
    size_t gw = std::max(1, (int)std::ceil(width / spacing)), gh = std::max(1, (int)std::ceil(height / spacing));
    size_t cells = gw * gh, tiles = (cells + kScanTile - 1) / kScanTile;
    n = std::max<size_t>(n, 1);
    return aligned(8 * n) * 3 + aligned(8 * kGradWords * n) + aligned(4 * n) * 3 + aligned(8 * n) + aligned(4 * (cells + 1)) * 2 +
           aligned(8 * (tiles + 1)) + aligned(8 * cap) * 2 + aligned(4 * cap) * 3 + 8 * cap /* queue share */;
}

int vmb_add_fit(vmb_batch *b, const vmb_fit *in, int *fitId)
{
    vmh::NvtxRange range("vmb_add_fit");
    if (!b || !in || !fitId) return fail(VM_ERR_ARG, "vmb_add_fit: bad arguments");
    *fitId = -1;
    if (in->slotsW < 0 || in->slotsH < 0 || in->nTargets < 0 || !(in->width > 0) || !(in->height > 0) ||
        !(in->spacing > 0))
        return fail(VM_ERR_ARG, "vmb_add_fit: bad fit");
    // the single-fit limits: slots as in vm_set_generators, the hash grid as in vm_create
    const long long n64 = (long long)in->slotsW * in->slotsH;
    if (n64 > 0x7FFFFFFF / kMaxCellVerts) return fail(VM_ERR_ARG, "vmb_add_fit: too many generator slots");
    if ((double)std::ceil(in->width / in->spacing) * (double)std::ceil(in->height / in->spacing) > 1.5e9)
        return fail(VM_ERR_ARG, "vmb_add_fit: hash grid too large");
    const int n = (int)n64;
    if ((n > 0 && !in->generators) || (in->nTargets > 0 && !in->targets))
        return fail(VM_ERR_ARG, "vmb_add_fit: NULL buffer");
    int K = in->params.lossK;
    if (K != 8 && K != 12 && K != 16 && K != 24 && K != 32) return fail(VM_ERR_UNSUPPORTED, "lossK");
    int id = -1;
    for (int k = 0; k < (int)b->fits.size(); ++k)
        if (!b->fits[k].live) {
            id = k;
            break;
        }
    if (id < 0) {
        if ((int)b->fits.size() >= b->maxFits) return fail_budget("vmb_add_fit: fit table full");
        b->fits.emplace_back();
        id = (int)b->fits.size() - 1;
    }
    BFit &f = b->fits[id];
    f = BFit();
    f.width = in->width;
    f.height = in->height;
    f.spacing = in->spacing;
    f.slotCellSize = in->slotCellSize;
    f.params = in->params;
    f.slotsW = in->slotsW;
    f.slotsH = in->slotsH;
    f.n = n;
    f.gridW = std::max(1, (int)std::ceil(in->width / in->spacing));
    f.gridH = std::max(1, (int)std::ceil(in->height / in->spacing));
    f.cells = f.gridW * f.gridH;
    f.tiles = (f.cells + kScanTile - 1) / kScanTile;
    f.cap = std::max(in->nTargets, 1);
    // ---- memory: all-or-nothing from the arena
    size_t nn = std::max(n, 1);
    size_t sizes[] = {8 * nn, 8 * nn, 8 * nn, 8 * kGradWords * nn, 4 * nn, 4 * nn, 4 * nn, 8 * nn, 4 * ((size_t)f.cells + 1),
                      4 * ((size_t)f.cells + 1), 8 * ((size_t)f.tiles + 1), 8 * (size_t)f.cap, 4 * (size_t)f.cap,
                      4 * (size_t)f.cap, 8 * (size_t)f.cap, 4 * (size_t)f.cap};
    char *ptrs[16];
    for (int k = 0; k < 16; ++k) {
        size_t off;
        if (!b->arena.alloc(sizes[k], &off)) {
            release_fit(b, f);
            return fail_budget("vmb_add_fit: over the HBM budget");
        }
        f.blocks.push_back({off, sizes[k]});
        ptrs[k] = b->arena.base + off;
    }
    VmFit &D = f.desc;
    D.nSlots = n;
    D.slotsW = f.slotsW;
    D.slotsH = f.slotsH;
    D.gridW = f.gridW;
    D.gridH = f.gridH;
    D.cell = f.spacing;
    D.inv = 1.0f / f.spacing;
    D.width = f.width;
    D.height = f.height;
    D.K = K;
    D.gen = reinterpret_cast<float2 *>(ptrs[0]);
    D.m = reinterpret_cast<float2 *>(ptrs[1]);
    D.v = reinterpret_cast<float2 *>(ptrs[2]);
    D.gradX = reinterpret_cast<long long *>(ptrs[3]);
    D.key = reinterpret_cast<int *>(ptrs[4]);
    D.rank = reinterpret_cast<int *>(ptrs[5]);
    D.sortedIdx = reinterpret_cast<int *>(ptrs[6]);
    D.sortedPos = reinterpret_cast<float2 *>(ptrs[7]);
    D.counts = reinterpret_cast<int *>(ptrs[8]);
    D.start = reinterpret_cast<int *>(ptrs[9]);
    D.tileState = reinterpret_cast<unsigned long long *>(ptrs[10]);
    f.traw = reinterpret_cast<float2 *>(ptrs[11]);
    int *tkey = reinterpret_cast<int *>(ptrs[12]), *trank = reinterpret_cast<int *>(ptrs[13]);
    D.tpos = reinterpret_cast<float2 *>(ptrs[14]);
    D.tslot = reinterpret_cast<int *>(ptrs[15]);
    D.state = b->states.p + id;
    D.fraction = f.params.sampleFraction;
    D.seed = f.params.seed;
    D.gradExp = 40 - floor_log2f(f.spacing);
    D.lossExp = 64 - 2 * floor_log2f(f.spacing);
    D.active = 1;
    // BeginSchedule(params.iterations) over all slots (reference voro_optimizer.cu:652-687)
    D.lr = f.params.lrPerSpacing * f.spacing;
    D.gamma = f.params.gamma;
    D.beta1 = 0.9f;
    D.beta2 = 0.999f;
    D.eps = 1e-8f;
    for (int k = 0; k < 4; ++k) D.milestones[k] = f.params.milestones[k];
    D.cx0 = 0;
    D.cy0 = 0;
    D.cx1 = f.slotsW;
    D.cy1 = f.slotsH;
    float margin = 2.0f * f.spacing;
    D.bx0 = 0.0f * f.slotCellSize - margin;
    D.by0 = 0.0f * f.slotCellSize - margin;
    D.bx1 = (float)f.slotsW * f.slotCellSize + margin;
    D.by1 = (float)f.slotsH * f.slotCellSize + margin;
    f.sites = VmPointSet{D.gen, n, f.gridW, f.gridH, D.inv, D.key, D.rank, D.counts, D.start, nullptr,
                         D.sortedPos, D.sortedIdx, 1, 1};
    f.sites.tileState = D.tileState;
    f.tset = VmPointSet{f.traw, f.cap, f.gridW, f.gridH, D.inv, tkey, trank, D.counts, D.start, nullptr,
                        D.tpos, D.tslot, 0, 1};
    f.tset.tileState = D.tileState;
    cudaError_t e;
    if ((n && ((e = stage_copy(b, D.gen, in->generators, sizeof(float2) * n)) ||
               (e = cudaMemsetAsync(D.m, 0, 8 * (size_t)n, b->stream)) ||
               (e = cudaMemsetAsync(D.v, 0, 8 * (size_t)n, b->stream)) ||
               (e = cudaMemsetAsync(D.gradX, 0, 8 * kGradWords * (size_t)n, b->stream)))) ||
        (e = cudaMemsetAsync(D.counts, 0, 4 * ((size_t)f.cells + 1), b->stream)) ||
        (e = cudaMemsetAsync(D.tileState, 0, 8 * ((size_t)f.tiles + 1), b->stream)) ||
        (e = cudaMemsetAsync(D.state, 0, sizeof(VmState), b->stream)) ||
        (e = cudaMemsetAsync(f.traw, 0xFF, 8 * (size_t)f.cap, b->stream)) ||
        (in->nTargets && (e = stage_copy(b, f.traw, in->targets, 8 * (size_t)in->nTargets)))) {
        release_fit(b, f);
        return cuda_fail(e, "vmb_add_fit upload");
    }
    // targets sorted by (cell, 4x4 sub-cell) with temporary key arrays from the
    // arena; by cell alone, in the grid's arrays, if those do not fit
    int sub = 2;
    while (sub > 0 && ((long long)f.cells << (2 * sub)) > (1LL << 27)) --sub;
    long long keys = (long long)f.cells << (2 * sub);
    size_t tmpSizes[3] = {4 * (size_t)(keys + 1), 4 * (size_t)(keys + 1),
                          8 * (size_t)((keys + kScanTile - 1) / kScanTile + 1)};
    size_t tmpOff[3];
    int nTmp = 0;
    if (sub > 0)
        for (; nTmp < 3; ++nTmp)
            if (!b->arena.alloc(tmpSizes[nTmp], &tmpOff[nTmp])) break;
    auto releaseTmp = [&]() {
        for (int k = 0; k < nTmp; ++k) b->arena.release(tmpOff[k], tmpSizes[k]);
        nTmp = 0;
    };
    int *liveAt = D.start + f.cells;
    if (nTmp == 3) {
        f.tset.sub = sub;
        f.tset.counts = reinterpret_cast<int *>(b->arena.base + tmpOff[0]);
        f.tset.start = reinterpret_cast<int *>(b->arena.base + tmpOff[1]);
        f.tset.tileState = reinterpret_cast<unsigned long long *>(b->arena.base + tmpOff[2]);
        liveAt = f.tset.start + keys;
        if ((e = cudaMemsetAsync(f.tset.counts, 0, tmpSizes[0], b->stream)) ||
            (e = cudaMemsetAsync(f.tset.tileState, 0, tmpSizes[2], b->stream))) {
            releaseTmp();
            release_fit(b, f);
            return cuda_fail(e, "vmb_add_fit sort keys");
        }
    } else {
        releaseTmp();
    }
    int rc;
    if ((rc = single_set_build(b, f.tset, 0, 0))) {
        releaseTmp();
        release_fit(b, f);
        return rc;
    }
    if ((rc = b->block5Buf.reserve(1))) {
        releaseTmp();
        release_fit(b, f);
        return rc;
    }
    // the counts reach hcounts in stream order; the next table rebuild (or
    // fit query) syncs once for every fit added since (resolve_counts). The
    // temporary sort buffers go back to the arena now: whatever reuses them
    // is enqueued on the same stream, after these copies.
    int *slot = b->hcounts + 2 * id;
    if ((e = vm_launch_block5_max(f.tset.start, f.gridW, f.gridH, f.tset.sub, b->block5Buf.p, b->stream)) ||
        (e = cudaMemcpyAsync(slot, liveAt, sizeof(int), cudaMemcpyDeviceToHost, b->stream)) ||
        (e = cudaMemcpyAsync(slot + 1, b->block5Buf.p, sizeof(int), cudaMemcpyDeviceToHost, b->stream))) {
        releaseTmp();
        release_fit(b, f);
        return cuda_fail(e, "vmb_add_fit live targets");
    }
    releaseTmp();
    f.countsPending = true;
    if ((rc = single_set_build(b, f.sites, 1, 1))) { // the grid of the initial generators
        release_fit(b, f);
        return rc;
    }
    f.live = true;
    b->dirty = true;
    *fitId = id;
    return VM_OK;
}

int vmb_remove_fit(vmb_batch *b, int fitId)
{
    if (!b || fitId < 0 || fitId >= (int)b->fits.size() || !b->fits[fitId].live)
        return fail(VM_ERR_ARG, "vmb_remove_fit: no such fit");
    cudaStreamSynchronize(b->stream);
    release_fit(b, b->fits[fitId]);
    b->dirty = true;
    return VM_OK;
}

int vmb_set_active(vmb_batch *b, int fitId, int active)
{
    if (!b || fitId < 0 || fitId >= (int)b->fits.size() || !b->fits[fitId].live)
        return fail(VM_ERR_ARG, "vmb_set_active: no such fit");
    b->fits[fitId].done = !active;
    b->dirty = true;
    return VM_OK;
}

int vmb_step(vmb_batch *b, int iterations, float *gpuMs)
{
    vmh::NvtxRange range("vmb_step");
    if (!b || iterations < 0) return fail(VM_ERR_ARG, "vmb_step: bad arguments");
    if (gpuMs) *gpuMs = 0.0f;
    int rc;
    if (b->dirty && (rc = rebuild_tables(b))) return rc;
    if (b->order.empty() || iterations == 0) return VM_OK;
    if ((rc = ensure_batch_graph(b))) return rc;
    cudaError_t e;
    if ((e = cudaEventRecord(b->ev0, b->stream))) return cuda_fail(e, "event");
    for (int k = 0; k < iterations; ++k)
        if ((e = cudaGraphLaunch(b->graph, b->stream))) return cuda_fail(e, "batch graph launch");
    if ((e = cudaEventRecord(b->ev1, b->stream)) || (e = cudaEventSynchronize(b->ev1))) return cuda_fail(e, "event");
    float ms = 0;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    if (gpuMs) *gpuMs = ms;
    return VM_OK;
}

int vmb_evaluate(vmb_batch *b, float *losses)
{
    if (!b) return fail(VM_ERR_ARG, "vmb_evaluate: bad arguments");
    int rc;
    if (b->dirty && (rc = rebuild_tables(b))) return rc;
    int nf = (int)b->order.size();
    if (nf) {
        cudaError_t e;
        if ((e = vm_launch_loss(b->dFits.p, b->dPre.p + 2 * (nf + 1), nf, b->lossTiles, 1, b->lossGrid,
                                b->lossVariant, 0, b->queue.p, b->stream)) ||
            (e = vm_launch_finalize(b->dFits.p, nf, b->queue.p, b->stream)))
            return cuda_fail(e, "batch evaluate");
    }
    if ((rc = read_states(b))) return rc;
    if (losses)
        for (int id = 0; id < (int)b->fits.size(); ++id) {
            const VmState &s = b->hostStates[id];
            losses[id] = s.count > 0 ? s.loss / (float)s.count : 0.0f;
        }
    return VM_OK;
}

int vmb_fit_info(vmb_batch *b, int fitId, vmb_fit_info_t *out)
{
    if (!b || !out || fitId < 0 || fitId >= (int)b->fits.size() || !b->fits[fitId].live)
        return fail(VM_ERR_ARG, "vmb_fit_info: no such fit");
    int rc;
    if ((rc = resolve_counts(b)) || (rc = read_states(b))) return rc;
    const VmState &s = b->hostStates[fitId];
    out->iteration = s.iter;
    out->lastLoss = s.count > 0 ? s.loss / (float)s.count : 0.0f;
    out->numSlots = b->fits[fitId].n;
    out->liveTargets = b->fits[fitId].liveTargets;
    out->active = !b->fits[fitId].done;
    return VM_OK;
}

int vmb_get_generators(vmb_batch *b, int fitId, float *xy)
{
    if (!b || !xy || fitId < 0 || fitId >= (int)b->fits.size() || !b->fits[fitId].live)
        return fail(VM_ERR_ARG, "vmb_get_generators: no such fit");
    const BFit &f = b->fits[fitId];
    if (!f.n) return VM_OK;
    cudaError_t e = cudaMemcpyAsync(xy, f.desc.gen, sizeof(float2) * f.n, cudaMemcpyDeviceToHost, b->stream);
    if (!e) e = cudaStreamSynchronize(b->stream);
    if (e) return cuda_fail(e, "vmb_get_generators");
    return VM_OK;
}

int vmb_memory(vmb_batch *b, size_t *freeBytes, size_t *totalBytes, int *liveFits)
{
    if (!b) return fail(VM_ERR_ARG, "NULL batch");
    if (freeBytes) *freeBytes = b->arena.freeBytes();
    if (totalBytes) *totalBytes = b->arena.cap;
    if (liveFits) {
        int c = 0;
        for (auto &f : b->fits) c += f.live;
        *liveFits = c;
    }
    return VM_OK;
}

// ---------------------------------------------------------------------------
// serving loop
// ---------------------------------------------------------------------------
} // extern "C"

namespace {

// Every fit's loss per target from its last step's loss pass.
int step_losses(vmb_batch *b, float *losses)
{
    int rc;
    if ((rc = read_states(b))) return rc;
    for (int id = 0; id < (int)b->fits.size(); ++id) {
        const VmState &s = b->hostStates[id];
        losses[id] = s.count > 0 ? s.loss / (float)s.count : 0.0f;
    }
    return VM_OK;
}

} // namespace

extern "C" {

int vms_serve(const vms_request *reqs, int n, const vms_config *cfg, vms_result *res)
{
    vmh::NvtxRange range("vms_serve");
    if (n < 0 || (n && (!reqs || !res)) || !cfg || cfg->stepsPerRound < 1 || cfg->maxLive < 1)
        return fail(VM_ERR_ARG, "vms_serve: bad arguments");
    vmb_batch *b = nullptr;
    int rc = vmb_create(cfg->hbmBudgetBytes, std::max(cfg->maxLive, 1), cfg->lossVariant, &b);
    if (rc) return rc;
    using clk = std::chrono::steady_clock;
    auto t0 = clk::now();
    auto now = [&]() { return std::chrono::duration<double>(clk::now() - t0).count(); };
    std::vector<int> pending(n);
    for (int i = 0; i < n; ++i) pending[i] = i;
    std::stable_sort(pending.begin(), pending.end(), [&](int a, int c) { return reqs[a].arrival < reqs[c].arrival; });
    for (int i = 0; i < n; ++i) {
        res[i] = vms_result{};
        res[i].arrival = reqs[i].arrival;
        res[i].status = -1;
    }
    std::vector<int> liveReq(b->maxFits, -1); // fit id -> request
    std::vector<float> prevLoss(b->maxFits, -1.0f), losses(b->maxFits, 0.0f);
    std::vector<int> steps(b->maxFits, 0);
    size_t head = 0, liveTargets = 0;
    int done = 0, live = 0;
    auto targetsOf = [&](int r) { return (size_t)std::max(reqs[r].fit.nTargets, 0); };
    while (done < n) {
        // admit every arrived request that fits (FIFO; the head waits for memory
        // and, under a target cap, for live work to retire)
        while (head < pending.size() && reqs[pending[head]].arrival <= now() && live < cfg->maxLive &&
               (live == 0 || cfg->maxLiveTargets == 0 ||
                liveTargets + targetsOf(pending[head]) <= cfg->maxLiveTargets)) {
            int r = pending[head], id = -1;
            rc = vmb_add_fit(b, &reqs[r].fit, &id);
            if (rc == VM_ERR_BUDGET) {
                if (live == 0) { // can never fit: reject
                    res[r].status = VM_ERR_BUDGET;
                    res[r].finished = now();
                    ++done;
                    ++head;
                    continue;
                }
                break;
            }
            if (rc == VM_ERR_ARG || rc == VM_ERR_UNSUPPORTED) { // a bad request: rejected, the rest served
                res[r].status = rc;
                res[r].finished = now();
                ++done;
                ++head;
                continue;
            }
            if (rc) {
                vmb_destroy(b);
                return rc;
            }
            res[r].admitted = now();
            liveTargets += targetsOf(r);
            liveReq[id] = r;
            prevLoss[id] = -1.0f;
            steps[id] = 0;
            ++live;
            ++head;
        }
        if (live == 0) {
            if (head < pending.size()) {
                double wait = reqs[pending[head]].arrival - now();
                if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(wait));
            }
            continue;
        }
        // step all live fits together, then test each against its full-target loss:
        // the loss pass of the round's last step when every target counts every
        // step (sampleFraction 1), else a separate full-target evaluation
        bool evaluate = false;
        for (int id = 0; id < (int)liveReq.size(); ++id)
            if (liveReq[id] >= 0 && reqs[liveReq[id]].fit.params.sampleFraction < 1.0f) evaluate = true;
        if ((rc = vmb_step(b, cfg->stepsPerRound, nullptr)) ||
            (rc = evaluate ? vmb_evaluate(b, losses.data()) : step_losses(b, losses.data()))) {
            vmb_destroy(b);
            return rc;
        }
        for (int id = 0; id < (int)liveReq.size(); ++id) {
            int r = liveReq[id];
            if (r < 0) continue;
            steps[id] += cfg->stepsPerRound;
            float L = losses[id], P = prevLoss[id];
            bool converged = P >= 0.0f && L > 0.0f && std::fabs(L - P) / L < reqs[r].relTol;
            if (steps[id] >= reqs[r].maxSteps || converged) {
                if (reqs[r].outGenerators) vmb_get_generators(b, id, reqs[r].outGenerators);
                res[r].finished = now();
                res[r].steps = steps[id];
                res[r].finalLoss = L;
                res[r].status = VM_OK;
                vmb_remove_fit(b, id);
                liveTargets -= targetsOf(r);
                liveReq[id] = -1;
                --live;
                ++done;
            } else {
                prevLoss[id] = L;
            }
        }
    }
    vmb_destroy(b);
    return VM_OK;
}

} // extern "C"
