/*
 * vm_capi.h — C ABI of libvoromesh_gb300.so: the GB300 VoroMesh optimiser
 * (vm_*), Voronoi extraction, the Poisson-disk sampler (pd_*), the voxel
 * canvas (cv_*), and many fits at once (vmb_* batches, vms_serve).
 *
 * The reference exposes this path as C++ classes
 * (voromesh::VoroOptimizer, include/voromesh/voro_optimizer.h:70-138,
 * poisson::Sampler, include/poisson/poisson_disk.h:21-62, and the host-side
 * voromesh::Canvas, include/voromesh/canvas.h:25-89). Each vm_* / pd_* / cv_*
 * entry point below is one of their methods, flattened to plain pointers and
 * sizes: float pairs are (x, y) interleaved like Vec2 / Sample / float2, and
 * every host buffer is copied before the call returns, as the reference's
 * synchronous cudaMemcpy calls do. The library also implements the two C++
 * classes on top of these functions (include/voromesh, include/poisson).
 *
 * Every function returns VM_OK (0) or one of the VM_ERR_* codes; the message
 * of the last failure on the calling thread is available from
 * vm_last_error(). The C++ classes turn a non-zero status into the
 * reference's behaviour (message on stderr, exit(1)).
 *
 * Threading follows the reference: one handle is not thread-safe; separate
 * handles are independent. Each optimiser owns a non-blocking CUDA stream.
 */
#ifndef VM_CAPI_H
#define VM_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    VM_OK = 0,
    VM_ERR_ARG = 1,         /* invalid argument or size */
    VM_ERR_OOM = 2,         /* device or host allocation failed */
    VM_ERR_CUDA = 3,        /* CUDA runtime or kernel error */
    VM_ERR_STATE = 4,       /* call not valid in the current state */
    VM_ERR_BUDGET = 5,      /* request exceeds the memory budget (batch / serving) */
    VM_ERR_TIMEOUT = 6,     /* a bounded wait gave up */
    VM_ERR_UNSUPPORTED = 7, /* parameter outside what the kernels implement */
    VM_ERR_NODEVICE = 8     /* no CUDA device */
};

const char *vm_error_string(int code);
/* Copies the last failure message of this thread into buf (NUL-terminated). */
int vm_last_error(char *buf, int len);
/* Library version and the compute capability it was built for (e.g. 103). */
int vm_version(int *major, int *minor, int *sm);

/* ---- VoroMesh optimiser (voromesh::VoroOptimizer) ---------------------------- */

/* OptimizerParams (include/voromesh/voro_optimizer.h:34-44) plus the kNN size
 * of the loss, a compile-time constant (kLossK = 12) in the reference
 * (src/voromesh/voro_optimizer.cu:54). Supported lossK: 8, 12, 16, 24, 32. */
typedef struct {
    int iterations;      /* 400 */
    int localIterations; /* 100 */
    float lrPerSpacing;  /* 0.09 */
    float sampleFraction;/* 0.2 */
    float gamma;         /* 0.5 */
    int milestones[4];   /* 80 150 200 250 */
    unsigned seed;       /* 1 */
    int lossK;           /* 12 */
} vm_params;

typedef struct vm_optimizer vm_optimizer;

typedef struct {
    int iteration;        /* Iteration() */
    int scheduleLength;   /* ScheduleLength() */
    int numSlots;         /* NumSlots() */
    int targetCapacity;   /* target slots allocated */
    int liveTargets;      /* targets with x >= 0 */
    int gridW, gridH;     /* hash grid */
    float lastBatchLoss;  /* LastBatchLoss() */
    long long exactTargets; /* targets resolved by the exact ring search so far */
} vm_info_t;

typedef struct {
    int numGenerators;  /* slots */
    int numCellVerts;   /* CSR vertices of all cells */
    int numVertices;    /* boundary vertices */
    int numEdges;       /* boundary edges */
    int watertight, loops, unsafeCells, overflowCells;
    float gpuMs, hostMs;
} vm_mesh_info;

/* OptimizerParams{} defaults */
void vm_params_default(vm_params *p);
/* VoroOptimizer(width, height, spacing, params)  voro_optimizer.h:75 */
int vm_create(float width, float height, float spacing, const vm_params *params, vm_optimizer **out);
/* ~VoroOptimizer()  voro_optimizer.h:76 */
int vm_destroy(vm_optimizer *h);
/* SetTargets(slots)  voro_optimizer.h:82; xy holds n (x,y) pairs */
int vm_set_targets(vm_optimizer *h, const float *xy, int n);
/* UpdateTargets(dirty, slots)  voro_optimizer.h:84 */
int vm_update_targets(vm_optimizer *h, const int *dirty, int ndirty, const float *slots, int nslots);
/* SetOccupancy(masks, tilesX, tilesY, voxelSize)  voro_optimizer.h:87 */
int vm_set_occupancy(vm_optimizer *h, const uint64_t *masks, int tilesX, int tilesY, float voxelSize);
/* UpdateOccupancy(masks, tx0, ty0, tx1, ty1)  voro_optimizer.h:89 */
int vm_update_occupancy(vm_optimizer *h, const uint64_t *masks, int tx0, int ty0, int tx1, int ty1);
/* SetGenerators(slots, slotsW, slotsH, slotCellSize)  voro_optimizer.h:94 */
int vm_set_generators(vm_optimizer *h, const float *xy, int slotsW, int slotsH, float slotCellSize);
/* UpdateGenerators(slots, cx0, cy0, cx1, cy1)  voro_optimizer.h:96 */
int vm_update_generators(vm_optimizer *h, const float *xy, int cx0, int cy0, int cx1, int cy1);
/* BeginSchedule(iterations, cx0, cy0, cx1, cy1)  voro_optimizer.h:102 */
int vm_begin_schedule(vm_optimizer *h, int iterations, int cx0, int cy0, int cx1, int cy1);
/* Step(iterations) -> GPU ms  voro_optimizer.h:106 */
int vm_step(vm_optimizer *h, int iterations, float *gpuMs);
/* Step(iterations) run kernel by kernel with CUDA events between the stages;
 * stageMs[4] receives the mean ms per step of: loss (fast path + exact
 * queue), Adam + binning, cell-count scan, cell-sorted scatter. An addition
 * (no counterpart in the reference) used to attribute step time. */
int vm_step_timed(vm_optimizer *h, int iterations, float *stageMs);
/* Loss-kernel variant (block size, occupancy target): -1 = automatic. All
 * variants produce identical results; the autotuner times them at a fit's
 * first Step and keeps the fastest per fit-size bucket (power of two of live
 * targets). Additions, no reference counterpart. */
int vm_set_loss_variant(vm_optimizer *h, int variant);
int vm_get_loss_variant(vm_optimizer *h, int *variant, int *count);
/* EvaluateLoss()  voro_optimizer.h:113 */
int vm_evaluate_loss(vm_optimizer *h, float *loss);
/* Iteration / ScheduleLength / NumSlots / LastBatchLoss  voro_optimizer.h:111,118-120 */
int vm_info(vm_optimizer *h, vm_info_t *out);
/* Current generator slots (numSlots pairs). */
int vm_get_generators(vm_optimizer *h, float *xy);
/* Adam moments (numSlots pairs each; either may be NULL). */
int vm_get_moments(vm_optimizer *h, float *m, float *v);
/* Extract()  voro_optimizer.h:116: runs the clipper and boundary assembly and
 * keeps the result in the handle; sizes in *info, arrays via vm_mesh_copy. */
int vm_extract(vm_optimizer *h, vm_mesh_info *info);
/* Copies the last Extract(): generators (2n), inside (n), cellStart (n+1),
 * cellVerts (2 numCellVerts), vertices (2 numVertices), edges (2 numEdges);
 * cellLabels (numCellVerts edge labels) is an addition. Any may be NULL. */
int vm_mesh_copy(vm_optimizer *h, float *generators, uint8_t *inside, int *cellStart, float *cellVerts,
                 float *vertices, int *edges, int *cellLabels);

/* ---- checkpoint / resume (no counterpart in the reference) -------------------- */
/* The optimisation state of a fit, beside its generators and Adam moments:
 * the slot layout, the current schedule (BeginSchedule's length and slot
 * rectangle), the step counter and the last batch loss. */
typedef struct {
    int slotsW, slotsH;
    float slotCellSize;
    int scheduleLength, iteration;
    int cx0, cy0, cx1, cy1;
    float lastBatchLoss;
} vm_checkpoint_info;
/* Snapshot: info plus numSlots (x, y) pairs each of generators, m and v (any
 * array may be NULL). */
int vm_checkpoint(vm_optimizer *h, vm_checkpoint_info *info, float *gen, float *m, float *v);
/* Resume into an optimiser made with the same constructor arguments and the
 * same targets and occupancy: SetGenerators + BeginSchedule of the saved
 * schedule, then the saved moments and step counter. The next Step continues
 * the saved run bit for bit. */
int vm_restore(vm_optimizer *h, const vm_checkpoint_info *info, const float *gen, const float *m, const float *v);

/* ---- inspection (used by the parity tests) ----------------------------------- */
/* The hash grid of the current generators: start (gridW*gridH+1), sortedIdx and
 * sortedPos (live sites, cell order, ascending slot within a cell), genCell (numSlots). */
int vm_get_grid(vm_optimizer *h, int *start, int *sortedIdx, float *sortedPos, int *genCell);
/* Exact K nearest generators (K in 8,12,16,24,32) of nq query points, (d2, index) order. */
int vm_knn(vm_optimizer *h, const float *queries, int nq, int K, int *idx, float *d2);
/* One loss pass without moving anything. mode 0: the next Step's pass (active
 * box, subsample, gradient); mode 1: EvaluateLoss's pass. Per target slot
 * (targetCapacity entries, any may be NULL): nearest site, bisector
 * neighbour, loss (-1/-1/0 when unused). grad: 2*numSlots summed gradient
 * (mode 0). count, lossSum: the pass totals. */
int vm_probe(vm_optimizer *h, int mode, int *i0, int *j, float *loss, float *grad, int *count, float *lossSum);

/* ---- batched fits --------------------------------------------------------------
 * No counterpart in the reference, which runs one VoroOptimizer at a time
 * (apps/voromesh_demo.cpp:103-156). A batch holds independent fits of any
 * sizes in one device arena (its size is the HBM budget) and steps all of
 * them together: each stage of a step is one launch over all live fits.
 * A fit's results do not depend on the other fits in the batch (exact
 * fixed-point sums), so they equal what a VoroOptimizer computes alone. */
typedef struct vmb_batch vmb_batch;
typedef struct {
    float width, height, spacing; /* VoroOptimizer(width, height, spacing, params) */
    vm_params params;             /* the schedule is BeginSchedule(params.iterations) over all slots */
    const float *generators;      /* SetGenerators(generators, slotsW, slotsH, slotCellSize) */
    int slotsW, slotsH;
    float slotCellSize;
    const float *targets;         /* SetTargets(targets[0..nTargets)) */
    int nTargets;
} vmb_fit;
typedef struct {
    int iteration;   /* steps taken */
    float lastLoss;  /* loss / count of the last published pass */
    int numSlots, liveTargets, active;
} vmb_fit_info_t;

int vmb_create(size_t arenaBytes, int maxFits, int lossVariant, vmb_batch **out);
int vmb_destroy(vmb_batch *b);
/* Arena bytes a fit of this shape needs (admission control). */
size_t vmb_fit_bytes(int slotsW, int slotsH, int nTargets, float width, float height, float spacing);
/* Uploads a fit (copies the host buffers); VM_ERR_BUDGET when it does not fit the arena. */
int vmb_add_fit(vmb_batch *b, const vmb_fit *fit, int *fitId);
int vmb_remove_fit(vmb_batch *b, int fitId);
/* Inactive fits keep their memory but are not stepped. */
int vmb_set_active(vmb_batch *b, int fitId, int active);
/* `iterations` steps of every active fit; GPU ms of the whole run. It reads
 * nothing back: a fit's kernel error bits surface as VM_ERR_CUDA at the next
 * vmb_evaluate or vmb_fit_info. */
int vmb_step(vmb_batch *b, int iterations, float *gpuMs);
/* EvaluateLoss() of every active fit; losses[fitId] (maxFits entries). */
int vmb_evaluate(vmb_batch *b, float *losses);
int vmb_fit_info(vmb_batch *b, int fitId, vmb_fit_info_t *out);
int vmb_get_generators(vmb_batch *b, int fitId, float *xy);
int vmb_memory(vmb_batch *b, size_t *freeBytes, size_t *totalBytes, int *liveFits);

/* ---- serving: continuous batching of arriving fit requests -----------------------
 * Requests become visible at their arrival time (seconds after the call
 * starts). Arrived requests are admitted in arrival order while the HBM
 * budget and `maxLive` allow; all live fits step together, `stepsPerRound`
 * steps at a time; after each round every live fit's full-target loss is
 * taken (the loss pass of the round's last step when every live fit uses
 * sampleFraction 1, else a separate evaluation pass) and the fit retires
 * when it has taken maxSteps steps or its loss changed by less than relTol
 * (relative) since the previous round. A
 * retired fit's generators are copied to outGenerators (when non-NULL) and
 * its memory admits the next request. maxLive = 1 is the one-fit-at-a-time
 * loop. Times in vms_result are seconds since the call started. */
typedef struct {
    double arrival;
    vmb_fit fit;
    int maxSteps;
    float relTol;
    float *outGenerators; /* slotsW*slotsH (x,y) pairs, or NULL */
} vms_request;
typedef struct {
    size_t hbmBudgetBytes;
    int maxLive;
    int stepsPerRound;
    int lossVariant;       /* -1 = default */
    size_t maxLiveTargets; /* admit while the live fits' targets stay within this (0 = no cap); a
                              cap keeps the GPU busy while letting early requests finish sooner */
} vms_config;
typedef struct {
    double arrival, admitted, finished;
    int steps;
    float finalLoss;
    int status; /* VM_OK, or VM_ERR_BUDGET when the fit can never fit */
} vms_result;
int vms_serve(const vms_request *reqs, int n, const vms_config *cfg, vms_result *results);

/* ---- allocation-free hash-grid build --------------------------------------------
 * No counterpart in the reference. For callers that cannot let a library
 * allocate device memory (a per-frame edit loop where cudaMalloc's implicit
 * synchronisation would stall the frame, or a host that plans all device
 * memory itself): builds the cell-sorted hash grid of `n` generators
 * (device float2 array, x < 0 = empty slot) into caller-owned device arrays
 * start (gridW*gridH+1 ints), sortedIdx (n ints) and sortedPos (2n floats),
 * bit-identical to vm_get_grid's. Nothing is allocated: the scratch lives in
 * a fixed __device__ array of the library (about 3 MB per device, held until
 * exit) sized for at most VM_NOALLOC_MAX_POINTS generators and
 * VM_NOALLOC_MAX_CELLS cells; larger requests return VM_ERR_ARG. Work is
 * enqueued on `stream` (a cudaStream_t, NULL = the legacy default stream)
 * and the call returns without waiting. The first call on a device sets up
 * that device's scratch address; make it before any stream capture (a first
 * call on a capturing stream returns VM_ERR_UNSUPPORTED). A cudaDeviceReset
 * invalidates that address; the next call after a failed launch looks it up
 * again. All calls share the scratch array: calls that overlap on the GPU
 * race, so the caller must order them (one stream, or events). */
#define VM_NOALLOC_MAX_POINTS 262144
#define VM_NOALLOC_MAX_CELLS 262144
int vm_build_grid_noalloc(const float *generators, int n, int gridW, int gridH, float cellSize, int *start,
                          int *sortedIdx, float *sortedPos, void *stream);

/* ---- Poisson-disk sampler (poisson::Sampler) ---------------------------------- */
typedef struct pd_sampler pd_sampler;
typedef struct {
    float width, height, radius, cellSize;
    int gridW, gridH, trials;
    unsigned seed, roundBase;
} pd_info_t;

/* Sampler(width, height, radius, trials, seed): fills the whole domain  poisson_disk.h:24 */
int pd_create(float width, float height, float radius, int trials, unsigned seed, pd_sampler **out);
int pd_destroy(pd_sampler *s);
/* Resample(cx0, cy0, cx1, cy1) -> GPU ms  poisson_disk.h:33 */
int pd_resample(pd_sampler *s, int cx0, int cy0, int cx1, int cy1, float *gpuMs);
/* Resample(regions[4i..4i+3]) of n distinct samplers at once: each small
 * region (every phase in one pass of a block) runs as one block of a single
 * launch, larger ones as pd_resample. Same samples as n pd_resample calls.
 * An addition, no reference counterpart. */
int pd_resample_many(pd_sampler *const *samplers, const int *regions, int n, float *gpuMs);
/* Width/Height/Radius/CellSize/GridW/GridH/Trials  poisson_disk.h:44-50 */
int pd_info(pd_sampler *s, pd_info_t *out);
/* Cells(): gridW*gridH (x,y) pairs, x < 0 = empty  poisson_disk.h:41 */
int pd_cells(pd_sampler *s, float *xy);
/* Verify(cx0, cy0, cx1, cy1)  poisson_disk.h:37 */
int pd_verify(pd_sampler *s, int cx0, int cy0, int cx1, int cy1, int *ok);
/* Number of samples in the grid. */
int pd_count(pd_sampler *s, long long *n);

/* --------------------------------------------------------------------------
 * Canvas: the authoritative 2D shape, device-resident (voromesh::Canvas,
 * include/voromesh/canvas.h:25-89, src/voromesh/canvas.cpp). Voxel (i, j)
 * covers [i, i+1) x [j, j+1) * voxelSize; 8x8 voxels form a tile and voxel
 * (i, j) is bit (j & 7) * 8 + (i & 7) of its tile's word. Occupancy is a dense
 * row-major array of tile words; the surface (one mean boundary point and one
 * target slot per surface voxel) is dense per voxel on the device. The target
 * slot array (TargetSlots) lives on the device; {-1, -1} marks a free slot.
 *
 * Results equal the reference's Canvas on the same inputs, with one stated
 * difference: a stamp's new rim voxels take their slots from the free list in
 * tile-major voxel order, where the reference uses std::unordered_map order
 * (canvas.cpp:200). Slot indices can therefore differ by a relabelling; every
 * value, mask, point and count is the same.
 * ------------------------------------------------------------------------ */
typedef struct cv_canvas cv_canvas;

typedef struct {
    int tx0, ty0, tx1, ty1;     /* occupancy tiles [tx0,tx1) x [ty0,ty1) rewritten */
    int removed, added, flipped; /* surface samples, occupancy voxels */
    int ndirty;                 /* target slots whose value changed (cv_edit_dirty) */
} cv_edit;

typedef struct {
    int voxelsX, voxelsY, tilesX, tilesY;
    float voxelSize;
    int numSlots, freeSlots;   /* TargetSlots().size(); free-list length */
    long long surfaceCount;    /* Canvas::SurfaceCount */
    int surfaceTiles;          /* Canvas::SurfaceTileCount */
} cv_info_t;

/* Canvas(width, height, voxelSize) (canvas.cpp:33-38) */
int cv_create(float width, float height, float voxelSize, cv_canvas **out);
int cv_destroy(cv_canvas *c);
/* RasterizeShape(polygon) (canvas.cpp:71-134); n vertices (x, y), closed
 * implicitly. gpuMs (optional) = device time of the call. At most 131072
 * voxels per row and 32768 edge crossings on one scanline. */
int cv_rasterize(cv_canvas *c, const float *xy, int n, float *gpuMs);
/* StampDisc(center, radius, inside) (canvas.cpp:136-221) */
int cv_stamp_disc(cv_canvas *c, float cx, float cy, float radius, int inside, cv_edit *out);
/* The last edit's dirty slots (Edit::dirtySlots) and their new values
 * (x, y pairs; may be NULL); cap = room in the buffers. */
int cv_edit_dirty(cv_canvas *c, int *dirty, float *values, int cap);
int cv_info(cv_canvas *c, cv_info_t *out);
/* TargetSlots(): numSlots (x, y) pairs */
int cv_get_slots(cv_canvas *c, float *xy);
/* InsideMasks(): tilesX * tilesY words */
int cv_get_inside(cv_canvas *c, uint64_t *masks);
/* The words of tiles [tx0,tx1) x [ty0,ty1) only, into a tilesX * tilesY array */
int cv_get_inside_rect(cv_canvas *c, uint64_t *masks, int tx0, int ty0, int tx1, int ty1);
/* Dense surface state (each may be NULL): per tile its surface mask; per voxel
 * (tile-major, 64 per tile) its point and slot, (-1, -1) / -1 off the surface. */
int cv_get_surface(cv_canvas *c, uint64_t *masks, float *points, int *slots);
/* The free list, bottom to top (freeSlots entries) */
int cv_get_free(cv_canvas *c, int *freeList);
/* IsInside(i, j) / IsSurface(i, j) (canvas.cpp:40-49) */
int cv_is_inside(cv_canvas *c, int i, int j, int *out);
int cv_is_surface(cv_canvas *c, int i, int j, int *out);

/* Device-to-device hand-off from a canvas to an optimiser on the same GPU:
 *   vm_set_targets_from_canvas = SetTargets(TargetSlots()) followed by
 *     SetOccupancy(InsideMasks(), TilesX(), TilesY(), VoxelSize());
 *   vm_update_from_canvas = UpdateTargets(edit.dirtySlots, TargetSlots())
 *     followed by UpdateOccupancy(InsideMasks(), edit tile rectangle) for the
 *     canvas's last edit (the editor's sequence, apps/voromesh_demo.cpp:124-125).
 * No data passes through the host. */
int vm_set_targets_from_canvas(vm_optimizer *h, cv_canvas *c);
int vm_update_from_canvas(vm_optimizer *h, cv_canvas *c);

#ifdef __cplusplus
}
#endif

#endif
