/*
 * vm_oracle — CPU restatement of the reference's VoroMesh and Poisson paths.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker: it is loaded by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, never
 * by the product library or its Python package.
 *
 * Each function restates the reference's code in plain C (no FP contraction,
 * IEEE float ops in the reference's order) and cites the file:line it follows
 * (paths relative to the reference project root):
 *   src/voromesh/voro_optimizer.cu   hash grid, kNN, VoroLoss, Adam, clipper,
 *                                    boundary assembly
 *   src/poisson/poisson_disk.cu      phase-grid dart throwing
 *
 * Two accumulation modes exist for the loss/gradient sums:
 *   VO_ACC_REF    float sums in target-index order, as a serial execution of
 *                 the reference kernel produces (its GPU order is racy);
 *   VO_ACC_FIXED  the product's order-independent fixed-point sums (exact
 *                 split 64-bit word pairs per gradient component, 128-bit for
 *                 the loss), restated here independently so the GPU path can
 *                 be checked bit-exact.
 * Two bias-correction modes exist for Adam:
 *   VO_POW_REF    powf(beta, t) (reference voro_optimizer.cu:287-288);
 *   VO_POW_DET    double exponentiation by squaring rounded to float (the
 *                 product's platform-independent restatement of the same).
 */
#ifndef VM_ORACLE_H
#define VM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    float x, y;
} vo_f2;

enum { VO_ACC_REF = 0, VO_ACC_FIXED = 1 };
enum { VO_POW_REF = 0, VO_POW_DET = 1 };

/* RunParams (voro_optimizer.cu:88-95) */
typedef struct {
    float lr, gamma, beta1, beta2, eps;
    int milestones[4];
    float width, height;
    int slotsW;
    int cx0, cy0, cx1, cy1;
    float bx0, by0, bx1, by1;
} vo_run_params;

/* Cell-sorted hash grid (voro_optimizer.cu:115-121). start has w*h+1 entries. */
typedef struct {
    int w, h;
    float cellSize;
    const int *start;
    const int *idx;
    const vo_f2 *pos;
} vo_grid;

/* ---- hash grid ------------------------------------------------------------ */
int vo_cell_coord(float v, float inv, int n);
/* binKernel + ExclusiveSum + scatterKernel (voro_optimizer.cu:168-187,689-700)
 * with the within-cell order fixed to ascending slot index. genCell gets -1
 * for empty slots. start: gw*gh+1 ints; sortedIdx/sortedPos: n entries. */
void vo_build_grid(const vo_f2 *gen, int n, int gw, int gh, float cellSize, int *genCell, int *start,
                   int *sortedIdx, vo_f2 *sortedPos);

/* ---- kNN ------------------------------------------------------------------ */
/* knn<K> ring search (voro_optimizer.cu:130-163); ties ordered by site index. */
void vo_knn(const vo_grid *g, vo_f2 q, int K, int *idx, float *d2);
/* vo_knn for n queries (row i of idx / d2 for query i), split over nthreads threads. */
void vo_knn_many(const vo_grid *g, const vo_f2 *q, int n, int K, int *idx, float *d2, int nthreads);
/* Exhaustive K nearest by (d2, index) over all live slots (a test aid). */
void vo_knn_brute(const vo_f2 *gen, int n, vo_f2 q, int K, int *idx, float *d2);

/* ---- VoroLoss ----------------------------------------------------------------
 * vorolossKernel (voro_optimizer.cu:199-266) over all targets. rp may be NULL
 * (EvaluateLoss). grad (REF mode: float2[n]) or gradFixed (FIXED mode:
 * int64[4n], per site the words L.x, L.y, H.x, H.y of vo_fixed2_add) may be
 * NULL for a loss-only pass. Outputs the summed loss and the number of
 * contributing targets. nthreads > 1 only in FIXED mode. */
typedef struct {
    float loss;      /* float sum (REF) or the rounded fixed-point sum (FIXED) */
    int count;
    uint64_t lossLo, lossHi; /* FIXED mode 128-bit accumulator */
} vo_loss_sum;

void vo_loss(const vo_f2 *targets, int numTargets, const vo_grid *g, const vo_f2 *gen, int n, int K,
             const vo_run_params *rp, float fraction, unsigned seed, unsigned iter, int accMode, float spacing,
             float *grad, int64_t *gradFixed, vo_loss_sum *out, int nthreads);

/* Per-target record of the VoroLoss decision (a test aid): nearest site,
 * chosen bisector neighbour and loss, or -1/-1/0 when the target is unused. */
void vo_loss_detail(const vo_f2 *targets, int numTargets, const vo_grid *g, const vo_f2 *gen, int K,
                    const vo_run_params *rp, float fraction, unsigned seed, unsigned iter, int *i0, int *bestJ,
                    float *loss);

/* ---- fixed-point helpers (product accumulation, restated) ----------------- */
int vo_fixed_grad_exp(float spacing);
int vo_fixed_loss_exp(float spacing);
int64_t vo_fixed_from_float(float v, int e);
float vo_fixed_to_float(int64_t v, int e);
/* exact split sums: add v to (H, L); S = H * 2^32 + L rounded once to float, times 2^-e */
void vo_fixed2_add(int64_t v, int64_t *H, uint64_t *L);
float vo_fixed2_to_float(int64_t H, uint64_t L, int e);
void vo_fixed_loss_add(float v, int e, uint64_t *lo, uint64_t *hi);
float vo_fixed_loss_to_float(uint64_t lo, uint64_t hi, int e);

/* ---- Adam --------------------------------------------------------------------
 * adamKernel (voro_optimizer.cu:271-301). gradFloat (REF) or gradFixed
 * (FIXED, 4 words per site, converted with vo_fixed2_to_float) is read and
 * zeroed. */
float vo_pow_det(float base, int t);
void vo_adam(vo_f2 *gen, vo_f2 *m, vo_f2 *v, float *gradFloat, int64_t *gradFixed, int gradExp, int n,
             int iter, int count, const vo_run_params *rp, int powMode, int nthreads);

/* ---- a whole optimiser (VoroOptimizer, voro_optimizer.cu:512-761) --------- */
typedef struct vo_fit vo_fit;

vo_fit *vo_fit_create(float width, float height, float spacing, int K, float lrPerSpacing, float sampleFraction,
                      float gamma, const int milestones[4], int paramIterations, unsigned seed, int accMode,
                      int powMode, int nthreads);
void vo_fit_destroy(vo_fit *f);
void vo_fit_set_targets(vo_fit *f, const vo_f2 *slots, int n);
void vo_fit_set_generators(vo_fit *f, const vo_f2 *slots, int slotsW, int slotsH, float slotCellSize);
void vo_fit_update_generators(vo_fit *f, const vo_f2 *slots, int cx0, int cy0, int cx1, int cy1);
void vo_fit_begin_schedule(vo_fit *f, int iterations, int cx0, int cy0, int cx1, int cy1);
/* Runs `steps` iterations; returns the last batch loss (loss / count). */
float vo_fit_step(vo_fit *f, int steps);
float vo_fit_eval_loss(vo_fit *f);
int vo_fit_iteration(const vo_fit *f);
int vo_fit_schedule_length(const vo_fit *f);
int vo_fit_grid_size(const vo_fit *f, int *gw, int *gh);
/* Copies out the generators (n float2) and, when non-NULL, m and v. */
void vo_fit_get(const vo_fit *f, vo_f2 *gen, vo_f2 *m, vo_f2 *v);
/* Builds the grid for the current generators and copies it out. */
void vo_fit_grid(vo_fit *f, int *start, int *sortedIdx, vo_f2 *sortedPos, int *genCell);
/* The gradient the next Step would apply: REF float sums / FIXED converted. */
void vo_fit_gradient(vo_fit *f, float *grad, int *count, float *loss);

/* ---- FP64 oracle ---------------------------------------------------------------
 * The same optimiser with every loss, gradient and Adam operation in double
 * (kNN by double distances, ties by index). Used for error bars only. */
typedef struct vo_fit64 vo_fit64;
vo_fit64 *vo_fit64_create(double width, double height, double spacing, int K, double lrPerSpacing,
                          double sampleFraction, double gamma, const int milestones[4], int paramIterations,
                          unsigned seed, int nthreads);
void vo_fit64_destroy(vo_fit64 *f);
void vo_fit64_set_targets(vo_fit64 *f, const vo_f2 *slots, int n);
void vo_fit64_set_generators(vo_fit64 *f, const vo_f2 *slots, int slotsW, int slotsH, double slotCellSize);
double vo_fit64_step(vo_fit64 *f, int steps);
double vo_fit64_eval_loss(vo_fit64 *f);
void vo_fit64_get(const vo_fit64 *f, double *gen);
void vo_fit64_gradient(vo_fit64 *f, double *grad, int *count, double *loss);
void vo_fit64_detail(vo_fit64 *f, int *i0, int *j);

/* ---- extraction ------------------------------------------------------------------
 * voronoiCellKernel (voro_optimizer.cu:361-437): FP64 Sutherland-Hodgman
 * clipping by the 32 nearest bisectors with the security-radius certificate
 * and the brute-force fallback, then occupancy of the centroid. */
enum { VO_MAX_CELL_VERTS = 24, VO_CELL_K = 32 };
void vo_extract_cells(const vo_grid *g, const vo_f2 *gen, int n, float width, float height, const uint64_t *masks,
                      int tilesX, int tilesY, float invVoxel, vo_f2 *outVerts, int *outEdges, int *outCount,
                      uint8_t *outInside, int *flags, int nthreads);
/* Boundary assembly (voro_optimizer.cu:798-854). Outputs are malloc'ed
 * buffers the caller frees with vo_free; returns the vertex count. */
int vo_assemble(const vo_f2 *verts, const int *labels, const int *counts, const uint8_t *inside, int n,
                int *cellStart /* n+1 */, vo_f2 **meshVerts, int **edges, int *numEdges, int *watertight,
                int *loops);
void vo_free(void *p);

/* ---- Poisson -------------------------------------------------------------------
 * Sampler (poisson_disk.cu:119-177): the grid is float2[gridW*gridH]. */
typedef struct {
    float width, height, radius, cellSize;
    int gridW, gridH, trials;
    unsigned seed, roundBase;
} vo_poisson;
void vo_poisson_init(vo_poisson *p, float width, float height, float radius, int trials, unsigned seed);
void vo_poisson_resample(vo_poisson *p, vo_f2 *grid, int cx0, int cy0, int cx1, int cy1);
/* The same with the rows of each phase split over nthreads threads (the same
 * result: cells of a phase are independent). */
void vo_poisson_resample_mt(vo_poisson *p, vo_f2 *grid, int cx0, int cy0, int cx1, int cy1, int nthreads);
int vo_poisson_verify(const vo_poisson *p, const vo_f2 *grid, int cx0, int cy0, int cx1, int cy1);

/* ---- RNG (voro_optimizer.cu:69-78, poisson_disk.cu:47-58) ------------------ */
unsigned vo_pcg_hash(unsigned v);
float vo_rand01(unsigned index, unsigned iter, unsigned seed);
float vo_poisson_rand01(unsigned cell, unsigned round, unsigned seed, unsigned stream);

#ifdef __cplusplus
}
#endif

#endif
