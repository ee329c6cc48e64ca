/*
 * vm_oracle.c — CPU restatement of the reference VoroMesh optimiser, Voronoi
 * clipper, boundary assembly and Poisson sampler.
 *
 * TEST INFRASTRUCTURE: the checker for the CUDA path and the CPU baseline of
 * bench.py. Nothing in the product loads it. Build: oracle/Makefile
 * (gcc -O2 -ffp-contract=off; no -ffast-math, so every float operation is a
 * single IEEE-rounded operation in the order written, as in the reference).
 *
 * Citations are file:line in the reference project.
 */
#include "vm_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------------------
 * small parallel-for over [0, n)
 * ------------------------------------------------------------------------- */
typedef void (*vo_range_fn)(void *ctx, int64_t lo, int64_t hi, int tid);
typedef struct {
    vo_range_fn fn;
    void *ctx;
    int64_t lo, hi;
    int tid;
} vo_job;

static void *vo_job_run(void *arg)
{
    vo_job *j = (vo_job *)arg;
    j->fn(j->ctx, j->lo, j->hi, j->tid);
    return NULL;
}

static void vo_parallel(int nthreads, int64_t n, vo_range_fn fn, void *ctx)
{
    if (nthreads <= 1 || n < 2 * (int64_t)nthreads) {
        fn(ctx, 0, n, 0);
        return;
    }
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    vo_job jobs[256];
    int64_t chunk = (n + nthreads - 1) / nthreads;
    int started = 0;
    for (int t = 0; t < nthreads; ++t) {
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].lo = t * chunk;
        jobs[t].hi = (t + 1) * chunk < n ? (t + 1) * chunk : n;
        jobs[t].tid = t;
        if (jobs[t].lo >= jobs[t].hi) break;
        if (pthread_create(&th[t], NULL, vo_job_run, &jobs[t]) != 0) {
            fn(ctx, jobs[t].lo, jobs[t].hi, t);
            th[t] = 0;
        }
        started = t + 1;
    }
    for (int t = 0; t < started; ++t)
        if (th[t]) pthread_join(th[t], NULL);
}

/* ---------------------------------------------------------------------------
 * RNG: voro_optimizer.cu:69-78, poisson_disk.cu:47-58
 * ------------------------------------------------------------------------- */
unsigned vo_pcg_hash(unsigned v)
{
    unsigned state = v * 747796405u + 2891336453u;
    unsigned word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

float vo_rand01(unsigned index, unsigned iter, unsigned seed)
{
    unsigned h = vo_pcg_hash(index ^ vo_pcg_hash(iter * 2654435761u ^ vo_pcg_hash(seed)));
    return (float)(h & 0x00FFFFFFu) * (1.0f / 16777216.0f);
}

float vo_poisson_rand01(unsigned cell, unsigned round, unsigned seed, unsigned stream)
{
    unsigned h = vo_pcg_hash(cell ^ vo_pcg_hash(round * 2654435761u ^ vo_pcg_hash(seed + stream * 0x9E3779B9u)));
    return (float)(h & 0x00FFFFFFu) * (1.0f / 16777216.0f);
}

/* ---------------------------------------------------------------------------
 * Hash grid: cellCoord voro_optimizer.cu:123-125, binKernel :168-177,
 * scan :697, scatterKernel :179-187.
 * int(v * inv) is the GPU's saturating truncation (NaN -> 0), then clamped.
 * ------------------------------------------------------------------------- */
int vo_cell_coord(float v, float inv, int n)
{
    float f = v * inv;
    int c;
    if (f != f) c = 0;
    else if (f >= 2147483648.0f) c = 2147483647;
    else if (f <= -2147483648.0f) c = -2147483647 - 1;
    else c = (int)f;
    if (c < 0) c = 0;
    if (c > n - 1) c = n - 1;
    return c;
}

void vo_build_grid(const vo_f2 *gen, int n, int gw, int gh, float cellSize, int *genCell, int *start,
                   int *sortedIdx, vo_f2 *sortedPos)
{
    int cells = gw * gh;
    float inv = 1.0f / cellSize;
    memset(start, 0, sizeof(int) * (size_t)(cells + 1));
    for (int i = 0; i < n; ++i) {
        if (gen[i].x < 0.0f) {
            genCell[i] = -1;
            continue;
        }
        int c = vo_cell_coord(gen[i].y, inv, gh) * gw + vo_cell_coord(gen[i].x, inv, gw);
        genCell[i] = c;
        start[c + 1] += 1;
    }
    for (int c = 0; c < cells; ++c) start[c + 1] += start[c];
    int *fill = (int *)calloc((size_t)cells + 1, sizeof(int));
    for (int i = 0; i < n; ++i) {
        int c = genCell[i];
        if (c < 0) continue;
        int s = start[c] + fill[c]++;
        sortedIdx[s] = i;
        sortedPos[s] = gen[i];
    }
    free(fill);
}

/* ---------------------------------------------------------------------------
 * kNN: voro_optimizer.cu:130-163. Insertion keeps (d2, index) ascending, so
 * exact distance ties are ordered by site index (the reference orders them by
 * visit order, which its atomic binning makes run-dependent within a cell).
 * ------------------------------------------------------------------------- */
static int key_less(float dd, int id, float D, int I)
{
    return dd < D || (dd == D && (unsigned)id < (unsigned)I);
}

void vo_knn(const vo_grid *g, vo_f2 q, int K, int *idx, float *d2)
{
    for (int k = 0; k < K; ++k) {
        idx[k] = -1;
        d2[k] = FLT_MAX;
    }
    float inv = 1.0f / g->cellSize;
    int cx = vo_cell_coord(q.x, inv, g->w), cy = vo_cell_coord(q.y, inv, g->h);
    for (int ring = 0;; ++ring) {
        int x0 = cx - ring, x1 = cx + ring, y0 = cy - ring, y1 = cy + ring;
        int ya = y0 > 0 ? y0 : 0, yb = y1 < g->h - 1 ? y1 : g->h - 1;
        for (int y = ya; y <= yb; ++y) {
            int stride = (y == y0 || y == y1) ? 1 : (x1 - x0 > 1 ? x1 - x0 : 1);
            for (int x = x0; x <= x1; x += stride) {
                if (x < 0 || x >= g->w) continue;
                int c = y * g->w + x;
                for (int s = g->start[c]; s < g->start[c + 1]; ++s) {
                    vo_f2 p = g->pos[s];
                    float dx = p.x - q.x, dy = p.y - q.y;
                    float dd = dx * dx + dy * dy;
                    int id = g->idx[s];
                    if (!key_less(dd, id, d2[K - 1], idx[K - 1])) continue;
                    int k = K - 1;
                    while (k > 0 && key_less(dd, id, d2[k - 1], idx[k - 1])) {
                        d2[k] = d2[k - 1];
                        idx[k] = idx[k - 1];
                        --k;
                    }
                    d2[k] = dd;
                    idx[k] = id;
                }
            }
        }
        if (x0 <= 0 && y0 <= 0 && x1 >= g->w - 1 && y1 >= g->h - 1) break;
        float cs = g->cellSize;
        float safe = fminf(fminf(q.x - (float)x0 * cs, (float)(x1 + 1) * cs - q.x),
                           fminf(q.y - (float)y0 * cs, (float)(y1 + 1) * cs - q.y));
        safe = fmaxf(safe, 0.0f);
        if (d2[K - 1] <= safe * safe) break;
    }
}

typedef struct {
    const vo_grid *g;
    const vo_f2 *q;
    int K;
    int *idx;
    float *d2;
} knn_job;

static void knn_range(void *ctx, int64_t lo, int64_t hi, int tid)
{
    (void)tid;
    knn_job *J = (knn_job *)ctx;
    for (int64_t i = lo; i < hi; ++i) vo_knn(J->g, J->q[i], J->K, J->idx + i * J->K, J->d2 + i * J->K);
}

void vo_knn_many(const vo_grid *g, const vo_f2 *q, int n, int K, int *idx, float *d2, int nthreads)
{
    knn_job J = {g, q, K, idx, d2};
    vo_parallel(nthreads, n, knn_range, &J);
}

void vo_knn_brute(const vo_f2 *gen, int n, vo_f2 q, int K, int *idx, float *d2)
{
    for (int k = 0; k < K; ++k) {
        idx[k] = -1;
        d2[k] = FLT_MAX;
    }
    for (int i = 0; i < n; ++i) {
        if (gen[i].x < 0.0f) continue;
        float dx = gen[i].x - q.x, dy = gen[i].y - q.y;
        float dd = dx * dx + dy * dy;
        if (!key_less(dd, i, d2[K - 1], idx[K - 1])) continue;
        int k = K - 1;
        while (k > 0 && key_less(dd, i, d2[k - 1], idx[k - 1])) {
            d2[k] = d2[k - 1];
            idx[k] = idx[k - 1];
            --k;
        }
        d2[k] = dd;
        idx[k] = i;
    }
}

/* ---------------------------------------------------------------------------
 * Fixed-point accumulation (the product's order-independent sums).
 *   eh = floor(log2(spacing))
 *   gradient component: int64 of round-half-even(v * 2^(40-eh)), |.| <= 2^62
 *   loss term (>= 0):   128-bit floor(v * 2^(64-2 eh)) from the float's bits
 * ------------------------------------------------------------------------- */
static int floor_log2f(float h)
{
    int e = 0;
    frexpf(h, &e);
    return e - 1;
}

int vo_fixed_grad_exp(float spacing) { return 40 - floor_log2f(spacing); }
int vo_fixed_loss_exp(float spacing) { return 64 - 2 * floor_log2f(spacing); }

int64_t vo_fixed_from_float(float v, int e)
{
    if (v != v) return 0;
    float s = v * ldexpf(1.0f, e);
    const float lim = 4611686018427387904.0f; /* 2^62 */
    if (s >= lim) return (int64_t)4611686018427387904LL;
    if (s <= -lim) return -(int64_t)4611686018427387904LL;
    return (int64_t)llrintf(s);
}

float vo_fixed_to_float(int64_t v, int e) { return (float)v * ldexpf(1.0f, -e); }

/* Exact per-site gradient sums: each int64 term v is added to two words,
 * L += v mod 2^32 (unsigned) and H += v >> 32 (arithmetic), so the site's sum
 * S = H * 2^32 + L is exact for fewer than 2^31 terms, where one 64-bit sum
 * would wrap past 2^63. S is formed in 128 bits and rounded to float once
 * (the C conversion from __int128 rounds to nearest even), then scaled. */
void vo_fixed2_add(int64_t v, int64_t *H, uint64_t *L)
{
    __atomic_fetch_add(L, (uint64_t)v & 0xFFFFFFFFull, __ATOMIC_RELAXED);
    __atomic_fetch_add(H, v >> 32, __ATOMIC_RELAXED);
}

float vo_fixed2_to_float(int64_t H, uint64_t L, int e)
{
    __int128 S = (__int128)H * ((__int128)1 << 32) + (__int128)L;
    return (float)S * ldexpf(1.0f, -e);
}

void vo_fixed_loss_add(float v, int e, uint64_t *lo, uint64_t *hi)
{
    if (!(v > 0.0f)) return;
    uint32_t bits;
    memcpy(&bits, &v, 4);
    int ex = (int)((bits >> 23) & 0xFFu);
    uint64_t m = bits & 0x7FFFFFu;
    uint64_t alo = 0, ahi = 0;
    if (ex == 0xFF) {
        ahi = 1ULL << 62;
    } else {
        int k;
        if (ex == 0) k = -149 + e;
        else {
            m |= 0x800000u;
            k = ex - 150 + e;
        }
        if (k >= 104) ahi = 1ULL << 62;
        else if (k >= 64) ahi = m << (k - 64);
        else if (k > 0) {
            alo = m << k;
            ahi = m >> (64 - k);
        } else if (k == 0) alo = m;
        else if (k > -64) alo = m >> (-k);
    }
    uint64_t old = *lo;
    *lo = old + alo;
    *hi = *hi + ahi + (*lo < old ? 1u : 0u);
}

float vo_fixed_loss_to_float(uint64_t lo, uint64_t hi, int e)
{
    double d = (double)hi * 18446744073709551616.0 + (double)lo;
    d = d * ldexp(1.0, -e);
    return (float)d;
}

/* ---------------------------------------------------------------------------
 * VoroLoss for one target: voro_optimizer.cu:210-256.
 * Returns 1 when the target contributes; fills the nearest site, the chosen
 * neighbour, the loss and the four gradient terms in the reference's order
 * (grad[bestJ].x, .y, grad[i0].x, .y).
 * ------------------------------------------------------------------------- */
typedef struct {
    int i0, j;
    float loss;
    float g[4];
} vo_target_out;

static int loss_target(const vo_f2 *targets, int i, const vo_grid *g, const vo_f2 *gen, int K,
                       const vo_run_params *rp, float fraction, unsigned seed, unsigned iter, int wantGrad,
                       vo_target_out *o)
{
    vo_f2 p = targets[i];
    int take = p.x >= 0.0f;
    if (take && rp) take = p.x >= rp->bx0 && p.x <= rp->bx1 && p.y >= rp->by0 && p.y <= rp->by1;
    if (take && fraction < 1.0f) take = vo_rand01((unsigned)i, iter, seed) < fraction;
    if (!take) return 0;
    int idx[64];
    float d2[64];
    vo_knn(g, p, K, idx, d2);
    if (idx[0] < 0) return 0;
    int i0 = idx[0];
    vo_f2 c0 = gen[i0];
    float ux = p.x - c0.x, uy = p.y - c0.y;
    float best = FLT_MAX, bestD = 0.0f;
    int bestJ = -1;
    for (int k = 1; k < K; ++k) {
        int j = idx[k];
        if (j < 0) break;
        float ex = gen[j].x - c0.x, ey = gen[j].y - c0.y;
        float l = sqrtf(ex * ex + ey * ey);
        if (l < 1e-12f) continue;
        float d = (ux * ex + uy * ey) / l - 0.5f * l;
        if (d * d < best) {
            best = d * d;
            bestD = d;
            bestJ = j;
        }
    }
    if (bestJ < 0) return 0;
    o->i0 = i0;
    o->j = bestJ;
    o->loss = best;
    if (wantGrad) {
        float ex = gen[bestJ].x - c0.x, ey = gen[bestJ].y - c0.y;
        float l = sqrtf(ex * ex + ey * ey);
        float il = 1.0f / l;
        float nx = il * ex, ny = il * ey;
        float un = ux * nx + uy * ny;
        float tx = ux - un * nx, ty = uy - un * ny;
        float il2 = 1.0f / l;
        float dcx = il2 * tx - 0.5f * nx, dcy = il2 * ty - 0.5f * ny;
        float s = 2.0f * bestD;
        o->g[0] = s * dcx;
        o->g[1] = s * dcy;
        o->g[2] = -s * (nx + dcx);
        o->g[3] = -s * (ny + dcy);
    }
    return 1;
}

typedef struct {
    const vo_f2 *targets;
    const vo_grid *g;
    const vo_f2 *gen;
    int K;
    const vo_run_params *rp;
    float fraction;
    unsigned seed, iter;
    int ge, le;
    int64_t *gradFixed;
    uint64_t lo[256], hi[256];
    int count[256];
} vo_loss_job;

static void loss_fixed_range(void *ctx, int64_t lo, int64_t hi, int tid)
{
    vo_loss_job *J = (vo_loss_job *)ctx;
    uint64_t llo = 0, lhi = 0;
    int cnt = 0;
    for (int64_t i = lo; i < hi; ++i) {
        vo_target_out o;
        if (!loss_target(J->targets, (int)i, J->g, J->gen, J->K, J->rp, J->fraction, J->seed, J->iter,
                         J->gradFixed != NULL, &o))
            continue;
        ++cnt;
        vo_fixed_loss_add(o.loss, J->le, &llo, &lhi);
        if (J->gradFixed) {
            /* words per site: L.x, L.y, H.x, H.y */
            int64_t *gj = J->gradFixed + 4 * (size_t)o.j, *g0 = J->gradFixed + 4 * (size_t)o.i0;
            vo_fixed2_add(vo_fixed_from_float(o.g[0], J->ge), &gj[2], (uint64_t *)&gj[0]);
            vo_fixed2_add(vo_fixed_from_float(o.g[1], J->ge), &gj[3], (uint64_t *)&gj[1]);
            vo_fixed2_add(vo_fixed_from_float(o.g[2], J->ge), &g0[2], (uint64_t *)&g0[0]);
            vo_fixed2_add(vo_fixed_from_float(o.g[3], J->ge), &g0[3], (uint64_t *)&g0[1]);
        }
    }
    J->lo[tid] = llo;
    J->hi[tid] = lhi;
    J->count[tid] = cnt;
}

void vo_loss(const vo_f2 *targets, int numTargets, const vo_grid *g, const vo_f2 *gen, int n, int K,
             const vo_run_params *rp, float fraction, unsigned seed, unsigned iter, int accMode, float spacing,
             float *grad, int64_t *gradFixed, vo_loss_sum *out, int nthreads)
{
    (void)n;
    memset(out, 0, sizeof(*out));
    if (accMode == VO_ACC_REF) {
        float loss = 0.0f;
        int count = 0;
        for (int i = 0; i < numTargets; ++i) {
            vo_target_out o;
            if (!loss_target(targets, i, g, gen, K, rp, fraction, seed, iter, grad != NULL, &o)) continue;
            if (grad) {
                grad[2 * o.j] += o.g[0];
                grad[2 * o.j + 1] += o.g[1];
                grad[2 * o.i0] += o.g[2];
                grad[2 * o.i0 + 1] += o.g[3];
            }
            loss += o.loss;
            count += 1;
        }
        out->loss = loss;
        out->count = count;
        return;
    }
    vo_loss_job *J = (vo_loss_job *)calloc(1, sizeof(vo_loss_job));
    J->targets = targets;
    J->g = g;
    J->gen = gen;
    J->K = K;
    J->rp = rp;
    J->fraction = fraction;
    J->seed = seed;
    J->iter = iter;
    J->ge = vo_fixed_grad_exp(spacing);
    J->le = vo_fixed_loss_exp(spacing);
    J->gradFixed = gradFixed;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    vo_parallel(nthreads, numTargets, loss_fixed_range, J);
    uint64_t lo = 0, hi = 0;
    int count = 0;
    for (int t = 0; t < 256; ++t) {
        uint64_t old = lo;
        lo += J->lo[t];
        hi += J->hi[t] + (lo < old ? 1u : 0u);
        count += J->count[t];
    }
    out->lossLo = lo;
    out->lossHi = hi;
    out->count = count;
    out->loss = vo_fixed_loss_to_float(lo, hi, J->le);
    free(J);
}

void vo_loss_detail(const vo_f2 *targets, int numTargets, const vo_grid *g, const vo_f2 *gen, int K,
                    const vo_run_params *rp, float fraction, unsigned seed, unsigned iter, int *i0, int *bestJ,
                    float *loss)
{
    for (int i = 0; i < numTargets; ++i) {
        vo_target_out o;
        if (loss_target(targets, i, g, gen, K, rp, fraction, seed, iter, 0, &o)) {
            i0[i] = o.i0;
            bestJ[i] = o.j;
            loss[i] = o.loss;
        } else {
            i0[i] = -1;
            bestJ[i] = -1;
            loss[i] = 0.0f;
        }
    }
}

/* ---------------------------------------------------------------------------
 * Adam + MultiStepLR + clamp: voro_optimizer.cu:271-301
 * ------------------------------------------------------------------------- */
float vo_pow_det(float base, int t)
{
    double r = 1.0, x = (double)base;
    unsigned e = t < 0 ? 0u : (unsigned)t;
    while (e) {
        if (e & 1u) r = r * x;
        x = x * x;
        e >>= 1;
    }
    return (float)r;
}

typedef struct {
    vo_f2 *gen, *m, *v;
    float *gradFloat;
    int64_t *gradFixed;
    int gradExp, iter, count, powMode;
    const vo_run_params *rp;
} vo_adam_job;

static void adam_range(void *ctx, int64_t lo, int64_t hi, int tid)
{
    (void)tid;
    vo_adam_job *J = (vo_adam_job *)ctx;
    const vo_run_params *rp = J->rp;
    for (int64_t ii = lo; ii < hi; ++ii) {
        int i = (int)ii;
        float grx, gry;
        if (J->gradFixed) {
            int64_t *w = J->gradFixed + 4 * (size_t)i;
            grx = vo_fixed2_to_float(w[2], (uint64_t)w[0], J->gradExp);
            gry = vo_fixed2_to_float(w[3], (uint64_t)w[1], J->gradExp);
            w[0] = w[1] = w[2] = w[3] = 0;
        } else {
            grx = J->gradFloat[2 * i];
            gry = J->gradFloat[2 * i + 1];
            J->gradFloat[2 * i] = 0.0f;
            J->gradFloat[2 * i + 1] = 0.0f;
        }
        vo_f2 p = J->gen[i];
        int sx = i % rp->slotsW, sy = i / rp->slotsW;
        if (p.x < 0.0f || sx < rp->cx0 || sx >= rp->cx1 || sy < rp->cy0 || sy >= rp->cy1) continue;
        int t = J->iter;
        float lr = rp->lr;
        for (int k = 0; k < 4; ++k)
            if (t - 1 >= rp->milestones[k]) lr *= rp->gamma;
        float bc1, bc2;
        if (J->powMode == VO_POW_REF) {
            bc1 = 1.0f - powf(rp->beta1, (float)t);
            bc2 = 1.0f - powf(rp->beta2, (float)t);
        } else {
            bc1 = 1.0f - vo_pow_det(rp->beta1, t);
            bc2 = 1.0f - vo_pow_det(rp->beta2, t);
        }
        float sc = 1.0f / (float)(J->count > 1 ? J->count : 1);
        grx = sc * grx;
        gry = sc * gry;
        float mx = rp->beta1 * J->m[i].x + (1.0f - rp->beta1) * grx;
        float my = rp->beta1 * J->m[i].y + (1.0f - rp->beta1) * gry;
        float vx = rp->beta2 * J->v[i].x + (1.0f - rp->beta2) * (grx * grx);
        float vy = rp->beta2 * J->v[i].y + (1.0f - rp->beta2) * (gry * gry);
        J->m[i].x = mx;
        J->m[i].y = my;
        J->v[i].x = vx;
        J->v[i].y = vy;
        p.x -= lr * (mx / bc1) / (sqrtf(vx / bc2) + rp->eps);
        p.y -= lr * (my / bc1) / (sqrtf(vy / bc2) + rp->eps);
        p.x = fminf(fmaxf(p.x, 0.0f), rp->width);
        p.y = fminf(fmaxf(p.y, 0.0f), rp->height);
        J->gen[i] = p;
    }
}

void vo_adam(vo_f2 *gen, vo_f2 *m, vo_f2 *v, float *gradFloat, int64_t *gradFixed, int gradExp, int n, int iter,
             int count, const vo_run_params *rp, int powMode, int nthreads)
{
    vo_adam_job J = {gen, m, v, gradFloat, gradFixed, gradExp, iter, count, powMode, rp};
    vo_parallel(nthreads, n, adam_range, &J);
}

/* ---------------------------------------------------------------------------
 * VoroOptimizer restated: voro_optimizer.cu:512-761
 * ------------------------------------------------------------------------- */
struct vo_fit {
    float width, height, spacing;
    int K;
    float lrPerSpacing, sampleFraction, gamma;
    int milestones[4];
    int paramIterations;
    unsigned seed;
    int accMode, powMode, nthreads;
    int gw, gh;
    int slotsW, slotsH;
    float slotCellSize;
    vo_f2 *gen, *m, *v;
    float *gradF;
    int64_t *gradX;
    int *genCell, *start, *sortedIdx;
    vo_f2 *sortedPos;
    vo_f2 *targets;
    int targetCapacity;
    vo_run_params rp;
    int iter, count;
    float loss;
    int scheduleLength, iteration;
    float lastBatchLoss;
};

vo_fit *vo_fit_create(float width, float height, float spacing, int K, float lrPerSpacing, float sampleFraction,
                      float gamma, const int milestones[4], int paramIterations, unsigned seed, int accMode,
                      int powMode, int nthreads)
{
    vo_fit *f = (vo_fit *)calloc(1, sizeof(vo_fit));
    f->width = width;
    f->height = height;
    f->spacing = spacing;
    f->K = K;
    f->lrPerSpacing = lrPerSpacing;
    f->sampleFraction = sampleFraction;
    f->gamma = gamma;
    memcpy(f->milestones, milestones, sizeof(int) * 4);
    f->paramIterations = paramIterations;
    f->seed = seed;
    f->accMode = accMode;
    f->powMode = powMode;
    f->nthreads = nthreads < 1 ? 1 : nthreads;
    /* voro_optimizer.cu:520-521 */
    int gw = (int)ceilf(width / spacing), gh = (int)ceilf(height / spacing);
    f->gw = gw > 1 ? gw : 1;
    f->gh = gh > 1 ? gh : 1;
    f->start = (int *)calloc((size_t)f->gw * f->gh + 1, sizeof(int));
    return f;
}

void vo_fit_destroy(vo_fit *f)
{
    if (!f) return;
    free(f->gen); free(f->m); free(f->v); free(f->gradF); free(f->gradX);
    free(f->genCell); free(f->start); free(f->sortedIdx); free(f->sortedPos); free(f->targets);
    free(f);
}

/* SetTargets: voro_optimizer.cu:549-560 (NaN padding, capacity >= 1) */
void vo_fit_set_targets(vo_fit *f, const vo_f2 *slots, int n)
{
    int cap = n > 1 ? n : 1;
    free(f->targets);
    f->targets = (vo_f2 *)malloc(sizeof(vo_f2) * (size_t)cap);
    memset(f->targets, 0xFF, sizeof(vo_f2) * (size_t)cap);
    if (n > 0) memcpy(f->targets, slots, sizeof(vo_f2) * (size_t)n);
    f->targetCapacity = cap;
}

/* SetGenerators: voro_optimizer.cu:613-638 */
void vo_fit_set_generators(vo_fit *f, const vo_f2 *slots, int slotsW, int slotsH, float slotCellSize)
{
    int n = slotsW * slotsH;
    if (slotsW != f->slotsW || slotsH != f->slotsH) {
        f->slotsW = slotsW;
        f->slotsH = slotsH;
        free(f->gen); free(f->m); free(f->v); free(f->gradF); free(f->gradX);
        free(f->genCell); free(f->sortedIdx); free(f->sortedPos);
        size_t nn = (size_t)(n > 0 ? n : 1);
        f->gen = (vo_f2 *)malloc(sizeof(vo_f2) * nn);
        f->m = (vo_f2 *)calloc(nn, sizeof(vo_f2));
        f->v = (vo_f2 *)calloc(nn, sizeof(vo_f2));
        f->gradF = (float *)calloc(2 * nn, sizeof(float));
        f->gradX = (int64_t *)calloc(4 * nn, sizeof(int64_t));
        f->genCell = (int *)malloc(sizeof(int) * nn);
        f->sortedIdx = (int *)malloc(sizeof(int) * nn);
        f->sortedPos = (vo_f2 *)malloc(sizeof(vo_f2) * nn);
    }
    f->slotCellSize = slotCellSize;
    if (n > 0) memcpy(f->gen, slots, sizeof(vo_f2) * (size_t)n);
    memset(f->gradF, 0, sizeof(float) * 2 * (size_t)(n > 0 ? n : 1));
    memset(f->gradX, 0, sizeof(int64_t) * 4 * (size_t)(n > 0 ? n : 1));
    vo_fit_begin_schedule(f, f->paramIterations, 0, 0, f->slotsW, f->slotsH);
}

/* UpdateGenerators: voro_optimizer.cu:640-650 (the slots of the clamped
 * rectangle are copied from the full slot array; nothing else changes) */
void vo_fit_update_generators(vo_fit *f, const vo_f2 *slots, int cx0, int cy0, int cx1, int cy1)
{
    cx0 = cx0 > 0 ? cx0 : 0;
    cy0 = cy0 > 0 ? cy0 : 0;
    cx1 = cx1 < f->slotsW ? cx1 : f->slotsW;
    cy1 = cy1 < f->slotsH ? cy1 : f->slotsH;
    if (cx0 >= cx1 || cy0 >= cy1) return;
    for (int y = cy0; y < cy1; ++y)
        memcpy(f->gen + (size_t)y * f->slotsW + cx0, slots + (size_t)y * f->slotsW + cx0,
               sizeof(vo_f2) * (size_t)(cx1 - cx0));
}

/* BeginSchedule: voro_optimizer.cu:652-687 */
void vo_fit_begin_schedule(vo_fit *f, int iterations, int cx0, int cy0, int cx1, int cy1)
{
    cx0 = cx0 > 0 ? cx0 : 0;
    cy0 = cy0 > 0 ? cy0 : 0;
    cx1 = cx1 < f->slotsW ? cx1 : f->slotsW;
    cy1 = cy1 < f->slotsH ? cy1 : f->slotsH;
    vo_run_params *rp = &f->rp;
    rp->lr = f->lrPerSpacing * f->spacing;
    rp->gamma = f->gamma;
    rp->beta1 = 0.9f;
    rp->beta2 = 0.999f;
    rp->eps = 1e-8f;
    for (int k = 0; k < 4; ++k)
        rp->milestones[k] = (int)lround((double)f->milestones[k] * iterations / f->paramIterations);
    rp->width = f->width;
    rp->height = f->height;
    rp->slotsW = f->slotsW;
    rp->cx0 = cx0; rp->cy0 = cy0; rp->cx1 = cx1; rp->cy1 = cy1;
    float margin = 2.0f * f->spacing;
    rp->bx0 = (float)cx0 * f->slotCellSize - margin;
    rp->by0 = (float)cy0 * f->slotCellSize - margin;
    rp->bx1 = (float)cx1 * f->slotCellSize + margin;
    rp->by1 = (float)cy1 * f->slotCellSize + margin;
    for (int y = cy0; y < cy1; ++y)
        for (int x = cx0; x < cx1; ++x) {
            size_t i = (size_t)y * f->slotsW + x;
            f->m[i].x = f->m[i].y = 0.0f;
            f->v[i].x = f->v[i].y = 0.0f;
        }
    f->iter = 0;
    f->count = 0;
    f->loss = 0.0f;
    f->scheduleLength = iterations;
    f->iteration = 0;
    f->lastBatchLoss = 0.0f;
}

static void fit_grid(vo_fit *f, vo_grid *g)
{
    int n = f->slotsW * f->slotsH;
    vo_build_grid(f->gen, n, f->gw, f->gh, f->spacing, f->genCell, f->start, f->sortedIdx, f->sortedPos);
    g->w = f->gw;
    g->h = f->gh;
    g->cellSize = f->spacing;
    g->start = f->start;
    g->idx = f->sortedIdx;
    g->pos = f->sortedPos;
}

/* Step: voro_optimizer.cu:724-744 with EnqueueIteration :702-711 */
float vo_fit_step(vo_fit *f, int steps)
{
    int n = f->slotsW * f->slotsH;
    if (steps <= 0 || n == 0 || f->targetCapacity == 0) return 0.0f;
    for (int s = 0; s < steps; ++s) {
        f->iter += 1; /* beginIterationKernel :192-197 */
        f->count = 0;
        f->loss = 0.0f;
        vo_grid g;
        fit_grid(f, &g);
        vo_loss_sum ls;
        vo_loss(f->targets, f->targetCapacity, &g, f->gen, n, f->K, &f->rp, f->sampleFraction, f->seed,
                (unsigned)f->iter, f->accMode, f->spacing, f->accMode == VO_ACC_REF ? f->gradF : NULL,
                f->accMode == VO_ACC_FIXED ? f->gradX : NULL, &ls, f->nthreads);
        f->count = ls.count;
        f->loss = ls.loss;
        vo_adam(f->gen, f->m, f->v, f->accMode == VO_ACC_REF ? f->gradF : NULL,
                f->accMode == VO_ACC_FIXED ? f->gradX : NULL, vo_fixed_grad_exp(f->spacing), n, f->iter,
                f->count, &f->rp, f->powMode, f->nthreads);
    }
    f->iteration = f->iter;
    f->lastBatchLoss = f->count > 0 ? f->loss / (float)f->count : 0.0f;
    return f->lastBatchLoss;
}

/* EvaluateLoss: voro_optimizer.cu:746-761 */
float vo_fit_eval_loss(vo_fit *f)
{
    int n = f->slotsW * f->slotsH;
    if (n == 0 || f->targetCapacity == 0) return 0.0f;
    vo_grid g;
    fit_grid(f, &g);
    vo_loss_sum ls;
    vo_loss(f->targets, f->targetCapacity, &g, f->gen, n, f->K, NULL, 1.0f, f->seed, (unsigned)f->iter,
            f->accMode, f->spacing, NULL, NULL, &ls, f->nthreads);
    f->count = ls.count;
    f->loss = ls.loss;
    return ls.count > 0 ? ls.loss / (float)ls.count : 0.0f;
}

int vo_fit_iteration(const vo_fit *f) { return f->iteration; }
int vo_fit_schedule_length(const vo_fit *f) { return f->scheduleLength; }

int vo_fit_grid_size(const vo_fit *f, int *gw, int *gh)
{
    *gw = f->gw;
    *gh = f->gh;
    return f->gw * f->gh;
}

void vo_fit_get(const vo_fit *f, vo_f2 *gen, vo_f2 *m, vo_f2 *v)
{
    size_t n = (size_t)f->slotsW * f->slotsH;
    if (gen) memcpy(gen, f->gen, sizeof(vo_f2) * n);
    if (m) memcpy(m, f->m, sizeof(vo_f2) * n);
    if (v) memcpy(v, f->v, sizeof(vo_f2) * n);
}

void vo_fit_grid(vo_fit *f, int *start, int *sortedIdx, vo_f2 *sortedPos, int *genCell)
{
    vo_grid g;
    fit_grid(f, &g);
    int n = f->slotsW * f->slotsH;
    int live = f->start[f->gw * f->gh];
    if (start) memcpy(start, f->start, sizeof(int) * ((size_t)f->gw * f->gh + 1));
    if (sortedIdx) memcpy(sortedIdx, f->sortedIdx, sizeof(int) * (size_t)live);
    if (sortedPos) memcpy(sortedPos, f->sortedPos, sizeof(vo_f2) * (size_t)live);
    if (genCell) memcpy(genCell, f->genCell, sizeof(int) * (size_t)n);
}

void vo_fit_gradient(vo_fit *f, float *grad, int *count, float *loss)
{
    int n = f->slotsW * f->slotsH;
    vo_grid g;
    fit_grid(f, &g);
    vo_loss_sum ls;
    unsigned it = (unsigned)f->iter + 1u;
    if (f->accMode == VO_ACC_REF) {
        float *gf = (float *)calloc(2 * (size_t)n, sizeof(float));
        vo_loss(f->targets, f->targetCapacity, &g, f->gen, n, f->K, &f->rp, f->sampleFraction, f->seed, it,
                VO_ACC_REF, f->spacing, gf, NULL, &ls, 1);
        memcpy(grad, gf, sizeof(float) * 2 * (size_t)n);
        free(gf);
    } else {
        int64_t *gx = (int64_t *)calloc(4 * (size_t)(n > 0 ? n : 1), sizeof(int64_t));
        vo_loss(f->targets, f->targetCapacity, &g, f->gen, n, f->K, &f->rp, f->sampleFraction, f->seed, it,
                VO_ACC_FIXED, f->spacing, NULL, gx, &ls, f->nthreads);
        int e = vo_fixed_grad_exp(f->spacing);
        for (int i = 0; i < n; ++i) {
            const int64_t *w = gx + 4 * (size_t)i;
            grad[2 * i] = vo_fixed2_to_float(w[2], (uint64_t)w[0], e);
            grad[2 * i + 1] = vo_fixed2_to_float(w[3], (uint64_t)w[1], e);
        }
        free(gx);
    }
    *count = ls.count;
    *loss = ls.loss;
}

/* ---------------------------------------------------------------------------
 * FP64 optimiser (error bars): the same algorithm in double.
 * ------------------------------------------------------------------------- */
struct vo_fit64 {
    double width, height, spacing;
    int K;
    double lrPerSpacing, sampleFraction, gamma;
    int milestones[4];
    int paramIterations;
    unsigned seed;
    int nthreads;
    int gw, gh;
    int slotsW, slotsH;
    double slotCellSize;
    double *gen, *m, *v, *grad;
    int *start, *sortedIdx, *cell;
    double *targets;
    int targetCapacity;
    double lr, bx0, by0, bx1, by1;
    int ms[4], cx0, cy0, cx1, cy1;
    int iter, count;
    double loss;
};

vo_fit64 *vo_fit64_create(double width, double height, double spacing, int K, double lrPerSpacing,
                          double sampleFraction, double gamma, const int milestones[4], int paramIterations,
                          unsigned seed, int nthreads)
{
    vo_fit64 *f = (vo_fit64 *)calloc(1, sizeof(vo_fit64));
    f->width = width;
    f->height = height;
    f->spacing = spacing;
    f->K = K;
    f->lrPerSpacing = lrPerSpacing;
    f->sampleFraction = sampleFraction;
    f->gamma = gamma;
    memcpy(f->milestones, milestones, sizeof(int) * 4);
    f->paramIterations = paramIterations;
    f->seed = seed;
    f->nthreads = nthreads < 1 ? 1 : nthreads;
    int gw = (int)ceil(width / spacing), gh = (int)ceil(height / spacing);
    f->gw = gw > 1 ? gw : 1;
    f->gh = gh > 1 ? gh : 1;
    f->start = (int *)calloc((size_t)f->gw * f->gh + 1, sizeof(int));
    return f;
}

void vo_fit64_destroy(vo_fit64 *f)
{
    if (!f) return;
    free(f->gen); free(f->m); free(f->v); free(f->grad); free(f->start); free(f->sortedIdx);
    free(f->cell); free(f->targets);
    free(f);
}

void vo_fit64_set_targets(vo_fit64 *f, const vo_f2 *slots, int n)
{
    int cap = n > 1 ? n : 1;
    free(f->targets);
    f->targets = (double *)malloc(sizeof(double) * 2 * (size_t)cap);
    for (int i = 0; i < cap; ++i) {
        f->targets[2 * i] = i < n ? (double)slots[i].x : NAN;
        f->targets[2 * i + 1] = i < n ? (double)slots[i].y : NAN;
    }
    f->targetCapacity = cap;
}

void vo_fit64_set_generators(vo_fit64 *f, const vo_f2 *slots, int slotsW, int slotsH, double slotCellSize)
{
    int n = slotsW * slotsH;
    size_t nn = (size_t)(n > 0 ? n : 1);
    free(f->gen); free(f->m); free(f->v); free(f->grad); free(f->sortedIdx); free(f->cell);
    f->slotsW = slotsW;
    f->slotsH = slotsH;
    f->slotCellSize = slotCellSize;
    f->gen = (double *)malloc(sizeof(double) * 2 * nn);
    f->m = (double *)calloc(2 * nn, sizeof(double));
    f->v = (double *)calloc(2 * nn, sizeof(double));
    f->grad = (double *)calloc(2 * nn, sizeof(double));
    f->sortedIdx = (int *)malloc(sizeof(int) * nn);
    f->cell = (int *)malloc(sizeof(int) * nn);
    for (int i = 0; i < n; ++i) {
        f->gen[2 * i] = slots[i].x;
        f->gen[2 * i + 1] = slots[i].y;
    }
    int iterations = f->paramIterations;
    f->lr = f->lrPerSpacing * f->spacing;
    for (int k = 0; k < 4; ++k) f->ms[k] = (int)lround((double)f->milestones[k] * iterations / f->paramIterations);
    f->cx0 = 0; f->cy0 = 0; f->cx1 = slotsW; f->cy1 = slotsH;
    double margin = 2.0 * f->spacing;
    f->bx0 = -margin;
    f->by0 = -margin;
    f->bx1 = slotsW * slotCellSize + margin;
    f->by1 = slotsH * slotCellSize + margin;
    f->iter = 0;
}

static int cell64(double v, double inv, int n)
{
    double f = v * inv;
    int c = f != f ? 0 : (f > 2e9 ? 2000000000 : (f < -2e9 ? -2000000000 : (int)f));
    return c < 0 ? 0 : (c > n - 1 ? n - 1 : c);
}

static void grid64(vo_fit64 *f)
{
    int n = f->slotsW * f->slotsH, cells = f->gw * f->gh;
    double inv = 1.0 / f->spacing;
    memset(f->start, 0, sizeof(int) * (size_t)(cells + 1));
    for (int i = 0; i < n; ++i) {
        if (f->gen[2 * i] < 0.0) { f->cell[i] = -1; continue; }
        int c = cell64(f->gen[2 * i + 1], inv, f->gh) * f->gw + cell64(f->gen[2 * i], inv, f->gw);
        f->cell[i] = c;
        f->start[c + 1]++;
    }
    for (int c = 0; c < cells; ++c) f->start[c + 1] += f->start[c];
    int *fill = (int *)calloc((size_t)cells + 1, sizeof(int));
    for (int i = 0; i < n; ++i)
        if (f->cell[i] >= 0) f->sortedIdx[f->start[f->cell[i]] + fill[f->cell[i]]++] = i;
    free(fill);
}

static int key_less64(double dd, int id, double D, int I)
{
    return dd < D || (dd == D && (unsigned)id < (unsigned)I);
}

static void knn64(const vo_fit64 *f, double qx, double qy, int K, int *idx, double *d2)
{
    for (int k = 0; k < K; ++k) { idx[k] = -1; d2[k] = DBL_MAX; }
    double cs = f->spacing, inv = 1.0 / cs;
    int cx = cell64(qx, inv, f->gw), cy = cell64(qy, inv, f->gh);
    for (int ring = 0;; ++ring) {
        int x0 = cx - ring, x1 = cx + ring, y0 = cy - ring, y1 = cy + ring;
        for (int y = y0 > 0 ? y0 : 0; y <= (y1 < f->gh - 1 ? y1 : f->gh - 1); ++y) {
            int stride = (y == y0 || y == y1) ? 1 : (x1 - x0 > 1 ? x1 - x0 : 1);
            for (int x = x0; x <= x1; x += stride) {
                if (x < 0 || x >= f->gw) continue;
                int c = y * f->gw + x;
                for (int s = f->start[c]; s < f->start[c + 1]; ++s) {
                    int id = f->sortedIdx[s];
                    double dx = f->gen[2 * id] - qx, dy = f->gen[2 * id + 1] - qy;
                    double dd = dx * dx + dy * dy;
                    if (!key_less64(dd, id, d2[K - 1], idx[K - 1])) continue;
                    int k = K - 1;
                    while (k > 0 && key_less64(dd, id, d2[k - 1], idx[k - 1])) {
                        d2[k] = d2[k - 1]; idx[k] = idx[k - 1]; --k;
                    }
                    d2[k] = dd; idx[k] = id;
                }
            }
        }
        if (x0 <= 0 && y0 <= 0 && x1 >= f->gw - 1 && y1 >= f->gh - 1) break;
        double safe = fmin(fmin(qx - x0 * cs, (x1 + 1) * cs - qx), fmin(qy - y0 * cs, (y1 + 1) * cs - qy));
        safe = fmax(safe, 0.0);
        if (d2[K - 1] <= safe * safe) break;
    }
}

typedef struct {
    vo_fit64 *f;
    int useBox, wantGrad;
    double fraction;
    unsigned iter;
    double loss[256];
    int count[256];
    pthread_mutex_t *mu;
    int *i0Out, *jOut; /* optional per-target decisions (-1 = unused) */
} vo_l64_job;

static void loss64_range(void *ctx, int64_t lo, int64_t hi, int tid)
{
    vo_l64_job *J = (vo_l64_job *)ctx;
    vo_fit64 *f = J->f;
    double loss = 0.0;
    int cnt = 0;
    int idx[64];
    double d2[64];
    for (int64_t ii = lo; ii < hi; ++ii) {
        int i = (int)ii;
        if (J->i0Out) J->i0Out[i] = J->jOut[i] = -1;
        double px = f->targets[2 * i], py = f->targets[2 * i + 1];
        int take = px >= 0.0;
        if (take && J->useBox) take = px >= f->bx0 && px <= f->bx1 && py >= f->by0 && py <= f->by1;
        if (take && J->fraction < 1.0) take = vo_rand01((unsigned)i, J->iter, f->seed) < (float)J->fraction;
        if (!take) continue;
        knn64(f, px, py, f->K, idx, d2);
        if (idx[0] < 0) continue;
        int i0 = idx[0];
        double c0x = f->gen[2 * i0], c0y = f->gen[2 * i0 + 1];
        double ux = px - c0x, uy = py - c0y, best = DBL_MAX, bestD = 0.0;
        int bestJ = -1;
        for (int k = 1; k < f->K; ++k) {
            int j = idx[k];
            if (j < 0) break;
            double ex = f->gen[2 * j] - c0x, ey = f->gen[2 * j + 1] - c0y;
            double l = sqrt(ex * ex + ey * ey);
            if (l < 1e-12) continue;
            double d = (ux * ex + uy * ey) / l - 0.5 * l;
            if (d * d < best) { best = d * d; bestD = d; bestJ = j; }
        }
        if (bestJ < 0) continue;
        if (J->i0Out) {
            J->i0Out[i] = i0;
            J->jOut[i] = bestJ;
        }
        loss += best;
        ++cnt;
        if (J->wantGrad) {
            double ex = f->gen[2 * bestJ] - c0x, ey = f->gen[2 * bestJ + 1] - c0y;
            double l = sqrt(ex * ex + ey * ey);
            double nx = ex / l, ny = ey / l, un = ux * nx + uy * ny;
            double dcx = (ux - un * nx) / l - 0.5 * nx, dcy = (uy - un * ny) / l - 0.5 * ny;
            double s = 2.0 * bestD;
            pthread_mutex_lock(J->mu);
            f->grad[2 * bestJ] += s * dcx;
            f->grad[2 * bestJ + 1] += s * dcy;
            f->grad[2 * i0] += -s * (nx + dcx);
            f->grad[2 * i0 + 1] += -s * (ny + dcy);
            pthread_mutex_unlock(J->mu);
        }
    }
    J->loss[tid] = loss;
    J->count[tid] = cnt;
}

static void loss64_detail(vo_fit64 *f, int useBox, double fraction, unsigned iter, int wantGrad, double *loss,
                          int *count, int *i0Out, int *jOut)
{
    vo_l64_job *J = (vo_l64_job *)calloc(1, sizeof(vo_l64_job));
    J->i0Out = i0Out;
    J->jOut = jOut;
    pthread_mutex_t mu = PTHREAD_MUTEX_INITIALIZER;
    J->f = f;
    J->useBox = useBox;
    J->wantGrad = wantGrad;
    J->fraction = fraction;
    J->iter = iter;
    J->mu = &mu;
    vo_parallel(f->nthreads, f->targetCapacity, loss64_range, J);
    double l = 0.0;
    int c = 0;
    for (int t = 0; t < 256; ++t) { l += J->loss[t]; c += J->count[t]; }
    *loss = l;
    *count = c;
    free(J);
}

static void loss64(vo_fit64 *f, int useBox, double fraction, unsigned iter, int wantGrad, double *loss, int *count)
{
    loss64_detail(f, useBox, fraction, iter, wantGrad, loss, count, NULL, NULL);
}

double vo_fit64_step(vo_fit64 *f, int steps)
{
    int n = f->slotsW * f->slotsH;
    double last = 0.0;
    for (int s = 0; s < steps; ++s) {
        f->iter += 1;
        grid64(f);
        double loss;
        int count;
        loss64(f, 1, f->sampleFraction, (unsigned)f->iter, 1, &loss, &count);
        f->count = count;
        f->loss = loss;
        int t = f->iter;
        double lr = f->lr;
        for (int k = 0; k < 4; ++k)
            if (t - 1 >= f->ms[k]) lr *= f->gamma;
        double b1 = 0.9, b2 = 0.999, eps = 1e-8;
        double bc1 = 1.0 - pow(b1, t), bc2 = 1.0 - pow(b2, t);
        double sc = 1.0 / (count > 1 ? count : 1);
        for (int i = 0; i < n; ++i) {
            double gx = sc * f->grad[2 * i], gy = sc * f->grad[2 * i + 1];
            f->grad[2 * i] = f->grad[2 * i + 1] = 0.0;
            if (f->gen[2 * i] < 0.0) continue;
            int sx = i % f->slotsW, sy = i / f->slotsW;
            if (sx < f->cx0 || sx >= f->cx1 || sy < f->cy0 || sy >= f->cy1) continue;
            double *m = &f->m[2 * i], *v = &f->v[2 * i], *p = &f->gen[2 * i];
            m[0] = b1 * m[0] + (1.0 - b1) * gx;
            m[1] = b1 * m[1] + (1.0 - b1) * gy;
            v[0] = b2 * v[0] + (1.0 - b2) * gx * gx;
            v[1] = b2 * v[1] + (1.0 - b2) * gy * gy;
            p[0] -= lr * (m[0] / bc1) / (sqrt(v[0] / bc2) + eps);
            p[1] -= lr * (m[1] / bc1) / (sqrt(v[1] / bc2) + eps);
            p[0] = fmin(fmax(p[0], 0.0), f->width);
            p[1] = fmin(fmax(p[1], 0.0), f->height);
        }
        last = count > 0 ? loss / count : 0.0;
    }
    return last;
}

double vo_fit64_eval_loss(vo_fit64 *f)
{
    grid64(f);
    double loss;
    int count;
    loss64(f, 0, 1.0, (unsigned)f->iter, 0, &loss, &count);
    return count > 0 ? loss / count : 0.0;
}

void vo_fit64_get(const vo_fit64 *f, double *gen)
{
    memcpy(gen, f->gen, sizeof(double) * 2 * (size_t)f->slotsW * f->slotsH);
}

/* Per target: nearest site and bisector neighbour of the full-target pass
 * (EvaluateLoss's decisions) at the current generators, in double. */
void vo_fit64_detail(vo_fit64 *f, int *i0, int *j)
{
    double loss;
    int count;
    grid64(f);
    loss64_detail(f, 0, 1.0, (unsigned)f->iter, 0, &loss, &count, i0, j);
}

void vo_fit64_gradient(vo_fit64 *f, double *grad, int *count, double *loss)
{
    int n = f->slotsW * f->slotsH;
    grid64(f);
    memset(f->grad, 0, sizeof(double) * 2 * (size_t)n);
    loss64(f, 1, f->sampleFraction, (unsigned)f->iter + 1u, 1, loss, count);
    memcpy(grad, f->grad, sizeof(double) * 2 * (size_t)n);
    memset(f->grad, 0, sizeof(double) * 2 * (size_t)n);
}

/* ---------------------------------------------------------------------------
 * Extraction: CellPoly / clipByBisector / maxRadius2 / voronoiCellKernel,
 * voro_optimizer.cu:312-437; occupied() :104-112.
 * ------------------------------------------------------------------------- */
typedef struct {
    double vx[VO_MAX_CELL_VERTS], vy[VO_MAX_CELL_VERTS];
    int e[VO_MAX_CELL_VERTS];
    int n;
} vo_poly;

static int clip_bisector(vo_poly *poly, double rx, double ry, int label)
{
    double c = 0.5 * (rx * rx + ry * ry);
    int anyOut = 0;
    for (int k = 0; k < poly->n; ++k) anyOut |= poly->vx[k] * rx + poly->vy[k] * ry - c > 0.0;
    if (!anyOut) return 1;
    vo_poly out;
    out.n = 0;
    int ok = 1;
    for (int k = 0; k < poly->n; ++k) {
        int k1 = (k + 1) % poly->n;
        double ax = poly->vx[k], ay = poly->vy[k], bx = poly->vx[k1], by = poly->vy[k1];
        double fa = ax * rx + ay * ry - c;
        double fb = bx * rx + by * ry - c;
        int inA = fa <= 0.0, inB = fb <= 0.0;
        if (inA) {
            if (out.n < VO_MAX_CELL_VERTS) {
                out.vx[out.n] = ax; out.vy[out.n] = ay; out.e[out.n] = poly->e[k]; ++out.n;
            } else ok = 0;
        }
        if (inA != inB) {
            double t = fa / (fa - fb);
            double xx = ax + t * (bx - ax), xy = ay + t * (by - ay);
            if (out.n < VO_MAX_CELL_VERTS) {
                out.vx[out.n] = xx; out.vy[out.n] = xy; out.e[out.n] = inA ? label : poly->e[k]; ++out.n;
            } else ok = 0;
        }
    }
    *poly = out;
    return ok;
}

static double max_radius2(const vo_poly *p)
{
    double r2 = 0.0;
    for (int k = 0; k < p->n; ++k) r2 = fmax(r2, p->vx[k] * p->vx[k] + p->vy[k] * p->vy[k]);
    return r2;
}

static int occupied(const uint64_t *masks, int tilesX, int tilesY, float invVoxel, vo_f2 p)
{
    if (!masks) return 0;
    float fx = floorf(p.x * invVoxel), fy = floorf(p.y * invVoxel);
    if (!(fx >= 0.0f) || !(fy >= 0.0f) || fx >= 2147483647.0f || fy >= 2147483647.0f) return 0;
    int i = (int)fx, j = (int)fy;
    int tx = i >> 3, ty = j >> 3;
    if (tx >= tilesX || ty >= tilesY) return 0;
    return (int)((masks[(size_t)ty * tilesX + tx] >> (((j & 7) << 3) | (i & 7))) & 1ull);
}

typedef struct {
    const vo_grid *g;
    const vo_f2 *gen;
    int n;
    float width, height;
    const uint64_t *masks;
    int tilesX, tilesY;
    float invVoxel;
    vo_f2 *outVerts;
    int *outEdges, *outCount;
    uint8_t *outInside;
    int unsafe[256], overflow[256];
} vo_cells_job;

static void cells_range(void *ctx, int64_t lo, int64_t hi, int tid)
{
    vo_cells_job *J = (vo_cells_job *)ctx;
    const vo_f2 *gen = J->gen;
    int idx[VO_CELL_K];
    float d2[VO_CELL_K];
    int unsafe = 0, overflow = 0;
    for (int64_t ii = lo; ii < hi; ++ii) {
        int i = (int)ii;
        vo_f2 ci = gen[i];
        if (ci.x < 0.0f) {
            J->outCount[i] = 0;
            J->outInside[i] = 0;
            continue;
        }
        vo_knn(J->g, ci, VO_CELL_K, idx, d2);
        vo_poly poly;
        double x0 = -(double)ci.x, y0 = -(double)ci.y;
        double x1 = (double)J->width - (double)ci.x, y1 = (double)J->height - (double)ci.y;
        poly.vx[0] = x0; poly.vy[0] = y0; poly.e[0] = -1;
        poly.vx[1] = x1; poly.vy[1] = y0; poly.e[1] = -2;
        poly.vx[2] = x1; poly.vy[2] = y1; poly.e[2] = -3;
        poly.vx[3] = x0; poly.vy[3] = y1; poly.e[3] = -4;
        poly.n = 4;
        int ok = 1, certified = 0;
        double r2max = max_radius2(&poly);
        for (int k = 0; k < VO_CELL_K; ++k) {
            int j = idx[k];
            if (j < 0) { certified = 1; break; }
            if (j == i) continue;
            if ((double)d2[k] > 4.0 * r2max) { certified = 1; break; }
            vo_f2 cj = gen[j];
            ok &= clip_bisector(&poly, (double)cj.x - ci.x, (double)cj.y - ci.y, j);
            r2max = max_radius2(&poly);
        }
        if (!certified && (double)d2[VO_CELL_K - 1] > 4.0 * r2max) certified = 1;
        if (!certified) {
            ++unsafe;
            for (int j = 0; j < J->n; ++j) {
                if (j == i || gen[j].x < 0.0f) continue;
                int seen = 0;
                for (int k = 0; k < VO_CELL_K; ++k) seen |= idx[k] == j;
                if (seen) continue;
                double rx = (double)gen[j].x - ci.x, ry = (double)gen[j].y - ci.y;
                if (rx * rx + ry * ry > 4.0 * r2max) continue;
                ok &= clip_bisector(&poly, rx, ry, j);
                r2max = max_radius2(&poly);
            }
        }
        if (!ok) ++overflow;
        double area = 0.0, cx = 0.0, cy = 0.0;
        for (int k = 0; k < poly.n; ++k) {
            int k1 = (k + 1) % poly.n;
            double ax = poly.vx[k], ay = poly.vy[k], bx = poly.vx[k1], by = poly.vy[k1];
            double cr = ax * by - bx * ay;
            area += cr;
            cx += (ax + bx) * cr;
            cy += (ay + by) * cr;
        }
        vo_f2 centroid = ci;
        if (fabs(area) > 1e-12) {
            centroid.x += (float)(cx / (3.0 * area));
            centroid.y += (float)(cy / (3.0 * area));
        }
        J->outInside[i] = occupied(J->masks, J->tilesX, J->tilesY, J->invVoxel, centroid) ? 1 : 0;
        J->outCount[i] = poly.n;
        for (int k = 0; k < poly.n; ++k) {
            J->outVerts[(size_t)i * VO_MAX_CELL_VERTS + k].x = (float)(ci.x + poly.vx[k]);
            J->outVerts[(size_t)i * VO_MAX_CELL_VERTS + k].y = (float)(ci.y + poly.vy[k]);
            J->outEdges[(size_t)i * VO_MAX_CELL_VERTS + k] = poly.e[k];
        }
    }
    J->unsafe[tid] = unsafe;
    J->overflow[tid] = overflow;
}

void vo_extract_cells(const vo_grid *g, const vo_f2 *gen, int n, float width, float height, const uint64_t *masks,
                      int tilesX, int tilesY, float invVoxel, vo_f2 *outVerts, int *outEdges, int *outCount,
                      uint8_t *outInside, int *flags, int nthreads)
{
    vo_cells_job *J = (vo_cells_job *)calloc(1, sizeof(vo_cells_job));
    J->g = g; J->gen = gen; J->n = n; J->width = width; J->height = height;
    J->masks = masks; J->tilesX = tilesX; J->tilesY = tilesY; J->invVoxel = invVoxel;
    J->outVerts = outVerts; J->outEdges = outEdges; J->outCount = outCount; J->outInside = outInside;
    vo_parallel(nthreads, n, cells_range, J);
    flags[0] = flags[1] = 0;
    for (int t = 0; t < 256; ++t) { flags[0] += J->unsafe[t]; flags[1] += J->overflow[t]; }
    free(J);
}

/* ---------------------------------------------------------------------------
 * Boundary assembly: voro_optimizer.cu:798-854. The vertex map keeps first-
 * insertion order (the reference's unordered_map::try_emplace numbering).
 * ------------------------------------------------------------------------- */
typedef struct {
    uint64_t *keys;
    int *vals;
    size_t cap;
} vo_map;

static uint64_t mix64(uint64_t x)
{
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

static int map_get_or_add(vo_map *m, uint64_t key, int val, int *inserted)
{
    size_t mask = m->cap - 1, h = mix64(key) & mask;
    for (;;) {
        if (m->vals[h] < 0) {
            m->keys[h] = key;
            m->vals[h] = val;
            *inserted = 1;
            return val;
        }
        if (m->keys[h] == key) {
            *inserted = 0;
            return m->vals[h];
        }
        h = (h + 1) & mask;
    }
}

static uint64_t tri_key(int a, int b, int c)
{
    uint64_t v0 = (uint64_t)(a + 4), v1 = (uint64_t)(b + 4), v2 = (uint64_t)(c + 4), t;
    if (v0 > v1) { t = v0; v0 = v1; v1 = t; }
    if (v1 > v2) { t = v1; v1 = v2; v2 = t; }
    if (v0 > v1) { t = v0; v0 = v1; v1 = t; }
    return (v0 << 42) | (v1 << 21) | v2;
}

int vo_assemble(const vo_f2 *verts, const int *labels, const int *counts, const uint8_t *inside, int n,
                int *cellStart, vo_f2 **meshVerts, int **edgesOut, int *numEdges, int *watertight, int *loops)
{
    cellStart[0] = 0;
    for (int i = 0; i < n; ++i) cellStart[i + 1] = cellStart[i] + counts[i];
    size_t maxEdges = 0;
    for (int i = 0; i < n; ++i)
        if (inside[i]) maxEdges += (size_t)counts[i];
    vo_map map;
    map.cap = 64;
    while (map.cap < 4 * (maxEdges + 16)) map.cap <<= 1;
    map.keys = (uint64_t *)malloc(sizeof(uint64_t) * map.cap);
    map.vals = (int *)malloc(sizeof(int) * map.cap);
    for (size_t h = 0; h < map.cap; ++h) map.vals[h] = -1;
    vo_f2 *mv = (vo_f2 *)malloc(sizeof(vo_f2) * (2 * maxEdges + 1));
    int *ed = (int *)malloc(sizeof(int) * 2 * (maxEdges + 1));
    int nv = 0, ne = 0;
    for (int i = 0; i < n; ++i) {
        if (!inside[i]) continue;
        int c = counts[i];
        const int *lab = labels + (size_t)i * VO_MAX_CELL_VERTS;
        const vo_f2 *pos = verts + (size_t)i * VO_MAX_CELL_VERTS;
        for (int k = 0; k < c; ++k) {
            int l = lab[k];
            if (l >= 0 && inside[l]) continue;
            int prev = lab[(k + c - 1) % c], next = lab[(k + 1) % c];
            int ins;
            int a = map_get_or_add(&map, tri_key(i, prev, l), nv, &ins);
            if (ins) mv[nv++] = pos[k];
            int b = map_get_or_add(&map, tri_key(i, l, next), nv, &ins);
            if (ins) mv[nv++] = pos[(k + 1) % c];
            ed[2 * ne] = a;
            ed[2 * ne + 1] = b;
            ++ne;
        }
    }
    int *nxt = (int *)malloc(sizeof(int) * (size_t)(nv + 1));
    int *indeg = (int *)calloc((size_t)nv + 1, sizeof(int));
    for (int v = 0; v < nv; ++v) nxt[v] = -1;
    int wt = 1;
    for (int e = 0; e < ne; ++e) {
        int a = ed[2 * e], b = ed[2 * e + 1];
        if (nxt[a] != -1) wt = 0;
        nxt[a] = b;
        ++indeg[b];
    }
    for (int v = 0; v < nv; ++v)
        if (nxt[v] == -1 || indeg[v] != 1) wt = 0;
    int lp = 0;
    if (wt) {
        unsigned char *seen = (unsigned char *)calloc((size_t)nv + 1, 1);
        for (int v = 0; v < nv; ++v) {
            if (seen[v]) continue;
            ++lp;
            for (int w = v; !seen[w]; w = nxt[w]) seen[w] = 1;
        }
        free(seen);
    }
    free(nxt);
    free(indeg);
    free(map.keys);
    free(map.vals);
    *meshVerts = mv;
    *edgesOut = ed;
    *numEdges = ne;
    *watertight = wt;
    *loops = lp;
    return nv;
}

void vo_free(void *p) { free(p); }

/* ---------------------------------------------------------------------------
 * Poisson disk sampler: poisson_disk.cu:74-177
 * ------------------------------------------------------------------------- */
void vo_poisson_init(vo_poisson *p, float width, float height, float radius, int trials, unsigned seed)
{
    p->width = width;
    p->height = height;
    p->radius = radius;
    p->cellSize = radius / sqrtf(2.0f);
    p->gridW = (int)ceilf(width / p->cellSize);
    p->gridH = (int)ceilf(height / p->cellSize);
    p->trials = trials;
    p->seed = seed;
    p->roundBase = 0;
}

/* One phase of one round over rows [lo, hi) of the phase's rows: a dart per
 * empty phase cell, rejected if any sample of the 5x5 neighbourhood is nearer
 * than the radius (dartPhaseKernel, poisson_disk.cu:74-107). Cells of a phase
 * are 3 apart and read only cells of other phases, so rows of a phase can run
 * in parallel with the same result as in order. */
typedef struct {
    const vo_poisson *p;
    vo_f2 *grid;
    int x0, x1, y0, px, py;
    unsigned rnd;
} vo_phase_job;

static void poisson_phase_rows(void *ctx, int64_t lo, int64_t hi, int tid)
{
    (void)tid;
    const vo_phase_job *J = (const vo_phase_job *)ctx;
    const vo_poisson *p = J->p;
    vo_f2 *grid = J->grid;
    float r2 = p->radius * p->radius;
    for (int64_t row = lo; row < hi; ++row) {
        int cy = J->y0 + J->py + 3 * (int)row;
        for (int cx = J->x0 + J->px; cx < J->x1; cx += 3) {
            int cellId = cy * p->gridW + cx;
            if (grid[cellId].x >= 0.0f) continue;
            float x = ((float)cx + vo_poisson_rand01((unsigned)cellId, J->rnd, p->seed, 0)) * p->cellSize;
            float y = ((float)cy + vo_poisson_rand01((unsigned)cellId, J->rnd, p->seed, 1)) * p->cellSize;
            if (x >= p->width || y >= p->height) continue;
            int nx0 = cx - 2 > 0 ? cx - 2 : 0, nx1 = cx + 2 < p->gridW - 1 ? cx + 2 : p->gridW - 1;
            int ny0 = cy - 2 > 0 ? cy - 2 : 0, ny1 = cy + 2 < p->gridH - 1 ? cy + 2 : p->gridH - 1;
            int reject = 0;
            for (int ny = ny0; ny <= ny1 && !reject; ++ny)
                for (int nx = nx0; nx <= nx1; ++nx) {
                    vo_f2 q = grid[(size_t)ny * p->gridW + nx];
                    if (q.x < 0.0f) continue;
                    float dx = q.x - x, dy = q.y - y;
                    if (dx * dx + dy * dy < r2) { reject = 1; break; }
                }
            if (reject) continue;
            grid[cellId].x = x;
            grid[cellId].y = y;
        }
    }
}

/* Sampler::Resample (poisson_disk.cu:141-177): clear the region, then
 * trials rounds of 9 phases (3x3 colour classes). */
void vo_poisson_resample_mt(vo_poisson *p, vo_f2 *grid, int cx0, int cy0, int cx1, int cy1, int nthreads)
{
    int x0 = cx0 > 0 ? cx0 : 0, y0 = cy0 > 0 ? cy0 : 0;
    int x1 = cx1 < p->gridW ? cx1 : p->gridW, y1 = cy1 < p->gridH ? cy1 : p->gridH;
    if (x0 >= x1 || y0 >= y1) return;
    for (int y = y0; y < y1; ++y)
        for (int x = x0; x < x1; ++x) {
            grid[(size_t)y * p->gridW + x].x = -1.0f;
            grid[(size_t)y * p->gridW + x].y = -1.0f;
        }
    for (int round = 0; round < p->trials; ++round)
        for (int py = 0; py < 3; ++py)
            for (int px = 0; px < 3; ++px) {
                vo_phase_job J = {p, grid, x0, x1, y0, px, py, p->roundBase + (unsigned)round};
                int rows = y0 + py < y1 ? (y1 - 1 - (y0 + py)) / 3 + 1 : 0;
                int nt = nthreads;
                if ((int64_t)rows * ((x1 - x0 + 2) / 3) < 65536) nt = 1; /* small phases: no threads */
                vo_parallel(nt, rows, poisson_phase_rows, &J);
            }
    p->roundBase += (unsigned)p->trials;
}

void vo_poisson_resample(vo_poisson *p, vo_f2 *grid, int cx0, int cy0, int cx1, int cy1)
{
    vo_poisson_resample_mt(p, grid, cx0, cy0, cx1, cy1, 1);
}

/* Sampler::Verify: poisson_disk.cu:179-199 */
int vo_poisson_verify(const vo_poisson *p, const vo_f2 *grid, int cx0, int cy0, int cx1, int cy1)
{
    float r2 = p->radius * p->radius;
    int vx0 = cx0 - 2 > 0 ? cx0 - 2 : 0, vx1 = cx1 + 2 < p->gridW ? cx1 + 2 : p->gridW;
    int vy0 = cy0 - 2 > 0 ? cy0 - 2 : 0, vy1 = cy1 + 2 < p->gridH ? cy1 + 2 : p->gridH;
    for (int cy = vy0; cy < vy1; ++cy)
        for (int cx = vx0; cx < vx1; ++cx) {
            vo_f2 a = grid[(size_t)cy * p->gridW + cx];
            if (a.x < 0) continue;
            for (int ny = cy - 2 > 0 ? cy - 2 : 0; ny <= (cy + 2 < p->gridH - 1 ? cy + 2 : p->gridH - 1); ++ny)
                for (int nx = cx - 2 > 0 ? cx - 2 : 0; nx <= (cx + 2 < p->gridW - 1 ? cx + 2 : p->gridW - 1); ++nx) {
                    if (nx == cx && ny == cy) continue;
                    vo_f2 b = grid[(size_t)ny * p->gridW + nx];
                    if (b.x < 0) continue;
                    float dx = a.x - b.x, dy = a.y - b.y;
                    if (dx * dx + dy * dy < r2) return 0;
                }
        }
    return 1;
}
