/*
 * vo_canvas — CPU restatement of the reference's Canvas (test infrastructure;
 * see vo_canvas.h). Citations are to src/voromesh/canvas.cpp.
 */
#include "vo_canvas.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define TILE_LOG2 3
#define TILE 8

struct vo_canvas {
    float vs;
    int vx, vy, tx, ty;
    uint64_t *inside; /* tiles */
    uint64_t *smask;  /* tiles */
    vo_f2 *spt;       /* tiles * 64 */
    int *sslot;       /* tiles * 64 */
    vo_f2 *slots;
    int nslots, capSlots;
    int *freel;
    int nfree, capFree;
    long long surfaceCount;
    int surfaceTiles;
    int *dirty;
    int ndirty, capDirty;
};

typedef struct {
    long long key; /* tile-major voxel index: (ty*tilesX + tx)*64 + bit */
    int idx;       /* sample order */
    float x, y;
} sample_t;

static int bit_of(int i, int j) { return ((j & (TILE - 1)) << TILE_LOG2) | (i & (TILE - 1)); }

static long long vkey(const vo_canvas *c, int i, int j)
{
    return ((long long)(j >> TILE_LOG2) * c->tx + (i >> TILE_LOG2)) * 64 + bit_of(i, j);
}

static int in_domain(const vo_canvas *c, int i, int j) { return i >= 0 && j >= 0 && i < c->vx && j < c->vy; }

static int is_inside(const vo_canvas *c, int i, int j)
{
    return in_domain(c, i, j) &&
           (int)((c->inside[(size_t)(j >> TILE_LOG2) * c->tx + (i >> TILE_LOG2)] >> bit_of(i, j)) & 1u);
}

static int cmp_sample(const void *pa, const void *pb)
{
    const sample_t *a = (const sample_t *)pa, *b = (const sample_t *)pb;
    if (a->key != b->key) return a->key < b->key ? -1 : 1;
    return (a->idx > b->idx) - (a->idx < b->idx);
}

static int cmp_float(const void *pa, const void *pb)
{
    float a = *(const float *)pa, b = *(const float *)pb;
    return (a > b) - (a < b);
}

static int grow(void **p, int *cap, int need, size_t elem)
{
    if (need <= *cap) return 0;
    int nc = *cap > 0 ? *cap : 64;
    while (nc < need) nc *= 2;
    void *q = realloc(*p, (size_t)nc * elem);
    if (!q) return -1;
    *p = q;
    *cap = nc;
    return 0;
}

static int push_dirty(vo_canvas *c, int s)
{
    if (grow((void **)&c->dirty, &c->capDirty, c->ndirty + 1, sizeof(int))) return -1;
    c->dirty[c->ndirty++] = s;
    return 0;
}

/* Canvas::AllocSlot (canvas.cpp:51-63) */
static int alloc_slot(vo_canvas *c, vo_f2 p)
{
    int s;
    if (c->nfree > 0) {
        s = c->freel[--c->nfree];
    } else {
        if (grow((void **)&c->slots, &c->capSlots, c->nslots + 1, sizeof(vo_f2))) return -1;
        s = c->nslots++;
    }
    c->slots[s] = p;
    return s;
}

/* Canvas::FreeSlot (canvas.cpp:65-69) */
static int free_slot(vo_canvas *c, int s)
{
    c->slots[s].x = -1.0f;
    c->slots[s].y = -1.0f;
    if (grow((void **)&c->freel, &c->capFree, c->nfree + 1, sizeof(int))) return -1;
    c->freel[c->nfree++] = s;
    return 0;
}

/* Mean of one voxel's run of sorted samples, summed in sample order in double
 * (canvas.cpp:13-25). */
static vo_f2 run_mean(const sample_t *s, int n)
{
    double sx = 0.0, sy = 0.0;
    for (int k = 0; k < n; ++k) {
        sx += s[k].x;
        sy += s[k].y;
    }
    vo_f2 m = {(float)(sx / n), (float)(sy / n)};
    return m;
}

vo_canvas *vo_canvas_create(float width, float height, float voxelSize)
{
    vo_canvas *c = (vo_canvas *)calloc(1, sizeof(vo_canvas));
    if (!c) return NULL;
    /* canvas.cpp:33-38 */
    c->vs = voxelSize;
    c->vx = (int)ceilf(width / voxelSize);
    c->vy = (int)ceilf(height / voxelSize);
    c->tx = (c->vx + TILE - 1) / TILE;
    c->ty = (c->vy + TILE - 1) / TILE;
    size_t tiles = (size_t)c->tx * c->ty;
    c->inside = (uint64_t *)calloc(tiles ? tiles : 1, sizeof(uint64_t));
    c->smask = (uint64_t *)calloc(tiles ? tiles : 1, sizeof(uint64_t));
    c->spt = (vo_f2 *)malloc((tiles ? tiles : 1) * 64 * sizeof(vo_f2));
    c->sslot = (int *)malloc((tiles ? tiles : 1) * 64 * sizeof(int));
    if (!c->inside || !c->smask || !c->spt || !c->sslot) {
        vo_canvas_destroy(c);
        return NULL;
    }
    return c;
}

void vo_canvas_destroy(vo_canvas *c)
{
    if (!c) return;
    free(c->inside);
    free(c->smask);
    free(c->spt);
    free(c->sslot);
    free(c->slots);
    free(c->freel);
    free(c->dirty);
    free(c);
}

/* Canvas::RasterizeShape (canvas.cpp:71-134) */
int vo_canvas_rasterize(vo_canvas *c, const vo_f2 *poly, int n)
{
    size_t tiles = (size_t)c->tx * c->ty;
    memset(c->smask, 0, tiles * sizeof(uint64_t));
    memset(c->inside, 0, tiles * sizeof(uint64_t));
    c->nslots = c->nfree = 0;
    c->surfaceCount = 0;
    c->surfaceTiles = 0;
    c->ndirty = 0;
    if (n <= 0) return 0;

    /* surface: every segment walked in quarter-voxel steps (:79-94) */
    const float inv = 1.0f / c->vs;
    const float step = 0.25f * c->vs;
    long long total = 0;
    for (int s = 0; s < n; ++s) {
        vo_f2 a = poly[s], b = poly[(s + 1) % n];
        float len = hypotf(b.x - a.x, b.y - a.y);
        int m = (int)ceilf(len / step);
        total += m > 1 ? m : 1;
    }
    sample_t *smp = (sample_t *)malloc((size_t)(total ? total : 1) * sizeof(sample_t));
    if (!smp) return -1;
    int ns = 0, idx = 0;
    for (int s = 0; s < n; ++s) {
        vo_f2 a = poly[s], b = poly[(s + 1) % n];
        float len = hypotf(b.x - a.x, b.y - a.y);
        int m = (int)ceilf(len / step);
        if (m < 1) m = 1;
        for (int k = 0; k < m; ++k, ++idx) {
            float t = (float)k / (float)m;
            float x = a.x + t * (b.x - a.x), y = a.y + t * (b.y - a.y);
            int i = (int)floorf(x * inv), j = (int)floorf(y * inv);
            if (!in_domain(c, i, j)) continue;
            smp[ns].key = vkey(c, i, j);
            smp[ns].idx = idx;
            smp[ns].x = x;
            smp[ns].y = y;
            ++ns;
        }
    }
    /* slots in tile-major voxel order (:96-114) */
    qsort(smp, (size_t)ns, sizeof(sample_t), cmp_sample);
    for (int k = 0; k < ns;) {
        int e = k + 1;
        while (e < ns && smp[e].key == smp[k].key) ++e;
        long long v = smp[k].key;
        size_t t = (size_t)(v >> 6);
        if (!c->smask[t]) ++c->surfaceTiles;
        c->smask[t] |= (uint64_t)1 << (v & 63);
        c->spt[v] = run_mean(smp + k, e - k);
        c->sslot[v] = alloc_slot(c, c->spt[v]);
        if (c->sslot[v] < 0) {
            free(smp);
            return -1;
        }
        ++c->surfaceCount;
        k = e;
    }
    free(smp);

    /* occupancy: even-odd scanline fill through voxel centres (:116-133) */
    float *xs = (float *)malloc((size_t)n * sizeof(float));
    if (!xs) return -1;
    for (int j = 0; j < c->vy; ++j) {
        float y = ((float)j + 0.5f) * c->vs;
        int m = 0;
        for (int s = 0, t = n - 1; s < n; t = s++) {
            vo_f2 a = poly[s], b = poly[t];
            if ((a.y > y) != (b.y > y)) xs[m++] = a.x + (y - a.y) * (b.x - a.x) / (b.y - a.y);
        }
        qsort(xs, (size_t)m, sizeof(float), cmp_float);
        for (int k = 0; k + 1 < m; k += 2) {
            int i0 = (int)ceilf(xs[k] * inv - 0.5f);
            int i1 = (int)floorf(xs[k + 1] * inv - 0.5f);
            if (i0 < 0) i0 = 0;
            if (i1 > c->vx - 1) i1 = c->vx - 1;
            for (int i = i0; i <= i1; ++i)
                c->inside[(size_t)(j >> TILE_LOG2) * c->tx + (i >> TILE_LOG2)] |= (uint64_t)1 << bit_of(i, j);
        }
    }
    free(xs);
    return 0;
}

/* Canvas::StampDisc (canvas.cpp:136-221) */
int vo_canvas_stamp(vo_canvas *c, float cx, float cy, float radius, int inside, vo_canvas_edit *e)
{
    memset(e, 0, sizeof(*e));
    c->ndirty = 0;
    const float inv = 1.0f / c->vs;
    const float r2 = radius * radius;
    int i0 = (int)floorf((cx - radius) * inv), j0 = (int)floorf((cy - radius) * inv);
    int i1 = (int)floorf((cx + radius) * inv), j1 = (int)floorf((cy + radius) * inv);
    if (i0 < 0) i0 = 0;
    if (j0 < 0) j0 = 0;
    if (i1 > c->vx - 1) i1 = c->vx - 1;
    if (j1 > c->vy - 1) j1 = c->vy - 1;
    if (i0 > i1 || j0 > j1) return 0;
    inside = inside != 0;

    /* 1. rim samples on the other side of the current occupancy (:148-158) */
    int n = (int)ceilf(2.0f * 3.14159265f * radius / (0.25f * c->vs));
    if (n < 16) n = 16;
    sample_t *rim = (sample_t *)malloc((size_t)n * sizeof(sample_t));
    if (!rim) return -1;
    int nr = 0;
    for (int k = 0; k < n; ++k) {
        float a = 2.0f * 3.14159265f * (float)k / (float)n;
        float x = cx + radius * cosf(a), y = cy + radius * sinf(a);
        int i = (int)floorf(x * inv), j = (int)floorf(y * inv);
        if (in_domain(c, i, j) && is_inside(c, i, j) != inside) {
            rim[nr].key = vkey(c, i, j);
            rim[nr].idx = k;
            rim[nr].x = x;
            rim[nr].y = y;
            ++nr;
        }
    }
    qsort(rim, (size_t)nr, sizeof(sample_t), cmp_sample);

    /* 2. surface samples strictly inside the disc are deleted (:160-181) */
    for (int ty = j0 >> TILE_LOG2; ty <= j1 >> TILE_LOG2; ++ty) {
        for (int tx = i0 >> TILE_LOG2; tx <= i1 >> TILE_LOG2; ++tx) {
            size_t t = (size_t)ty * c->tx + tx;
            uint64_t before = c->smask[t];
            for (uint64_t m = before; m; m &= m - 1) {
                int bit = __builtin_ctzll(m);
                vo_f2 p = c->spt[t * 64 + bit];
                if ((p.x - cx) * (p.x - cx) + (p.y - cy) * (p.y - cy) >= r2) continue;
                c->smask[t] &= ~((uint64_t)1 << bit);
                int s = c->sslot[t * 64 + bit];
                if (free_slot(c, s) || push_dirty(c, s)) {
                    free(rim);
                    return -1;
                }
                --c->surfaceCount;
                ++e->removed;
            }
            if (before && !c->smask[t]) --c->surfaceTiles;
        }
    }

    /* 3. occupancy of voxel centres inside the disc (:183-197) */
    for (int j = j0; j <= j1; ++j) {
        float dy = ((float)j + 0.5f) * c->vs - cy;
        for (int i = i0; i <= i1; ++i) {
            float dx = ((float)i + 0.5f) * c->vs - cx;
            if (dx * dx + dy * dy >= r2) continue;
            uint64_t *word = &c->inside[(size_t)(j >> TILE_LOG2) * c->tx + (i >> TILE_LOG2)];
            uint64_t bit = (uint64_t)1 << bit_of(i, j);
            if (((*word & bit) != 0) != inside) {
                *word ^= bit;
                ++e->flipped;
            }
        }
    }

    /* 4. the kept rim becomes surface (:199-214), rim voxels in tile-major order */
    for (int k = 0; k < nr;) {
        int q = k + 1;
        while (q < nr && rim[q].key == rim[k].key) ++q;
        long long v = rim[k].key;
        size_t t = (size_t)(v >> 6);
        uint64_t bit = (uint64_t)1 << (v & 63);
        vo_f2 p = run_mean(rim + k, q - k);
        if (c->smask[t] & bit) {
            c->slots[c->sslot[v]] = p;
        } else {
            if (!c->smask[t]) ++c->surfaceTiles;
            c->smask[t] |= bit;
            c->sslot[v] = alloc_slot(c, p);
            if (c->sslot[v] < 0) {
                free(rim);
                return -1;
            }
            ++c->surfaceCount;
            ++e->added;
        }
        c->spt[v] = p;
        if (push_dirty(c, c->sslot[v])) {
            free(rim);
            return -1;
        }
        k = q;
    }
    free(rim);

    e->tx0 = i0 >> TILE_LOG2;
    e->ty0 = j0 >> TILE_LOG2;
    e->tx1 = (i1 >> TILE_LOG2) + 1;
    e->ty1 = (j1 >> TILE_LOG2) + 1;
    e->ndirty = c->ndirty;
    return 0;
}

void vo_canvas_dims(const vo_canvas *c, int *dims)
{
    dims[0] = c->vx;
    dims[1] = c->vy;
    dims[2] = c->tx;
    dims[3] = c->ty;
}

void vo_canvas_counts(const vo_canvas *c, long long *counts)
{
    counts[0] = c->nslots;
    counts[1] = c->nfree;
    counts[2] = c->surfaceCount;
    counts[3] = c->surfaceTiles;
}

void vo_canvas_get(const vo_canvas *c, vo_f2 *slots, int *freeList, uint64_t *inside, uint64_t *smask, vo_f2 *spt,
                   int *sslot, int *dirty)
{
    size_t tiles = (size_t)c->tx * c->ty;
    if (slots && c->nslots) memcpy(slots, c->slots, (size_t)c->nslots * sizeof(vo_f2));
    if (freeList && c->nfree) memcpy(freeList, c->freel, (size_t)c->nfree * sizeof(int));
    if (inside) memcpy(inside, c->inside, tiles * sizeof(uint64_t));
    if (smask) memcpy(smask, c->smask, tiles * sizeof(uint64_t));
    if (dirty && c->ndirty) memcpy(dirty, c->dirty, (size_t)c->ndirty * sizeof(int));
    for (size_t t = 0; t < tiles; ++t) {
        for (int b = 0; b < 64; ++b) {
            int on = (int)((c->smask[t] >> b) & 1u);
            if (spt) {
                vo_f2 off = {-1.0f, -1.0f};
                spt[t * 64 + b] = on ? c->spt[t * 64 + b] : off;
            }
            if (sslot) sslot[t * 64 + b] = on ? c->sslot[t * 64 + b] : -1;
        }
    }
}
