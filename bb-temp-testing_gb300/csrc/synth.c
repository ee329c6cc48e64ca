/*
 * Seeded synthetic inputs for the VoroMesh workloads.
 *
 * Every generator here uses only integer arithmetic and the five correctly
 * rounded IEEE double operations (+ - * / sqrt), compiled without FP
 * contraction, so the same seed yields the same bytes on x86_64 and aarch64.
 * Transcendentals (sin, cos, log) are evaluated by the short series below
 * instead of the platform libm for that reason.
 *
 * Coordinates: shapes are defined on [-1,1]^2 and shifted by +1 (one float
 * add) into the optimiser's [0,2]^2 domain when `shift` is non-zero, so the
 * configs keep their stated geometry while the domain stays [0,w]x[0,h].
 */
#include "synth.h"

#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ---- PCG32 (O'Neill 2014): 64-bit LCG state, XSH-RR output -------------- */
typedef struct {
    uint64_t state, inc;
} pcg32;

static uint32_t pcg32_next(pcg32 *r)
{
    uint64_t old = r->state;
    r->state = old * 6364136223846793005ULL + r->inc;
    uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
}

static void pcg32_seed(pcg32 *r, uint64_t seed, uint64_t stream)
{
    r->state = 0u;
    r->inc = (stream << 1u) | 1u;
    pcg32_next(r);
    r->state += seed;
    pcg32_next(r);
}

/* uniform double in [0,1) with 53 random bits */
static double unif(pcg32 *r)
{
    uint64_t hi = pcg32_next(r), lo = pcg32_next(r);
    uint64_t v = ((hi << 32) | lo) >> 11;
    return (double)v * (1.0 / 9007199254740992.0);
}

/* uniform integer in [0, n) without modulo bias */
static uint32_t unif_int(pcg32 *r, uint32_t n)
{
    uint32_t threshold = (uint32_t)(-n) % n;
    for (;;) {
        uint32_t v = pcg32_next(r);
        if (v >= threshold) return v % n;
    }
}

/* ---- portable transcendentals ------------------------------------------- */
static const double kPi = 3.14159265358979323846;

/* sin and cos of x after reduction to [-pi/4, pi/4]; Taylor series to x^17. */
static double sin_poly(double x)
{
    double x2 = x * x, term = x, sum = x;
    for (int k = 1; k <= 8; ++k) {
        term = -term * x2 / (double)((2 * k) * (2 * k + 1));
        sum = sum + term;
    }
    return sum;
}

static double cos_poly(double x)
{
    double x2 = x * x, term = 1.0, sum = 1.0;
    for (int k = 1; k <= 8; ++k) {
        term = -term * x2 / (double)((2 * k - 1) * (2 * k));
        sum = sum + term;
    }
    return sum;
}

static void sincos_det(double a, double *s, double *c)
{
    /* reduce to a in [0, 2pi), then to quadrant q and r in [-pi/4, pi/4] */
    double twopi = 2.0 * kPi;
    double k = (double)(int64_t)(a / twopi);
    a = a - k * twopi;
    if (a < 0.0) a = a + twopi;
    int64_t q = (int64_t)(a / (0.5 * kPi) + 0.5);
    double r = a - (double)q * (0.5 * kPi);
    double sr = sin_poly(r), cr = cos_poly(r);
    switch (q & 3) {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = -sr; break;
    case 2: *s = -sr; *c = -cr; break;
    default: *s = -cr; *c = sr; break;
    }
}

/* natural log for x > 0: x = m 2^e with m in [sqrt(.5), sqrt(2)), then the
 * atanh series ln(m) = 2 (z + z^3/3 + ...), z = (m-1)/(m+1). */
static double log_det(double x)
{
    if (!(x > 0.0)) return -1e300;
    int e = 0;
    while (x >= 1.4142135623730951) { x = x * 0.5; ++e; }
    while (x < 0.7071067811865476) { x = x * 2.0; --e; }
    double z = (x - 1.0) / (x + 1.0), z2 = z * z, term = z, sum = z;
    for (int k = 1; k < 30; ++k) {
        term = term * z2;
        sum = sum + term / (double)(2 * k + 1);
    }
    return 2.0 * sum + (double)e * 0.69314718055994530942;
}

static double exp_det(double x)
{
    /* x = n ln2 + r, |r| <= ln2/2; Taylor series of e^r */
    double ln2 = 0.69314718055994530942;
    double nd = x / ln2;
    int64_t n = (int64_t)(nd < 0.0 ? nd - 0.5 : nd + 0.5);
    double r = x - (double)n * ln2, term = 1.0, sum = 1.0;
    for (int k = 1; k < 25; ++k) {
        term = term * r / (double)k;
        sum = sum + term;
    }
    while (n > 0) { sum = sum * 2.0; --n; }
    while (n < 0) { sum = sum * 0.5; ++n; }
    return sum;
}

/* standard normal by Box-Muller (one of the pair) */
static double normal(pcg32 *r)
{
    double u1 = unif(r), u2 = unif(r);
    if (u1 < 1e-300) u1 = 1e-300;
    double s, c;
    sincos_det(2.0 * kPi * u2, &s, &c);
    double m = -2.0 * log_det(u1);
    return __builtin_sqrt(m) * c;
}

static void put(float *out, int64_t i, double x, double y, int shift)
{
    float fx = (float)x, fy = (float)y;
    if (shift) { fx = fx + 1.0f; fy = fy + 1.0f; }
    out[2 * i] = fx;
    out[2 * i + 1] = fy;
}

/* ---- public generators --------------------------------------------------- */

void vm_synth_uniform(uint64_t seed, uint64_t stream, int64_t n, double lo, double hi, int shift,
                      float *out)
{
    pcg32 r;
    pcg32_seed(&r, seed, stream);
    for (int64_t i = 0; i < n; ++i) {
        double x = lo + (hi - lo) * unif(&r);
        double y = lo + (hi - lo) * unif(&r);
        put(out, i, x, y, shift);
    }
}

void vm_synth_circle(uint64_t seed, uint64_t stream, int64_t n, double radius, double sigma, int shift,
                     float *out)
{
    pcg32 r;
    pcg32_seed(&r, seed, stream);
    for (int64_t i = 0; i < n; ++i) {
        double th = 2.0 * kPi * unif(&r);
        double rad = radius + sigma * normal(&r);
        double s, c;
        sincos_det(th, &s, &c);
        put(out, i, rad * c, rad * s, shift);
    }
}

void vm_synth_lattice(uint64_t seed, uint64_t stream, int nx, int ny, double jitter, int shift, float *out)
{
    pcg32 r;
    pcg32_seed(&r, seed, stream);
    double px = 2.0 / nx, py = 2.0 / ny;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            double x = -1.0 + (i + 0.5) * px + jitter * (2.0 * unif(&r) - 1.0);
            double y = -1.0 + (j + 0.5) * py + jitter * (2.0 * unif(&r) - 1.0);
            put(out, (int64_t)j * nx + i, x, y, shift);
        }
}

/* Ellipse e: centre (cx,cy), semi-axes (a,b), rotation t. */
typedef struct {
    double cx, cy, a, b, cs, sn, perim;
} ellipse;

static int inside_ellipse(const ellipse *e, double x, double y)
{
    double dx = x - e->cx, dy = y - e->cy;
    double u = dx * e->cs + dy * e->sn, v = -dx * e->sn + dy * e->cs;
    return (u * u) / (e->a * e->a) + (v * v) / (e->b * e->b) < 1.0;
}

void vm_synth_ellipse_params(uint64_t seed, uint64_t stream, int count, double *params /* 5 per ellipse */)
{
    pcg32 r;
    pcg32_seed(&r, seed, stream);
    for (int k = 0; k < count; ++k) {
        params[5 * k + 0] = -0.8 + 1.6 * unif(&r);
        params[5 * k + 1] = -0.8 + 1.6 * unif(&r);
        params[5 * k + 2] = 0.05 + 0.25 * unif(&r);
        params[5 * k + 3] = 0.05 + 0.25 * unif(&r);
        params[5 * k + 4] = kPi * unif(&r);
    }
}

int64_t vm_synth_ellipse_union(uint64_t seed, uint64_t stream, int count, int64_t n, int shift, float *out)
{
    ellipse *es = (ellipse *)malloc(sizeof(ellipse) * (size_t)(count > 0 ? count : 1));
    double *prm = (double *)malloc(sizeof(double) * 5 * (size_t)(count > 0 ? count : 1));
    if (!es || !prm || count <= 0) { free(es); free(prm); return 0; }
    vm_synth_ellipse_params(seed, stream, count, prm);
    double total = 0.0;
    for (int k = 0; k < count; ++k) {
        ellipse *e = &es[k];
        e->cx = prm[5 * k]; e->cy = prm[5 * k + 1];
        e->a = prm[5 * k + 2]; e->b = prm[5 * k + 3];
        sincos_det(prm[5 * k + 4], &e->sn, &e->cs);
        /* Ramanujan's perimeter approximation: only weights the ellipse choice */
        double h = (e->a - e->b) * (e->a - e->b) / ((e->a + e->b) * (e->a + e->b));
        e->perim = kPi * (e->a + e->b) * (1.0 + 3.0 * h / (10.0 + __builtin_sqrt(4.0 - 3.0 * h)));
        total += e->perim;
    }
    pcg32 r;
    pcg32_seed(&r, seed, stream + 1000003u);
    int64_t made = 0;
    int64_t attempts = 0, limit = 200 * (n + 1000);
    while (made < n && attempts < limit) {
        ++attempts;
        /* ellipse by perimeter, then a point uniform by arc length (rejection on |dP/dt|) */
        double pick = unif(&r) * total, acc = 0.0;
        int k = 0;
        for (; k < count - 1; ++k) {
            acc += es[k].perim;
            if (pick < acc) break;
        }
        const ellipse *e = &es[k];
        double s, c, t;
        for (;;) {
            t = 2.0 * kPi * unif(&r);
            sincos_det(t, &s, &c);
            double speed = __builtin_sqrt(e->a * e->a * s * s + e->b * e->b * c * c);
            double vmax = e->a > e->b ? e->a : e->b;
            if (unif(&r) * vmax <= speed) break;
        }
        double u = e->a * c, v = e->b * s;
        double x = e->cx + u * e->cs - v * e->sn;
        double y = e->cy + u * e->sn + v * e->cs;
        /* keep the shape inside the [-1,1]^2 design domain */
        if (x < -1.0 || x >= 1.0 || y < -1.0 || y >= 1.0) continue;
        int hidden = 0;
        for (int q = 0; q < count && !hidden; ++q)
            if (q != k && inside_ellipse(&es[q], x, y)) hidden = 1;
        if (hidden) continue;
        put(out, made, x, y, shift);
        ++made;
    }
    free(es);
    free(prm);
    return made;
}

/* Star polygon: `arms` outer vertices interleaved with `arms` inner vertices,
 * vertex k at angle 2 pi k / (2 arms) + rot and radius radii[k]. Points are
 * uniform by arc length along the closed outline. */
void vm_synth_star(uint64_t seed, uint64_t stream, int arms, const double *radii, double rot, double cx,
                   double cy, int64_t n, int shift, float *out)
{
    int nv = 2 * arms;
    double *vx = (double *)malloc(sizeof(double) * (size_t)nv);
    double *vy = (double *)malloc(sizeof(double) * (size_t)nv);
    double *cum = (double *)malloc(sizeof(double) * (size_t)(nv + 1));
    if (!vx || !vy || !cum || nv < 3) { free(vx); free(vy); free(cum); return; }
    for (int k = 0; k < nv; ++k) {
        double s, c;
        sincos_det(2.0 * kPi * k / nv + rot, &s, &c);
        vx[k] = cx + radii[k] * c;
        vy[k] = cy + radii[k] * s;
    }
    cum[0] = 0.0;
    for (int k = 0; k < nv; ++k) {
        int k1 = (k + 1) % nv;
        double dx = vx[k1] - vx[k], dy = vy[k1] - vy[k];
        cum[k + 1] = cum[k] + __builtin_sqrt(dx * dx + dy * dy);
    }
    pcg32 r;
    pcg32_seed(&r, seed, stream);
    for (int64_t i = 0; i < n; ++i) {
        double at = unif(&r) * cum[nv];
        int lo = 0, hi = nv - 1;
        while (lo < hi) { /* last edge with cum[k] <= at */
            int mid = (lo + hi + 1) / 2;
            if (cum[mid] <= at) lo = mid; else hi = mid - 1;
        }
        int k = lo, k1 = (k + 1) % nv;
        double len = cum[k + 1] - cum[k];
        double f = len > 0.0 ? (at - cum[k]) / len : 0.0;
        put(out, i, vx[k] + f * (vx[k1] - vx[k]), vy[k] + f * (vy[k1] - vy[k]), shift);
    }
    free(vx);
    free(vy);
    free(cum);
}

void vm_synth_star_params(uint64_t seed, uint64_t stream, int *arms, double *radii /* >= 80 */, double *rot)
{
    pcg32 r;
    pcg32_seed(&r, seed, stream);
    *arms = 5 + (int)unif_int(&r, 36u);
    for (int k = 0; k < 2 * *arms; ++k) radii[k] = 0.2 + 0.7 * unif(&r);
    *rot = 2.0 * kPi * unif(&r);
}

/* Seeded uniform choice of k of the n indices [0, n) (partial Fisher-Yates),
 * returned in ascending order. */
int vm_synth_subset(uint64_t seed, uint64_t stream, int64_t n, int64_t k, int64_t *out)
{
    if (k > n || k < 0) return -1;
    int64_t *perm = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    if (!perm) return -2;
    for (int64_t i = 0; i < n; ++i) perm[i] = i;
    pcg32 r;
    pcg32_seed(&r, seed, stream);
    for (int64_t i = 0; i < k; ++i) {
        uint64_t span = (uint64_t)(n - i);
        uint64_t pick;
        if (span <= 0xFFFFFFFFu) pick = unif_int(&r, (uint32_t)span);
        else pick = ((uint64_t)pcg32_next(&r) << 32 | pcg32_next(&r)) % span;
        int64_t j = i + (int64_t)pick;
        int64_t t = perm[i]; perm[i] = perm[j]; perm[j] = t;
    }
    /* ascending order via counting on a bitmap */
    unsigned char *mark = (unsigned char *)calloc((size_t)(n > 0 ? n : 1), 1);
    if (!mark) { free(perm); return -2; }
    for (int64_t i = 0; i < k; ++i) mark[perm[i]] = 1;
    int64_t w = 0;
    for (int64_t i = 0; i < n; ++i)
        if (mark[i]) out[w++] = i;
    free(mark);
    free(perm);
    return 0;
}

double vm_synth_uniform01(uint64_t seed, uint64_t stream, int64_t n, double *out)
{
    pcg32 r;
    pcg32_seed(&r, seed, stream);
    for (int64_t i = 0; i < n; ++i) out[i] = unif(&r);
    return n > 0 ? out[0] : 0.0;
}

double vm_synth_log(double x) { return log_det(x); }
double vm_synth_exp(double x) { return exp_det(x); }
