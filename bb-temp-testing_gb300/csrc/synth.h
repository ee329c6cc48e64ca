/*
 * Seeded synthetic point sets for the VoroMesh workloads (host code, no GPU).
 * Identical bytes on x86_64 and aarch64 for the same (seed, stream).
 * Points are float2 pairs (x, y) written to `out`; `shift` adds 1.0f to both
 * coordinates, mapping the [-1,1]^2 design space onto the [0,2]^2 domain.
 */
#ifndef VM_SYNTH_H
#define VM_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* n points uniform in [lo,hi)^2 */
void vm_synth_uniform(uint64_t seed, uint64_t stream, int64_t n, double lo, double hi, int shift, float *out);
/* n points at uniform angle on a circle, radius + sigma * N(0,1) */
void vm_synth_circle(uint64_t seed, uint64_t stream, int64_t n, double radius, double sigma, int shift,
                     float *out);
/* nx*ny lattice cell centres on [-1,1]^2, each coordinate jittered by U(-jitter, jitter) */
void vm_synth_lattice(uint64_t seed, uint64_t stream, int nx, int ny, double jitter, int shift, float *out);
/* `count` ellipses: centre U[-.8,.8]^2, semi-axes U[.05,.3], angle U[0,pi] (5 doubles each) */
void vm_synth_ellipse_params(uint64_t seed, uint64_t stream, int count, double *params);
/* n points on the boundary of the union of those ellipses (uniform by arc
 * length on a perimeter-weighted ellipse, rejected when inside another one or
 * outside [-1,1)^2).
 * Returns the number of points written (n unless the attempt cap is hit). */
int64_t vm_synth_ellipse_union(uint64_t seed, uint64_t stream, int count, int64_t n, int shift, float *out);
/* n points uniform by arc length on a star outline with 2*arms vertices */
void vm_synth_star(uint64_t seed, uint64_t stream, int arms, const double *radii, double rot, double cx,
                   double cy, int64_t n, int shift, float *out);
/* random star: arms U{5..40}, 2*arms radii U[.2,.9], rotation U[0,2pi) */
void vm_synth_star_params(uint64_t seed, uint64_t stream, int *arms, double *radii, double *rot);
/* k of [0,n) chosen uniformly, ascending; 0 on success */
int vm_synth_subset(uint64_t seed, uint64_t stream, int64_t n, int64_t k, int64_t *out);
/* n uniform doubles in [0,1) */
double vm_synth_uniform01(uint64_t seed, uint64_t stream, int64_t n, double *out);
double vm_synth_log(double x);
double vm_synth_exp(double x);

#ifdef __cplusplus
}
#endif

#endif
