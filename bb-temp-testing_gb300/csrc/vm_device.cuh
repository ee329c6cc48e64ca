// Device helpers shared by the VoroMesh kernels.
//
// Every translation unit that includes this file is compiled with
// --fmad=false, so a*b+c is two IEEE-rounded operations exactly as in the
// reference source read literally; intrinsics (__fmaf_rn) are used only
// where a fused operation is intended.
#pragma once

#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

#include "vm_types.h"

namespace vmk {

constexpr unsigned kFull = 0xFFFFFFFFu;

// cellCoord (reference voro_optimizer.cu:123-125): clamp(int(v * inv), 0, n-1)
// with the GPU's saturating float->int conversion (NaN -> 0).
__device__ __forceinline__ int cell_coord(float v, float inv, int n)
{
    int c = __float2int_rz(v * inv);
    return min(max(c, 0), n - 1);
}

// (d2, index) ascending; index -1 (an empty entry) sorts last.
__device__ __forceinline__ bool key_less(float dd, int id, float D, int I)
{
    return dd < D || (dd == D && (unsigned)id < (unsigned)I);
}

// Stateless RNG (reference voro_optimizer.cu:69-78, poisson_disk.cu:47-58).
__host__ __device__ __forceinline__ unsigned pcg_hash(unsigned v)
{
    unsigned state = v * 747796405u + 2891336453u;
    unsigned word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

__device__ __forceinline__ float rand01(unsigned index, unsigned iter, unsigned seed)
{
    unsigned h = pcg_hash(index ^ pcg_hash(iter * 2654435761u ^ pcg_hash(seed)));
    return (float)(h & 0x00FFFFFFu) * (1.0f / 16777216.0f);
}

// ---- fixed-point accumulation ------------------------------------------------
// Gradient components are summed as int64 of round-half-even(v * 2^e); the
// loss as a 128-bit integer floor(v * 2^e) built from the float's bits. Both
// sums are exact integer additions, so the result does not depend on the
// order in which targets, warps or blocks contribute.
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((e + 127) << 23); }

// round-half-even(v * 2^e) as int64, saturating at +-2^62, NaN -> 0; integer
// operations only (64-bit float->int conversions run on the narrow FP64 pipe).
static __device__ __noinline__ long long fx_from_float_any(float v, int e)
{
    unsigned u = __float_as_uint(v);
    int ex = (int)((u >> 23) & 0xFFu);
    if (ex == 0xFF) return (u & 0x7FFFFFu) ? 0 : ((u >> 31) ? -4611686018427387904LL : 4611686018427387904LL);
    unsigned m = u & 0x7FFFFFu;
    int k; // |v| 2^e = m 2^k
    if (ex == 0) { // subnormal v
        if (!m) return 0;
        k = -149 + e;
    } else {
        m |= 0x800000u;
        k = ex - 150 + e;
    }
    long long mag;
    if (k >= 0) {
        mag = k > 38 ? 4611686018427387904LL : ((long long)m << k);
    } else if (k < -24) {
        mag = 0;
    } else {
        int r = -k;
        unsigned q = m >> r;
        unsigned rem = m & ((1u << r) - 1u);
        unsigned half = 1u << (r - 1);
        q += (rem > half || (rem == half && (q & 1u))) ? 1u : 0u;
        mag = q;
    }
    return (u >> 31) ? -mag : mag;
}

// The same with the common case inline: a normal v whose scaled value is an
// integer below 2^62 (a plain shift of the significand, no rounding).
__device__ __forceinline__ long long fx_from_float(float v, int e)
{
    unsigned u = __float_as_uint(v);
    int ex = (int)((u >> 23) & 0xFFu);
    int k = ex - 150 + e;
    if ((unsigned)(ex - 1) < 254u && (unsigned)k <= 38u) {
        long long mag = (long long)((u & 0x7FFFFFu) | 0x800000u) << k;
        return (u >> 31) ? -mag : mag;
    }
    return fx_from_float_any(v, e);
}

__device__ __forceinline__ float fx_to_float(long long v, int e) { return __ll2float_rn(v) * pow2f(-e); }

__device__ __forceinline__ void fxl_from_float(float v, int e, unsigned long long &lo, unsigned long long &hi)
{
    lo = 0;
    hi = 0;
    if (!(v > 0.0f)) return;
    unsigned bits = __float_as_uint(v);
    int ex = (int)((bits >> 23) & 0xFFu);
    unsigned long long m = bits & 0x7FFFFFu;
    if (ex == 0xFF) {
        hi = 1ULL << 62;
        return;
    }
    int k;
    if (ex == 0) k = -149 + e;
    else {
        m |= 0x800000u;
        k = ex - 150 + e;
    }
    if (k >= 104) hi = 1ULL << 62;
    else if (k >= 64) hi = m << (k - 64);
    else if (k > 0) {
        lo = m << k;
        hi = m >> (64 - k);
    } else if (k == 0) lo = m;
    else if (k > -64) lo = m >> (-k);
}

__device__ __forceinline__ float fxl_to_float(unsigned long long lo, unsigned long long hi, int e)
{
    double d = __dmul_rn(__ull2double_rn(hi), 18446744073709551616.0);
    d = __dadd_rn(d, __ull2double_rn(lo));
    d = __dmul_rn(d, __longlong_as_double((long long)(1023 - e) << 52));
    return __double2float_rn(d);
}

__device__ __forceinline__ void add128(unsigned long long &lo, unsigned long long &hi, unsigned long long blo,
                                       unsigned long long bhi)
{
    unsigned long long n = lo + blo;
    hi = hi + bhi + (n < lo ? 1ull : 0ull);
    lo = n;
}

// 128-bit atomic add as two 64-bit atomics; the carry of the low word is
// detected from its old value, so concurrent adders compose exactly.
__device__ __forceinline__ void atomic_add128(unsigned long long *lo, unsigned long long *hi, unsigned long long vlo,
                                              unsigned long long vhi)
{
    if (vlo) {
        unsigned long long old = atomicAdd(lo, vlo);
        if (old + vlo < old) vhi += 1ull;
    }
    if (vhi) atomicAdd(hi, vhi);
}

// Block index -> fit index by binary search in prefix[0..nFits] (prefix[0]=0).
__device__ __forceinline__ int find_fit(const int *prefix, int nFits, int b)
{
    int lo = 0, hi = nFits - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(&prefix[mid]) <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// base^t in double by exponentiation by squaring, rounded to float once: a
// deterministic stand-in for powf in the Adam bias corrections.
__device__ __forceinline__ float pow_det(float base, int t)
{
    double r = 1.0, x = (double)base;
    unsigned e = t < 0 ? 0u : (unsigned)t;
    while (e) {
        if (e & 1u) r = __dmul_rn(r, x);
        x = __dmul_rn(x, x);
        e >>= 1;
    }
    return __double2float_rn(r);
}

// The learning rate (MultiStepLR) and bias corrections of fit F's next step
// t = iter + 1 (reference adamKernel, voro_optimizer.cu:271-301), written to
// its state for the Adam kernel.
__device__ __forceinline__ void adam_schedule(const VmFit &F)
{
    VmState *st = F.state;
    int t = st->iter + 1;
    float lr = F.lr;
    for (int k = 0; k < 4; ++k)
        if (t - 1 >= F.milestones[k]) lr *= F.gamma;
    st->schedLr = lr;
    st->schedBc1 = 1.0f - pow_det(F.beta1, t);
    st->schedBc2 = 1.0f - pow_det(F.beta2, t);
}

// Targets the loss kernel's block certificates could not settle are deferred
// to this queue and resolved by k_loss_exact in dense warps, so one hard
// target does not stall the 31 other lanes of its warp on the long ring
// search. The queue holds every live target, so it cannot overflow.
struct SlowQueue {
    int count;
    int capacity;
    int2 *items; // (fit, local target index)
};

} // namespace vmk
