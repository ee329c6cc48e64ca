// Device helpers shared by the VoroMesh kernels.
//
// Every translation unit that includes this file is compiled with
// --fmad=false, so a*b+c is two IEEE-rounded operations exactly as in the
// reference source read literally; intrinsics (__fmaf_rn) are used only
// where a fused operation is intended.
#pragma once

#include <cfloat>
#include <cmath>
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
// A saturated term (|v| 2^e >= 2^62: near-coincident sites) is counted in
// *clamped when that pointer is given.
static __device__ __noinline__ long long fx_from_float_any(float v, int e, int *clamped)
{
    unsigned u = __float_as_uint(v);
    int ex = (int)((u >> 23) & 0xFFu);
    if (ex == 0xFF) {
        if (u & 0x7FFFFFu) return 0;
        if (clamped) atomicAdd(clamped, 1);
        return (u >> 31) ? -4611686018427387904LL : 4611686018427387904LL;
    }
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
        if (k > 38 && clamped) atomicAdd(clamped, 1);
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
__device__ __forceinline__ long long fx_from_float(float v, int e, int *clamped = nullptr)
{
    unsigned u = __float_as_uint(v);
    int ex = (int)((u >> 23) & 0xFFu);
    int k = ex - 150 + e;
    if ((unsigned)(ex - 1) < 254u && (unsigned)k <= 38u) {
        long long mag = (long long)((u & 0x7FFFFFu) | 0x800000u) << k;
        return (u >> 31) ? -mag : mag;
    }
    return fx_from_float_any(v, e, clamped);
}

__device__ __forceinline__ float fx_to_float(long long v, int e) { return __ll2float_rn(v) * pow2f(-e); }

// ---- exact per-site gradient sums ----------------------------------------------
// A site's gradient component is the exact integer sum S of int64
// contributions x (|x| < 2^63). Each x is split as x = hi * 2^32 + lo with
// lo = x mod 2^32 in [0, 2^32) and hi = x >> 32 (arithmetic), and the site
// keeps L = sum(lo) (unsigned) and H = sum(hi) (signed) in two 64-bit words.
// A site receives fewer than 2^31 contributions (one per target at most), so
// L < 2^63 and |H| < 2^62: neither word wraps and S = H * 2^32 + L exactly,
// for any input, where one 64-bit sum would wrap past 2^63. Per slot the
// words are laid out as {Lx, Ly, Hx, Hy} (kGradWords per slot).

__host__ __device__ __forceinline__ float vm_pow2f(int e)
{
#ifdef __CUDA_ARCH__
    return __int_as_float((e + 127) << 23);
#else
    return ldexpf(1.0f, e);
#endif
}

__host__ __device__ __forceinline__ float vm_u64_to_float(unsigned long long v)
{
#ifdef __CUDA_ARCH__
    return __ull2float_rn(v);
#else
    return (float)v;
#endif
}

__host__ __device__ __forceinline__ float vm_s64_to_float(long long v)
{
#ifdef __CUDA_ARCH__
    return __ll2float_rn(v);
#else
    return (float)v;
#endif
}

// S * 2^-e rounded once to float when |S| >= 2^63 (T = S >> 32 outside the
// int32 range, low = S mod 2^32): the 128-bit magnitude is shifted so its
// leading one is bit 63 of a 64-bit word, the bits shifted out are folded
// into bit 0 as a sticky bit (far below the rounding position), and the word
// is converted with round-to-nearest-even and scaled back by a power of two.
__host__ __device__ __noinline__ inline float fx2_to_float_wide(long long T, unsigned long long low, int e)
{
    unsigned long long lo = ((unsigned long long)T << 32) | low;
    unsigned long long hi = (unsigned long long)(T >> 32);
    bool neg = T < 0;
    if (neg) {
        lo = ~lo + 1ull;
        hi = ~hi + (lo == 0 ? 1ull : 0ull);
    }
    float f;
    if (hi == 0) {
        f = vm_u64_to_float(lo);
    } else {
#ifdef __CUDA_ARCH__
        int c = __clzll((long long)hi);
#else
        int c = __builtin_clzll(hi);
#endif
        // |S| < 2^95, so hi < 2^31 and c is in [33, 63]
        unsigned long long top = (hi << c) | (lo >> (64 - c));
        unsigned long long rest = lo << c;
        top |= rest != 0 ? 1ull : 0ull;
        f = vm_u64_to_float(top) * vm_pow2f(64 - c);
    }
    if (neg) f = -f;
    return f * vm_pow2f(-e);
}

// S * 2^-e, S = H * 2^32 + L, rounded once to float (the same value as
// converting S exactly and scaling, which is what (float)S * 2^-e gives when
// S fits an int64).
__host__ __device__ __forceinline__ float fx2_to_float(long long H, unsigned long long L, int e)
{
    long long T = H + (long long)(L >> 32); // S = T * 2^32 + (L mod 2^32)
    unsigned long long low = L & 0xFFFFFFFFull;
    if (T >= -2147483648LL && T <= 2147483647LL)
        return vm_s64_to_float((long long)(((unsigned long long)T << 32) | low)) * vm_pow2f(-e);
    return fx2_to_float_wide(T, low, e);
}

// Adds contributions x, y to the split words of site s (G: kGradWords per slot).
__device__ __forceinline__ void fx2_red(unsigned long long *G, int s, long long x, long long y)
{
    unsigned long long *g = G + (size_t)kGradWords * s;
    if (x) {
        atomicAdd(&g[0], (unsigned long long)x & 0xFFFFFFFFull);
        long long h = x >> 32;
        if (h) atomicAdd(&g[2], (unsigned long long)h);
    }
    if (y) {
        atomicAdd(&g[1], (unsigned long long)y & 0xFFFFFFFFull);
        long long h = y >> 32;
        if (h) atomicAdd(&g[3], (unsigned long long)h);
    }
}

// |v| < 2^62: a further term (|x| <= 2^62) can be added without overflow.
__device__ __forceinline__ bool fx_small(long long v)
{
    return (unsigned)((int)(v >> 32) + 0x40000000) < 0x80000000u;
}

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
