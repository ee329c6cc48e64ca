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

// The loss kernel's per-block flag: it met a gradient term beyond its fit's
// fastShift (see fx_from_float_any and vm_loss.cu).
__shared__ int sFastOver;

// round-half-even(v * 2^e) as int64, saturating at +-2^62, NaN -> 0; integer
// operations only (64-bit float->int conversions run on the narrow FP64 pipe).
// A term of 2^(fastShift + 24) or more (an infinite one included) raises
// the block's sFastOver; callers that do not check it pass fastShift = 64.
static __device__ __noinline__ long long fx_from_float_any(float v, int e, int fastShift)
{
    unsigned u = __float_as_uint(v);
    int ex = (int)((u >> 23) & 0xFFu);
    if (ex == 0xFF) {
        if (u & 0x7FFFFFu) return 0;
        if (fastShift < 64) sFastOver = 1;
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
    if (ex != 0 && k > fastShift) sFastOver = 1;
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
    return fx_from_float_any(v, e, 64);
}

__device__ __forceinline__ float fx_to_float(long long v, int e) { return __ll2float_rn(v) * pow2f(-e); }

// ---- exact per-site gradient sums ----------------------------------------------
// A site's gradient component is the exact integer sum S of its fixed-point
// terms (each at most 2^62 in magnitude). gradX holds three sections of
// 64-bit words per slot, (x, y) each:
//
//   L       the loss kernel's fast path: one 64-bit sum, exact modulo 2^64.
//           The fast path gives a target only sites of the 5x5 cell block
//           around its own cell, so a site receives at most T5 terms (T5: the
//           most live targets in any 5x5 block) and |S| <= T5 * max|term|.
//           The loss kernel converts terms below 2^(fastShift + 24) inline,
//           with fastShift = 38 - ceil(log2 T5) (vm_fast_shift), so those are
//           below 2^62 / T5 and no site sum can leave the int64 range: L
//           holds S itself. A larger term takes the out-of-line conversion,
//           which flags the block; the fit's whole gradient is then
//           recomputed into DL/DH (k_loss_exact), with L ignored.
//   DL, DH  the deferred (ring-search) targets and flagged fits, in the
//           unconditional split x = hi * 2^32 + lo, lo in [0, 2^32): a site
//           receives fewer than 2^31 terms, so neither word wraps.
//
// So every site sum is exact for any input, and the fast path costs one
// 64-bit reduction per component; the bound costs no instruction on the
// common path. At the 1M-site workload fastShift = 24 (terms up to 2^48)
// and the largest term is 2^40.7.

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

// v * 2^-e rounded once to float, v a 128-bit integer: the magnitude is
// shifted so its leading one is bit 63 of a 64-bit word, the bits shifted
// out are folded into bit 0 as a sticky bit (far below the rounding
// position), and the word is converted with round-to-nearest-even and scaled
// back by powers of two (exact).
__host__ __device__ __noinline__ inline float i128_to_float(__int128 v, int e)
{
    bool neg = v < 0;
    unsigned __int128 m = neg ? (unsigned __int128)0 - (unsigned __int128)v : (unsigned __int128)v;
    unsigned long long hi = (unsigned long long)(m >> 64), lo = (unsigned long long)m;
    float f;
    if (hi == 0) {
        f = vm_u64_to_float(lo);
    } else {
#ifdef __CUDA_ARCH__
        int c = __clzll((long long)hi);
#else
        int c = __builtin_clzll(hi);
#endif
        unsigned long long top = c ? (hi << c) | (lo >> (64 - c)) : hi;
        unsigned long long rest = lo << c;
        top |= rest != 0 ? 1ull : 0ull;
        f = vm_u64_to_float(top) * vm_pow2f(64 - c);
    }
    if (neg) f = -f;
    return f * vm_pow2f(-e);
}

// The site sum of one component, rounded once to float and scaled by 2^-e:
// L (when useL) plus DH * 2^32 + DL.
__host__ __device__ __noinline__ inline float fx_site_to_float(long long L, bool useL, unsigned long long DL,
                                                               long long DH, int e)
{
    __int128 v = (useL ? (__int128)L : (__int128)0) + (__int128)DH * ((__int128)1 << 32) + (__int128)DL;
    return i128_to_float(v, e);
}

// Adds a contribution (x, y) to site s in the unconditional split words
// (sections DL and DH of G, n slots).
static __device__ __noinline__ void fxd_red(unsigned long long *G, int n, int s, long long x, long long y, int *dUsed)
{
    unsigned long long *DL = G + 2 * (size_t)n + 2 * (size_t)s, *DH = DL + 2 * (size_t)n;
    if (x) {
        atomicAdd(&DL[0], (unsigned long long)x & 0xFFFFFFFFull);
        if (x >> 32) atomicAdd(&DH[0], (unsigned long long)(x >> 32));
    }
    if (y) {
        atomicAdd(&DL[1], (unsigned long long)y & 0xFFFFFFFFull);
        if (y >> 32) atomicAdd(&DH[1], (unsigned long long)(y >> 32));
    }
    atomicOr(dUsed, 1);
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
// The same header lists the fits whose fast-path gradient bound failed in
// the current pass (see the exact per-site sums above); k_loss_exact
// recomputes their gradients.
constexpr int kMaxFlagged = 256;
struct SlowQueue {
    int count;
    int capacity;
    int2 *items; // (fit, local target index)
    int nFlagged;
    int flagged[kMaxFlagged];
};

} // namespace vmk
