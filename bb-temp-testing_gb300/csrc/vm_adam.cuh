// Adam for one slot (reference adamKernel, voro_optimizer.cu:271-301), shared
// by the batch-table Adam kernel (vm_step.cu) and the one-block step of a
// small fit (vm_loss.cu).
#pragma once

#include "vm_device.cuh"

namespace vmk {

// This step's Adam values of a fit, read once per thread: the lr and bias
// corrections (adam_schedule, run by the loss pass), the gradient's 1 / count,
// and which gradient words hold the sums.
struct AdamStep {
    float lr, bc1, bc2, scale;
    bool split, useL;
};

__device__ __forceinline__ AdamStep adam_step(const VmFit &F)
{
    const VmState *st = F.state;
    AdamStep a;
    a.lr = st->schedLr;
    a.bc1 = st->schedBc1;
    a.bc2 = st->schedBc2;
    int count = st->accCount;
    a.scale = 1.0f / (float)(count > 1 ? count : 1);
    a.split = (st->dUsed | st->needExact) != 0;
    a.useL = !st->needExact;
    return a;
}

// Adam and the clamp for slot i (reference adamKernel, voro_optimizer.cu:271-301):
// reads and clears the slot's gradient words, updates gen, m and v; returns
// the slot's new position (x < 0: an empty slot).
__device__ __forceinline__ float2 adam_slot(const VmFit &F, const AdamStep &a, int i)
{
    // this slot's gradient: section L of gradX (one 64-bit sum per component)
    // or, when the pass used the exact split words (deferred targets, or a
    // fit whose fast-path bound failed), the exact sum of all three sections;
    // the words are cleared for the next step
    longlong2 *gw = reinterpret_cast<longlong2 *>(F.gradX) + i;
    // the slot's words are loaded together (m and v also for an empty slot,
    // which leaves them unused)
    longlong2 gl = gw[0];
    float2 p = F.gen[i], m = F.m[i], v = F.v[i];
    if (gl.x | gl.y) gw[0] = make_longlong2(0, 0);
    float lr = a.lr, bc1 = a.bc1, bc2 = a.bc2, scale = a.scale;
    float grx, gry;
    if (!a.split) {
        // a zero sum is +0 either way; it skips the 64-bit conversion
        grx = gl.x ? scale * fx_to_float(gl.x, F.gradExp) : 0.0f;
        gry = gl.y ? scale * fx_to_float(gl.y, F.gradExp) : 0.0f;
    } else {
        size_t sec = (size_t)F.nSlots;
        longlong2 gdl = gw[sec], gdh = gw[2 * sec];
        gw[sec] = make_longlong2(0, 0);
        gw[2 * sec] = make_longlong2(0, 0);
        grx = scale * fx_site_to_float(gl.x, a.useL, (unsigned long long)gdl.x, gdh.x, F.gradExp);
        gry = scale * fx_site_to_float(gl.y, a.useL, (unsigned long long)gdl.y, gdh.y, F.gradExp);
    }
    bool inRegion = true;
    if (F.cx0 != 0 || F.cy0 != 0 || F.cx1 != F.slotsW || F.cy1 != F.slotsH) {
        int sx = i % F.slotsW, sy = i / F.slotsW;
        inRegion = sx >= F.cx0 && sx < F.cx1 && sy >= F.cy0 && sy < F.cy1;
    }
    if (p.x >= 0.0f && inRegion) {
        float b1 = F.beta1, b2 = F.beta2, eps = F.eps;
        // A slot with a zero gradient and zero moments: the update keeps the
        // moments at +0 and subtracts +0 from p (+0 / bc1 = +0, sqrtf(+0) + eps
        // = eps, lr * +0 / eps = +0, p - +0 = p for every p), so only the clamp
        // acts. Exact for lr, bc1, bc2, eps > 0 and finite beta1, beta2
        // (checked); the slots far from every target take this path.
        bool idle = (__float_as_uint(grx) | __float_as_uint(gry) | __float_as_uint(m.x) | __float_as_uint(m.y) |
                     __float_as_uint(v.x) | __float_as_uint(v.y)) == 0u &&
                    lr > 0.0f && lr < FLT_MAX && bc1 > 0.0f && bc2 > 0.0f && eps > 0.0f && fabsf(b1) < FLT_MAX &&
                    fabsf(b2) < FLT_MAX;
        if (idle) {
            float2 q = make_float2(fminf(fmaxf(p.x, 0.0f), F.width), fminf(fmaxf(p.y, 0.0f), F.height));
            if (__float_as_uint(q.x) != __float_as_uint(p.x) || __float_as_uint(q.y) != __float_as_uint(p.y))
                F.gen[i] = q;
            p = q;
        } else {
            float mx = b1 * m.x + (1.0f - b1) * grx;
            float my = b1 * m.y + (1.0f - b1) * gry;
            float vx = b2 * v.x + (1.0f - b2) * (grx * grx);
            float vy = b2 * v.y + (1.0f - b2) * (gry * gry);
            F.m[i] = make_float2(mx, my);
            F.v[i] = make_float2(vx, vy);
            p.x -= lr * (mx / bc1) / (sqrtf(vx / bc2) + eps);
            p.y -= lr * (my / bc1) / (sqrtf(vy / bc2) + eps);
            p.x = fminf(fmaxf(p.x, 0.0f), F.width);
            p.y = fminf(fmaxf(p.y, 0.0f), F.height);
            F.gen[i] = p;
        }
    }
    return p;
}

} // namespace vmk
