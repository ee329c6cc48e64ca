// Plain-old-data descriptors shared by the host runtime and the kernels.
//
// A "fit" is one VoroMesh optimisation problem (one reference VoroOptimizer).
// Kernels are batch-native: every launch walks a table of VmFit descriptors
// and a prefix table that maps its blocks to fits, so one fit and a batch of
// hundreds of uneven fits run through the same code and the same launches.
#pragma once

#include <cstdint>

#ifndef __CUDACC__
struct vm_float2_pod {
    float x, y;
};
#define VM_F2 vm_float2_pod
#else
#include <cuda_runtime.h>
#define VM_F2 float2
#endif

// Per-fit device state (one 128-byte block per fit).
struct VmState {
    int iter;        // Adam step count; 1-based once a step has run (IterState::iter)
    int count;       // targets used by the last loss pass (IterState::count)
    float loss;      // their summed VoroLoss (IterState::loss)
    int fallbacks;   // targets resolved by the exact ring search in the last pass
    unsigned long long accLo, accHi; // 128-bit fixed-point loss accumulator of the running pass
    int accCount;    // used-target counter of the running pass
    int slowTotal;   // targets that needed the exact ring search (cumulative)
    int errors;      // error bits raised by kernels (see VM_KERR_*)
    float schedLr, schedBc1, schedBc2; // this step's learning rate and bias corrections
    int needExact;   // this pass's fast-path gradient bound failed: the whole gradient is redone exactly
    int dUsed;       // this pass added to the exact split words (gradX sections DL, DH)
    int pad[14];
};

enum : int {
    VM_KERR_CAPACITY = 2, // the deferred-target queue was full (it holds every live target, so never in practice)
};

struct VmFit {
    // ---- geometry ----
    int nSlots, slotsW, slotsH;
    int gridW, gridH;
    float cell, inv; // hash-grid cell (the reference's spacing) and 1.0f / cell
    float width, height;
    int K;           // kNN size of the loss
    // ---- schedule (RunParams, reference voro_optimizer.cu:88-95) ----
    float lr, gamma, beta1, beta2, eps;
    int milestones[4];
    int cx0, cy0, cx1, cy1;
    float bx0, by0, bx1, by1;
    float fraction;
    unsigned seed;
    int gradExp, lossExp; // fixed-point exponents
    int nTargets;         // live targets in tpos/tslot (cell-sorted)
    int active;           // 1: stepped by this launch
    int fastShift;        // a gradient term of 2^(fastShift + 24) or more flags the fit (see vm_fast_shift)
    // ---- device arrays ----
    VM_F2 *gen, *m, *v;   // slot order
    long long *gradX;     // kGradWords per slot in three sections of 2 per slot: L, DL, DH
    int *key, *rank;      // per slot: grid cell (-1 empty) and rank within the cell
    int *counts;          // gridW*gridH (+1): per-cell counts, zero between builds
    int *start;           // gridW*gridH + 1: cell start in the sorted arrays
    unsigned long long *tileState; // the site grid's scan words (VmPointSet::tileState)
    int *sortedIdx;       // live slots in cell order, ascending slot within a cell
    VM_F2 *sortedPos;
    VM_F2 *tpos;          // live targets in cell order
    int *tslot;           // their target slot index (subsampling RNG key)
    VmState *state;
    // optional per-target diagnostics (nullptr unless requested)
    int *dbgI0, *dbgJ;
    float *dbgLoss;
    // The loss pass's windows (a warp's iteration): nullptr for runs of 32 in
    // target order; else nWindows cell-aligned runs of at most 32 targets,
    // twin[w] the start of window w and twin[nWindows] = nTargets.
    const int *twin;
    int nWindows;
};

// A set of points to bin into a fit's hash grid (sites or targets).
struct VmPointSet {
    const VM_F2 *pts;
    int n;
    int gridW, gridH;
    float inv;
    int *key, *rank, *counts, *start, *tileSums;
    VM_F2 *outPos;
    int *outIdx;
    int canonical; // sort each cell's run by index after the scatter
    int useIndexOrder; // outIdx holds the source index (always 1 today)
    int sub;           // log2 of the sub-cells per cell side in the sort key (targets; 0 for sites)
    // The scan of vm_launch_scan: one word per scan tile (its sum, then its
    // prefix) and a done counter after them, zero between scans. tileSums
    // serves the allocation-free build's scan only.
    unsigned long long *tileState;
};

constexpr int kScanTile = 2048; // cells per scan tile (256 threads x 8)
constexpr int kGradWords = 6;   // 64-bit words of exact gradient sums per slot (three sections of (x, y))
