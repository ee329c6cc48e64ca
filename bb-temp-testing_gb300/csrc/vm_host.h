// Host-side helpers shared by the runtime translation units (internal).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "vm_capi.h"
#include "vm_types.h"

namespace vmh {

constexpr int kMaxCellVerts = 24;

// NVTX range over a public entry point (visible in Nsight timelines; no cost
// without a profiler attached).
struct NvtxRange {
    explicit NvtxRange(const char *name);
    ~NvtxRange();
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
int floor_log2f(float h);

// Owning device buffer. alloc() replaces the contents; reserve() keeps the
// buffer when it is already large enough.
template <class T> struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    int alloc(size_t count)
    {
        release();
        if (count == 0) return VM_OK;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e) {
            p = nullptr;
            return cuda_fail(e, "cudaMalloc");
        }
        n = count;
        return VM_OK;
    }
    int reserve(size_t count) { return count <= n && p ? VM_OK : alloc(count); }
};

// The tile words of a scan over `tiles` tiles (vm_launch_scan): allocated and
// zeroed when too small, kept otherwise (every scan leaves all of them zero).
inline int zeroed_tile_state(DevBuf<unsigned long long> &b, int tiles, cudaStream_t s)
{
    size_t need = (size_t)tiles + 1;
    if (b.p && b.n >= need) return VM_OK;
    int rc = b.alloc(need);
    if (rc) return rc;
    cudaError_t e = cudaMemsetAsync(b.p, 0, need * sizeof(unsigned long long), s);
    return e ? cuda_fail(e, "scan tile words") : VM_OK;
}

// The host part of the last Extract: the boundary (vertices, edges) and the
// summary; the cells themselves stay on the device until copied out.
struct MeshHost {
    int numGenerators = 0, numCellVerts = 0;
    std::vector<float2> vertices;
    std::vector<int> edges; // pairs
    bool watertight = false;
    int loops = 0, unsafeCells = 0, overflowCells = 0;
    float gpuMs = 0.0f, hostMs = 0.0f;
};

// Watertightness and loops of the boundary from mesh.edges / mesh.vertices
// (the edges and vertices themselves are assembled on the device).
void boundary_topology(MeshHost &mesh);

// Device view of a canvas for the optimiser hand-off (vm_canvas.cu): its
// target slots and occupancy, and the last edit's dirty slots, their values
// and tile rectangle. Valid until the next canvas call.
struct CanvasView {
    const float2 *slots;
    int nslots;
    const unsigned long long *inside;
    int tilesX, tilesY;
    float voxelSize;
    const int *dirty;
    const float2 *dirtyValues;
    int ndirty;
    int tx0, ty0, tx1, ty1;
    cudaStream_t stream;
};
int canvas_view(cv_canvas *c, CanvasView *v);
// p[0..n) = {-1, -1} (empty slots)
cudaError_t canvas_fill_empty(float2 *p, size_t n, cudaStream_t s);
// dst[rect] = src[rect] for tile words of row pitch `pitch`
cudaError_t canvas_copy_rect(const unsigned long long *src, unsigned long long *dst, int pitch, int tx0, int ty0,
                             int tx1, int ty1, cudaStream_t s);

} // namespace vmh
