// Prefix for compiling the reference's device code with a host C++ compiler.
//
// The reference's kernels (the anonymous-namespace sections of
// src/voromesh/voro_optimizer.cu and src/poisson/poisson_disk.cu) are plain
// scalar C++ apart from a few CUDA names. This prefix supplies host stand-ins
// for exactly those names so that each __global__ function can be called as
// an ordinary function, one "thread" at a time, with blockDim = (1,1,1).
// Every thread is then lane 0 of its own warp: the reference's warp-shuffle
// reduction (voro_optimizer.cu:258-265) adds nothing and each thread's loss is
// added to the iteration state by itself, in thread-index order.
//
// Used only by oracle/ref_shim/build_ref.sh to produce oracle/_ref/.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __restrict__ __restrict

struct float2 { float x, y; };
struct double2 { double x, y; };
static inline float2 make_float2(float x, float y) { float2 r; r.x = x; r.y = y; return r; }
static inline double2 make_double2(double x, double y) { double2 r; r.x = x; r.y = y; return r; }

struct shim_uint3 { unsigned x, y, z; };
static shim_uint3 blockIdx = {0, 0, 0}, blockDim = {1, 1, 1}, threadIdx = {0, 0, 0};

static inline int min(int a, int b) { return a < b ? a : b; }
static inline int max(int a, int b) { return a > b ? a : b; }

static inline int atomicAdd(int *p, int v) { int o = *p; *p = o + v; return o; }
static inline float atomicAdd(float *p, float v) { float o = *p; *p = o + v; return o; }
template <typename T> static inline T __shfl_down_sync(unsigned, T, int) { return T(0); }

typedef int cudaError_t;
static const int cudaSuccess = 0;
static inline const char *cudaGetErrorString(int) { return "shim"; }
static inline int cudaFree(void *p) { std::free(p); return 0; }
template <typename T> static inline int cudaMalloc(T **p, size_t bytes) { *p = (T *)std::malloc(bytes); return 0; }
#define CUDA_CHECK(call) (void)(call)
