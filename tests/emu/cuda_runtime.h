// Host stand-in for <cuda_runtime.h> used by the SIMT emulation of the engine's kernels
// (tests only): the CUDA qualifiers become plain C++, __shared__ variables become statics
// shared by the host threads of one block, and __syncthreads is a barrier.  Only kernels
// that use block-level synchronisation (no warp intrinsics, no tensor-core PTX) run here.
#pragma once
#include <cmath>
#include <cstddef>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))
#define __launch_bounds__(...)
#define __shared__ static

struct double2 { double x, y; };
struct int2 { int x, y; };
struct uint3 { unsigned x, y, z; };
struct dim3 { unsigned x, y, z; };
inline double2 make_double2(double x, double y) { return double2{x, y}; }

#ifdef EMU_FIBERS
extern uint3 threadIdx;      // the threads of a CTA are fibers of one host thread
#else
extern thread_local uint3 threadIdx;
#endif
extern uint3 blockIdx;
extern dim3 blockDim, gridDim;
void emu_syncthreads();
#define __syncthreads() emu_syncthreads()
template <class T> inline T __ldg(const T* p) { return *p; }
template <class T> inline T __ldcg(const T* p) { return *(const volatile T*)p; }
// device-wide ordering and the counter of the spread passes' last-CTA reductions
inline void __threadfence() { __atomic_thread_fence(__ATOMIC_SEQ_CST); }
inline unsigned atomicAdd(unsigned* a, unsigned v) { return __atomic_fetch_add(a, v, __ATOMIC_SEQ_CST); }
// CUDA's integer min / max overloads
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline long long min(long long a, long long b) { return a < b ? a : b; }
inline long long max(long long a, long long b) { return a > b ? a : b; }
inline size_t min(size_t a, size_t b) { return a < b ? a : b; }
inline size_t max(size_t a, size_t b) { return a > b ? a : b; }
using std::fma;
using std::sqrt;
using std::fabs;
using std::fmax;
using std::isfinite;

// the host helpers of w90g.cuh reference these; the emulation never calls them
typedef int cudaError_t;
typedef void* cudaStream_t;
enum cudaMemcpyKind { cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
struct cudaPitchedPtr { void* ptr; size_t pitch, xsize, ysize; };
struct cudaExtent { size_t width, height, depth; };
struct cudaPos { size_t x, y, z; };
struct cudaArray;
struct cudaMemcpy3DParms {
  cudaArray* srcArray; cudaPos srcPos; cudaPitchedPtr srcPtr;
  cudaArray* dstArray; cudaPos dstPos; cudaPitchedPtr dstPtr;
  cudaExtent extent; cudaMemcpyKind kind;
};
inline cudaPitchedPtr make_cudaPitchedPtr(void* d, size_t p, size_t x, size_t y) { return {d, p, x, y}; }
inline cudaExtent make_cudaExtent(size_t w, size_t h, size_t d) { return {w, h, d}; }
inline cudaError_t cudaMemcpy3DAsync(const cudaMemcpy3DParms*, cudaStream_t) { return 1; }
