/*
 * cuda_runtime.h -- CPU emulation of the CUDA C++ subset that the
 * reference's pyramid and colour-conversion kernels use
 * (source/CudaAccel/CudaPyramid2.cu, CudaUtil.cuh, ImageProc.cu), so that
 * their unchanged source compiles with g++ and runs on host cores.
 *
 * TEST INFRASTRUCTURE ONLY: this header is part of the recipe that builds
 * the reference's own code into oracle/_ref/ as the checker's pin.  It is
 * written for this project; it is not NVIDIA's header and does not include
 * it.
 *
 * Semantics emulated:
 *   - __global__, __device__ and __host__ are empty, __forceinline__ is
 *     `inline`;
 *   - __shared__ is a block-scope `static thread_local`: the threads of one
 *     block run as fibers on one host thread and so share it, as a CTA
 *     shares its shared memory; blocks of one launch run on several host
 *     threads, each with its own copy;
 *   - threadIdx / blockIdx / blockDim / gridDim are host-thread-local and
 *     are set by the scheduler before each fiber resumes;
 *   - __syncthreads() suspends the calling fiber until every thread of its
 *     block has reached the barrier or returned;
 *   - a launch `k<<<grid, block[, smem[, stream]]>>>(args);` is rewritten
 *     by the build recipe (a sed pass over the source, piped into g++) into
 *     `::psemu::launch(grid, block[, smem[, stream]], [&]() { k(args); });`.
 *     Launches run synchronously; streams are ignored.
 *   - vector types have CUDA's sizes and alignments; members that a kernel
 *     leaves unset stay indeterminate, as on the device (the recipe builds
 *     with -ftrivial-auto-var-init=zero so that they read as 0).
 */
#ifndef PSEMU_CUDA_RUNTIME_H
#define PSEMU_CUDA_RUNTIME_H

#include <cfenv>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <type_traits>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__ static thread_local
#define __align__(n) __attribute__((aligned(n)))

struct uint3 { unsigned int x, y, z; };
struct dim3 {
    unsigned int x, y, z;
    constexpr dim3(unsigned int vx = 1, unsigned int vy = 1, unsigned int vz = 1) : x(vx), y(vy), z(vz) {}
};

#define PSEMU_VEC2(T, N, A) struct __align__(A) N { T x, y; };
#define PSEMU_VEC3(T, N) struct N { T x, y, z; };
#define PSEMU_VEC4(T, N, A) struct __align__(A) N { T x, y, z, w; };
PSEMU_VEC2(unsigned char, uchar2, 2)
PSEMU_VEC2(short, short2, 4)
PSEMU_VEC2(unsigned short, ushort2, 4)
PSEMU_VEC2(int, int2, 8)
PSEMU_VEC2(float, float2, 8)
PSEMU_VEC3(unsigned char, uchar3)
PSEMU_VEC3(short, short3)
PSEMU_VEC3(int, int3)
PSEMU_VEC3(float, float3)
PSEMU_VEC4(unsigned char, uchar4, 4)
PSEMU_VEC4(signed char, char4, 4)
PSEMU_VEC4(short, short4, 8)
PSEMU_VEC4(unsigned short, ushort4, 8)
PSEMU_VEC4(int, int4, 16)
PSEMU_VEC4(float, float4, 16)
#undef PSEMU_VEC2
#undef PSEMU_VEC3
#undef PSEMU_VEC4

inline uchar4 make_uchar4(unsigned char x, unsigned char y, unsigned char z, unsigned char w) { return {x, y, z, w}; }
inline short4 make_short4(short x, short y, short z, short w) { return {x, y, z, w}; }
inline int4 make_int4(int x, int y, int z, int w) { return {x, y, z, w}; }
inline float4 make_float4(float x, float y, float z, float w) { return {x, y, z, w}; }
inline short2 make_short2(short x, short y) { return {x, y}; }
inline int2 make_int2(int x, int y) { return {x, y}; }
inline float2 make_float2(float x, float y) { return {x, y}; }
inline uchar3 make_uchar3(unsigned char x, unsigned char y, unsigned char z) { return {x, y, z}; }
inline int3 make_int3(int x, int y, int z) { return {x, y, z}; }
inline float3 make_float3(float x, float y, float z) { return {x, y, z}; }

/* CUDA's global integer and floating min / max overloads. */
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline unsigned int max(unsigned int a, unsigned int b) { return a > b ? a : b; }
inline unsigned int min(unsigned int a, unsigned int b) { return a < b ? a : b; }
inline float max(float a, float b) { return std::fmax(a, b); }
inline float min(float a, float b) { return std::fmin(a, b); }
inline double max(double a, double b) { return std::fmax(a, b); }
inline double min(double a, double b) { return std::fmin(a, b); }

extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

void __syncthreads();

/* fma rounded toward zero: the exact product-sum, then one rounding in that
   mode (the C library's fmaf honours the current rounding mode). */
inline float __fmaf_rz(float a, float b, float c)
{
    const int mode = std::fegetround();
    std::fesetround(FE_TOWARDZERO);
    volatile float r = std::fmaf(a, b, c);
    std::fesetround(mode);
    return r;
}

typedef struct psemu_stream* cudaStream_t;
typedef enum cudaError { cudaSuccess = 0, cudaErrorUnknown = 999 } cudaError_t;
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
inline const char* cudaGetErrorString(cudaError_t) { return "psemu"; }

namespace psemu {

/* Runs body(ctx) once per thread of every block of the grid. */
void run_grid(dim3 grid, dim3 block, void (*body)(void*), void* ctx);

template <class F>
void trampoline(void* f) { (*static_cast<F*>(f))(); }

template <class F>
void launch(dim3 grid, dim3 block, F&& f)
{
    using Fn = typename std::remove_reference<F>::type;
    run_grid(grid, block, &trampoline<Fn>, (void*)&f);
}

template <class F>
void launch(dim3 grid, dim3 block, size_t, F&& f) { launch(grid, block, static_cast<F&&>(f)); }

template <class F>
void launch(dim3 grid, dim3 block, size_t, cudaStream_t, F&& f) { launch(grid, block, static_cast<F&&>(f)); }

}  // namespace psemu

#endif
