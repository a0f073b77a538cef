// colo_emu.h -- host execution model for compiling the reference's CUDA
// sources with g++ (TEST INFRASTRUCTURE: golden-vector generation only).
//
// The reference (Codes/*.cu, *.h, *.cpp) is compiled unmodified except for
// its kernel-launch statements, which build_ref.py rewrites in memory into
// colo_emu_launch(...) calls.  Device memory is host memory; kernels run
// block by block; threads of a block run as user-level fibers so that
// __syncthreads is a real barrier.  Golden fixtures use integer coordinates,
// so every squared distance is exact and no rounding question arises.
#pragma once
#include <ucontext.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <numeric>
#include <vector>
// every standard header the reference includes, before the harness opens the
// reference's class for inspection
#include <ctime>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <iterator>
#include <limits>
#include <math.h>
#include <sstream>
#include <stdio.h>
#include <stdlib.h>
#include <string>
#include <type_traits>
#ifdef COLO_EMU_OPEN_CLASSES
#define private public
#endif

#define __global__
#define __device__
#define __host__
#define __constant__
#define __shared__ static
#define __forceinline__ inline
#define __inline__ inline
#define __launch_bounds__(...)

typedef int cudaError_t;
enum {
    cudaSuccess = 0,
    cudaErrorInvalidValue = 1,
    cudaErrorMemoryAllocation = 2,
};
enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3,
    cudaMemcpyDefault = 4
};
typedef void* cudaStream_t;
typedef struct colo_emu_event* cudaEvent_t;

struct uint3 {
    unsigned int x, y, z;
};
struct dim3 {
    unsigned int x, y, z;
    dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};
struct cudaDeviceProp {
    char name[256];
    int major, minor;
    size_t totalGlobalMem;
    int multiProcessorCount;
};

extern uint3 threadIdx, blockIdx;
extern dim3 blockDim, gridDim;

const float DEG_TO_RAD = 0.017453292519943295f;
const float EARTH_RADIUS_IN_METERS = 6372797.560856f;

// ---- device functions -----------------------------------------------------
// pow(float, int) is left to the host library: C++ promotes it to double, as
// the device does, so the reference's squared distance is formed in double
// and rounded to float once on both.
inline unsigned int atomicInc(unsigned int* a, unsigned int v) {
    unsigned int old = *a;
    *a = (old >= v) ? 0u : old + 1u;
    return old;
}
template <class T, class U>
inline T atomicAdd(T* a, U v) {
    T old = *a;
    *a = (T)(old + (T)v);
    return old;
}
template <class T, class U>
inline T atomicOr(T* a, U v) {
    T old = *a;
    *a = (T)(old | (T)v);
    return old;
}
void __syncthreads();

// ---- runtime API ------------------------------------------------------------
cudaError_t cudaMalloc(void** p, size_t n);
template <class T>
inline cudaError_t cudaMalloc(T** p, size_t n) {
    return cudaMalloc((void**)p, n);
}
cudaError_t cudaFree(void* p);
cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind k);
cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind k, cudaStream_t st = 0);
cudaError_t cudaMemset(void* d, int v, size_t n);
template <class T>
inline cudaError_t cudaMemcpyToSymbol(T& sym, const void* src, size_t n, size_t off = 0,
                                      cudaMemcpyKind = cudaMemcpyHostToDevice) {
    std::memcpy((char*)&sym + off, src, n);
    return cudaSuccess;
}
cudaError_t cudaEventCreate(cudaEvent_t* e);
cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t s = 0);
cudaError_t cudaEventSynchronize(cudaEvent_t e);
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t a, cudaEvent_t b);
cudaError_t cudaDeviceSynchronize();
cudaError_t cudaStreamSynchronize(cudaStream_t s);
cudaError_t cudaGetLastError();
const char* cudaGetErrorString(cudaError_t e);
cudaError_t cudaDeviceReset();
cudaError_t cudaGetDeviceCount(int* n);
cudaError_t cudaGetDeviceProperties(cudaDeviceProp* p, int dev);
cudaError_t cudaSetDevice(int dev);

// Kernel launch: every thread of every block runs `body` with threadIdx /
// blockIdx set.  `barriers` selects fiber execution for kernels that call
// __syncthreads; the others run thread after thread.
void colo_emu_launch(const char* name, dim3 grid, dim3 block, bool barriers, const std::function<void()>& body);

// Hooks the harness installs (called by the rewritten launches / Thrust).
extern void (*colo_emu_hook_threshold)(const unsigned int* countMap, unsigned int degree, unsigned int colocNum);
extern void (*colo_emu_hook_reduce)(size_t count, unsigned long long sum);
