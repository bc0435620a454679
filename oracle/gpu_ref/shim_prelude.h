/*
 * shim_prelude.h -- project-written shim that lets the reference's CUDA
 * kernel headers (gpu/src/cuda/integration_kernel.cuh, solver_kernel.cuh)
 * compile as plain host C++ (test infrastructure, oracle/_ref only).
 *
 * CUDA qualifiers become empty, the removed texture-reference API becomes a
 * pointer wrapper, thread indices become globals set by the driver (which
 * runs every kernel as one-thread blocks, sequentially -- the kernels'
 * results do not depend on the block size), and the few device intrinsics
 * the headers use get host definitions.  Force-included before the
 * reference headers.
 */
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#undef __global__
#undef __constant__
#undef __shared__
#undef __device__
#undef __host__
#define __global__
#define __constant__
#define __shared__
#define __device__
#define __host__

extern dim3 blockIdx, blockDim, threadIdx;

inline unsigned __umul24(unsigned a, unsigned b) { return a * b; }
inline int __mul24(int a, int b) { return a * b; }

template <class T, int D, int M>
struct texture {
    const T *ptr = nullptr;
};
template <class T, int D, int M>
inline T tex1Dfetch(const texture<T, D, M> &t, int i) { return t.ptr[i]; }

inline float min(float a, float b) { return a < b ? a : b; }
inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
inline float max(float a, float b) { return a > b ? a : b; }
inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }
inline void __syncthreads() {}
template <class T>
inline T atomicAdd(T *a, T v) {
    T o = *a;
    *a += v;
    return o;
}
