/*
 * cuda_emu.h -- serial host emulation of the handful of CUDA constructs that
 * the reference kernels (LB_kernel.cu, sem_kernel.cu) use, so that their own
 * source compiles with g++ and runs on the CPU.
 *
 * ORACLE TEST INFRASTRUCTURE ONLY.  This header and the harness built on it
 * exist to generate golden vectors from the reference implementation in the
 * development container (the only place its sources are present).  Nothing in
 * the product links it.
 *
 * Execution model: every launch runs its blocks in ascending linear order and
 * the threads of a block one after another (threadIdx.x fastest).  That is one
 * legal schedule of the GPU program: atomics then land in thread order, CAS
 * slot claims are won by the lowest thread id, and __syncthreads() is a no-op
 * (the only kernel that calls it, sem_Force_kernel, reads nothing after the
 * barrier that another thread writes before it).
 */
#ifndef PF_CUDA_EMU_H
#define PF_CUDA_EMU_H

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <math.h>
#include <stdlib.h>

/* CUDA's device abs() has double overloads; bring the C++ ones in. */
using std::abs;

#define __global__
#define __device__
#define __host__
#define __constant__
#define __forceinline__ inline
#define __shared__ static

struct dim3 {
  unsigned x, y, z;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};

extern dim3 threadIdx, blockIdx, blockDim, gridDim;

static inline void __syncthreads() {}

struct cudaPitchedPtr {
  void *ptr;
  size_t pitch;
  size_t xsize;
  size_t ysize;
};
struct cudaExtent {
  size_t width, height, depth;
};
static inline cudaExtent make_cudaExtent(size_t w, size_t h, size_t d) {
  cudaExtent e;
  e.width = w;
  e.height = h;
  e.depth = d;
  return e;
}
static inline cudaPitchedPtr make_cudaPitchedPtr(void *p, size_t pitch, size_t xs, size_t ys) {
  cudaPitchedPtr r;
  r.ptr = p;
  r.pitch = pitch;
  r.xsize = xs;
  r.ysize = ys;
  return r;
}

/* Integer atomics.  One address can be put in "deferred" mode: adds to it are
 * collected in a shadow counter and applied after the launch.  That models the
 * schedule in which every thread of a launch performs its plain reads before
 * any thread's atomicAdd to that address lands. */
extern int *g_emu_deferred_addr;
extern long long g_emu_deferred_sum;

static inline int atomicAdd(int *a, int v) {
  if (a == g_emu_deferred_addr) {
    g_emu_deferred_sum += v;
    return *a;
  }
  int old = *a;
  *a = old + v;
  return old;
}
static inline unsigned atomicAdd(unsigned *a, unsigned v) {
  unsigned old = *a;
  *a = old + v;
  return old;
}
static inline float atomicAdd(float *a, float v) {
  float old = *a;
  *a = old + v;
  return old;
}
static inline int atomicCAS(int *a, int cmp, int val) {
  int old = *a;
  if (old == cmp) *a = val;
  return old;
}
static inline unsigned long long atomicCAS(unsigned long long *a, unsigned long long cmp,
                                           unsigned long long val) {
  unsigned long long old = *a;
  if (old == cmp) *a = val;
  return old;
}
static inline long long __double_as_longlong(double d) {
  long long l;
  std::memcpy(&l, &d, sizeof l);
  return l;
}
static inline double __longlong_as_double(long long l) {
  double d;
  std::memcpy(&d, &l, sizeof d);
  return d;
}

#endif
