/*
 * ref_shim.h — lets the reference's CUDA C and OpenCL C kernel SOURCE STRINGS
 * (extracted at build time into oracle/_ref/, never committed) compile as
 * plain C for the CPU. Test infrastructure only.
 *
 * CUDA: __global__/__device__ vanish; blockIdx/threadIdx/blockDim/gridDim are
 * thread-local variables that the launch loops in ref_driver.c set; the
 * float atomicAdd becomes an OpenMP atomic update.
 * OpenCL: __kernel/__global vanish; get_global_id/get_global_size read
 * thread-local arrays; atomic_add becomes a relaxed atomic add; exp() on a
 * float is the binary32 expf (OpenCL's float overload).
 */
#ifndef REF_SHIM_H
#define REF_SHIM_H

#include <math.h>
#include <stdint.h>

typedef struct {
  unsigned int x, y, z;
} ref_dim3;

extern __thread ref_dim3 blockIdx, threadIdx, blockDim, gridDim;
extern __thread size_t ref_gid[3], ref_gsize[3];

#define __global__
#define __device__
#define __kernel
#define __global
typedef unsigned char uchar;

static inline size_t get_global_id(int d) { return ref_gid[d]; }
static inline size_t get_global_size(int d) { return ref_gsize[d]; }

static inline float atomicAdd(float* p, float v) {
  float old;
#pragma omp atomic capture
  {
    old = *p;
    *p += v;
  }
  return old;
}

static inline int atomic_add(volatile int* p, int v) { return __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }

/* reference kernels call exp() on binary32 values */
#define exp(x) expf(x)

#endif
