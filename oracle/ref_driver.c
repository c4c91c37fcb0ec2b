/*
 * ref_driver.c — CPU launch loops for the reference's own kernels, whose
 * source strings ref_extract.py writes to oracle/_ref/ref_sources.inc at build
 * time (never committed). Test infrastructure and CPU baseline only.
 *
 * A CUDA launch <<<grid, block>>> becomes nested loops over blocks and threads
 * (blocks spread over OpenMP threads); an OpenCL NDRange becomes loops over
 * global ids. Kernels are called exactly as the reference launches them:
 *   walkers   pycuda_small.py:96-106, pycuda_small_allx.py:163-173,
 *             pycuda_large_allx.py:393-400,
 *             pyopencl_small.py:124-132
 *   smoothing rw_small.py:104-125 (curvature then update, block (32,32,1))
 *   top-3 / uncertainty rw_small.py:155-161.
 */
#include <stddef.h>
#include <stdint.h>

#include "ref_shim.h"

__thread ref_dim3 blockIdx, threadIdx, blockDim, gridDim;
__thread size_t ref_gid[3], ref_gsize[3];

#include "_ref/ref_sources.inc"

typedef void (*cuda_walk_fn)(int, float*, int*, float*, int, int, int, int*, int, int);
typedef void (*cuda_walk_allx_fn)(int, int, float*, int*, float*, int, int, int, int*, int, float*, int);
typedef void (*post_fn)(float*, float*, int, int);

#define CUDA_LAUNCH_BEGIN(GX, GY, GZ)                                \
  _Pragma("omp parallel for collapse(2) schedule(dynamic, 1)")       \
  for (int bz = 0; bz < (GZ); ++bz)                                  \
    for (int by = 0; by < (GY); ++by) {                              \
      gridDim.x = (GX); gridDim.y = (GY); gridDim.z = (GZ);          \
      blockDim.x = 32; blockDim.y = 32; blockDim.z = 1;              \
      blockIdx.y = by; blockIdx.z = bz;                              \
      for (int bx = 0; bx < (GX); ++bx) {                            \
        blockIdx.x = bx;                                             \
        for (int ty = 0; ty < 32; ++ty)                              \
          for (int tx = 0; tx < 32; ++tx) {                          \
            threadIdx.x = tx; threadIdx.y = ty; threadIdx.z = 0;
#define CUDA_LAUNCH_END }}}

/* Launchers take the grid the reference passes (block is always (32,32,1)). */

/* pycuda_small walker. variant 0: int8 image, 1: float32 image. */
int ref_launch_walk(int variant, int gx, int gy, int gz, int segment, void* raw, int* slices, float* a, int xsh,
                    int ysh, int zsh, int* indices, int sorw, int nbrw) {
  cuda_walk_fn k = variant == 0 ? ref_cuda_walk_i8 : ref_cuda_walk_f32;
  CUDA_LAUNCH_BEGIN(gx, gy, gz)
  k(segment, (float*)raw, slices, a, xsh, ysh, zsh, indices, sorw, nbrw);
  CUDA_LAUNCH_END
  return 0;
}

/* pycuda_large walker (adaptive seeds), launched like the small one
 * (pycuda_large.py:404-407: block (32, 32, 1), grid (xsh/32+1, ysh/32+1, slices)). */
int ref_launch_walk_large(int variant, int gx, int gy, int gz, int segment, void* raw, int* slices, float* a,
                          int xsh, int ysh, int zsh, int* indices, int sorw, int nbrw) {
  cuda_walk_fn k = variant == 0 ? ref_cuda_walk_large_i8 : ref_cuda_walk_large_f32;
  CUDA_LAUNCH_BEGIN(gx, gy, gz)
  k(segment, (float*)raw, slices, a, xsh, ysh, zsh, indices, sorw, nbrw);
  CUDA_LAUNCH_END
  return 0;
}

/* pycuda_small_allx walker (one axis per launch). */
int ref_launch_walk_allx(int variant, int gx, int gy, int gz, int axis, int segment, void* raw, int* slices,
                         float* a, int xsh, int ysh, int zsh, int* indices, int sorw, float* beta, int nbrw) {
  cuda_walk_allx_fn k = variant == 0 ? ref_cuda_walk_allx_i8 : ref_cuda_walk_allx_f32;
  CUDA_LAUNCH_BEGIN(gx, gy, gz)
  k(axis, segment, (float*)raw, slices, a, xsh, ysh, zsh, indices, sorw, beta, nbrw);
  CUDA_LAUNCH_END
  return 0;
}

/* pycuda_large_allx walker (adaptive seeds in slice coordinates), one axis per
 * launch (pycuda_large_allx.py:393-400: block (32, 32, 1), grid (cols/32+1,
 * rows/32+1, slices of the axis)). */
int ref_launch_walk_large_allx(int variant, int gx, int gy, int gz, int axis, int segment, void* raw, int* slices,
                               float* a, int xsh, int ysh, int zsh, int* indices, int sorw, float* beta, int nbrw) {
  cuda_walk_allx_fn k = variant == 0 ? ref_cuda_walk_large_allx_i8 : ref_cuda_walk_large_allx_f32;
  CUDA_LAUNCH_BEGIN(gx, gy, gz)
  k(axis, segment, (float*)raw, slices, a, xsh, ysh, zsh, indices, sorw, beta, nbrw);
  CUDA_LAUNCH_END
  return 0;
}

/* Post kernels of gpu_kernels.py. kind 0: curvature(phi, curv),
 * 1: update(phi, curv), 2: max(max3, a), 3: uncertainty(max3, a). */
int ref_launch_post(int kind, int gx, int gy, int gz, float* p0, float* p1, int xsh, int ysh) {
  post_fn k = kind == 0 ? ref_curvature : kind == 1 ? ref_update : kind == 2 ? ref_max : ref_uncertainty;
  CUDA_LAUNCH_BEGIN(gx, gy, gz)
  k(p0, p1, xsh, ysh);
  CUDA_LAUNCH_END
  return 0;
}

/* pyopencl_small randomWalk over the NDRange (g0, g1, g2) = (zsh, ysh, xsh).
 * variant 0: char image, 1: float image; labels are uchar. */
int ref_ocl_walk(int variant, int g0, int g1, int g2, int segment, void* raw, uchar* slices, int* a, int xsh,
                 int ysh, int zsh, int sorw, int nbrw) {
#pragma omp parallel for collapse(2) schedule(dynamic, 1)
  for (int i0 = 0; i0 < g0; ++i0)
    for (int i1 = 0; i1 < g1; ++i1) {
      ref_gsize[0] = g0;
      ref_gsize[1] = g1;
      ref_gsize[2] = g2;
      ref_gid[0] = i0;
      ref_gid[1] = i1;
      for (int i2 = 0; i2 < g2; ++i2) {
        ref_gid[2] = i2;
        if (variant == 0)
          ref_ocl_walk_char(segment, (char*)raw, slices, a, xsh, ysh, zsh, sorw, nbrw);
        else
          ref_ocl_walk_float(segment, (float*)raw, slices, a, xsh, ysh, zsh, sorw, nbrw);
      }
    }
  return 0;
}

/* Same as ref_ocl_walk but visits only the listed first-dimension ids (the
 * planes that carry labels); work-items on other planes return immediately in
 * the reference kernel, so the hit maps are identical. Used to time bounded
 * samples of the reference CPU path. */
int ref_ocl_walk_planes(int variant, const int* planes, int nplanes, int g0, int g1, int g2, int segment, void* raw,
                        uchar* slices, int* a, int xsh, int ysh, int zsh, int sorw, int nbrw) {
#pragma omp parallel for collapse(3) schedule(dynamic, 32)
  for (int p = 0; p < nplanes; ++p)
    for (int i1 = 0; i1 < g1; ++i1)
      for (int i2 = 0; i2 < g2; ++i2) {
        ref_gsize[0] = g0;
        ref_gsize[1] = g1;
        ref_gsize[2] = g2;
        ref_gid[0] = planes[p];
        ref_gid[1] = i1;
        ref_gid[2] = i2;
        if (variant == 0)
          ref_ocl_walk_char(segment, (char*)raw, slices, a, xsh, ysh, zsh, sorw, nbrw);
        else
          ref_ocl_walk_float(segment, (float*)raw, slices, a, xsh, ysh, zsh, sorw, nbrw);
      }
  return 0;
}
