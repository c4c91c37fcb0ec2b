// Volume preparation kernels: label histogram, labelled-slice detection with
// bounding box, image min/max and the working-image builder.
//
// The zero pad of the reference (biomedisa/interpolation.py:157-158) is never
// materialised: kernels read the caller's unpadded volume and treat padded
// coordinates outside it as zero.
#include <cfloat>
#include <climits>

#include "si_common.cuh"
#include "si_internal.h"

namespace si {
namespace {

template <typename T>
__device__ __forceinline__ int load_label(const T* p, uint64_t i) {
  return static_cast<int>(p[i]);
}

// ---------------------------------------------------------------------------
// Histogram of label values. Zeros (the bulk of a sparse label volume) are
// counted in a register to avoid shared-atomic contention on one bin.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) label_hist_kernel(const T* __restrict__ lab, uint64_t n,
                                                         unsigned long long* __restrict__ hist) {
  __shared__ unsigned int sh[258];
  for (int i = threadIdx.x; i < 258; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  unsigned int zeros = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int v = load_label(lab, i);
    if (v == 0) {
      ++zeros;
    } else {
      const int b = v < 0 ? 256 : (v > 255 ? 257 : v);
      atomicAdd(&sh[b], 1u);
    }
  }
  zeros = __reduce_add_sync(0xffffffffu, zeros);
  if ((threadIdx.x & 31) == 0 && zeros) atomicAdd(&sh[0], zeros);
  __syncthreads();
  for (int i = threadIdx.x; i < 258; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], (unsigned long long)sh[i]);
}

// ---------------------------------------------------------------------------
// Labelled-slice flags and bounding box (padded coordinates).
// nz(v): value nonzero after pre-processing (negative -> nonzero, > 255 -> 0).
// All-axis test for a slice with in-slice rows r and columns c
// (biomedisa_helper.py:1047-1066): a nonzero pixel is dropped when both its
// row neighbours are zero; a remaining pixel is then dropped when both its
// column neighbours are dropped/zero; the slice counts if any pixel remains.
// Pixels outside the volume (the pad) are zero.
// ---------------------------------------------------------------------------
template <typename T>
struct LabelView {
  const T* lab;
  const uint8_t* nz_lut;  // shared-memory copy
  int Z0, Y0, X0;
  bool neg_nz;  // negative values count as nonzero (labels != 0) or as zero (labels > 0)
  // nonzero test at ORIGINAL coordinates, zero outside.
  __device__ __forceinline__ bool nz(int z, int y, int x) const {
    if ((unsigned)z >= (unsigned)Z0 || (unsigned)y >= (unsigned)Y0 || (unsigned)x >= (unsigned)X0) return false;
    const int v = load_label(lab, ((uint64_t)z * Y0 + y) * X0 + x);
    if (v < 0) return neg_nz;
    if (v > 255) return false;
    return nz_lut[v] != 0;
  }
};

// Row-direction survivor (rows along axis R, column index fixed).
template <typename V>
__device__ __forceinline__ bool ones1(const V& lv, int z, int y, int x, int rz, int ry, int rx) {
  if (!lv.nz(z, y, x)) return false;
  return lv.nz(z - rz, y - ry, x - rx) || lv.nz(z + rz, y + ry, x + rx);
}

template <typename V>
__device__ __forceinline__ bool survives(const V& lv, int z, int y, int x, int rz, int ry, int rx, int cz, int cy,
                                         int cx) {
  if (!ones1(lv, z, y, x, rz, ry, rx)) return false;
  return ones1(lv, z - cz, y - cy, x - cx, rz, ry, rx) || ones1(lv, z + cz, y + cy, x + cx, rz, ry, rx);
}

template <typename T>
__global__ void __launch_bounds__(256) slice_flags_kernel(const T* __restrict__ lab, int Z0, int Y0, int X0,
                                                          const uint8_t* __restrict__ nz_lut_g, int allaxis,
                                                          uint8_t* __restrict__ fz, uint8_t* __restrict__ fy,
                                                          uint8_t* __restrict__ fx, int32_t* __restrict__ bbox) {
  __shared__ uint8_t lut[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = nz_lut_g[i];
  __syncthreads();
  LabelView<T> lv{lab, lut, Z0, Y0, X0, allaxis != 2};
  int bmin[3] = {INT_MAX, INT_MAX, INT_MAX};
  int bmax[3] = {-1, -1, -1};
  const uint64_t n = (uint64_t)Z0 * Y0 * X0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int x = (int)(i % X0);
    const uint64_t zy = i / X0;
    const int y = (int)(zy % Y0);
    const int z = (int)(zy / Y0);
    if (!lv.nz(z, y, x)) continue;
    // padded coordinates
    const int pz = z + 1, py = y + 1, px = x + 1;
    bmin[0] = min(bmin[0], pz); bmax[0] = max(bmax[0], pz);
    bmin[1] = min(bmin[1], py); bmax[1] = max(bmax[1], py);
    bmin[2] = min(bmin[2], px); bmax[2] = max(bmax[2], px);
    if (!allaxis) {
      fz[pz] = 1;
    } else {
      // axis 0: slice at fixed z, rows along y, columns along x
      if (!fz[pz] && survives(lv, z, y, x, 0, 1, 0, 0, 0, 1)) fz[pz] = 1;
      // axis 1: slice at fixed y, rows along z, columns along x
      if (!fy[py] && survives(lv, z, y, x, 1, 0, 0, 0, 0, 1)) fy[py] = 1;
      // axis 2: slice at fixed x, rows along z, columns along y
      if (!fx[px] && survives(lv, z, y, x, 1, 0, 0, 0, 1, 0)) fx[px] = 1;
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int mn = __reduce_min_sync(0xffffffffu, bmin[a]);
    const int mx = __reduce_max_sync(0xffffffffu, bmax[a]);
    if ((threadIdx.x & 31) == 0) {
      if (mn != INT_MAX) atomicMin(&bbox[2 * a], mn);
      if (mx != -1) atomicMax(&bbox[2 * a + 1], mx);
    }
  }
}

// ---------------------------------------------------------------------------
// Image min/max after conversion to float32.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ float to_float(T v);
template <>
__device__ __forceinline__ float to_float<uint16_t>(uint16_t v) { return __uint2float_rn(v); }
template <>
__device__ __forceinline__ float to_float<int16_t>(int16_t v) { return __int2float_rn(v); }
template <>
__device__ __forceinline__ float to_float<int32_t>(int32_t v) { return __int2float_rn(v); }
template <>
__device__ __forceinline__ float to_float<float>(float v) { return v; }

__device__ __forceinline__ void atomic_min_float(float* addr, float v) {
  if (v >= 0.0f)
    atomicMin(reinterpret_cast<int*>(addr), __float_as_int(v));
  else
    atomicMax(reinterpret_cast<unsigned int*>(addr), __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_float(float* addr, float v) {
  if (v >= 0.0f)
    atomicMax(reinterpret_cast<int*>(addr), __float_as_int(v));
  else
    atomicMin(reinterpret_cast<unsigned int*>(addr), __float_as_uint(v));
}

template <typename T>
__global__ void __launch_bounds__(256) minmax_kernel(const T* __restrict__ img, uint64_t n, float* __restrict__ mm) {
  float lo = FLT_MAX, hi = -FLT_MAX;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float v = to_float<T>(img[i]);
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
  for (int o = 16; o; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_min_float(&mm[0], lo);
    atomic_max_float(&mm[1], hi);
  }
}

// ---------------------------------------------------------------------------
// Working image builder.
// ---------------------------------------------------------------------------
struct Crop {
  int Z0, Y0, X0;     // original dims
  int cz0, cy0, cx0;  // crop origin, padded frame
  int Zc, Yc, Xc;     // crop dims
};

// uint8 data domain (uint8 input, or int8 shifted by +128).
template <typename T>
__device__ __forceinline__ int u8_value(const T* img, uint64_t i);
template <>
__device__ __forceinline__ int u8_value<uint8_t>(const uint8_t* img, uint64_t i) { return img[i]; }
template <>
__device__ __forceinline__ int u8_value<int8_t>(const int8_t* img, uint64_t i) { return (int)img[i] + 128; }

template <typename T>
__global__ void __launch_bounds__(256) prepare_u8_kernel(const T* __restrict__ img, Crop cr, int denoise,
                                                         uint8_t* __restrict__ work) {
  const uint64_t n = (uint64_t)cr.Zc * cr.Yc * cr.Xc;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int xc = (int)(i % cr.Xc);
    const uint64_t zy = i / cr.Xc;
    const int yc = (int)(zy % cr.Yc);
    const int zc = (int)(zy / cr.Yc);
    const int z = zc + cr.cz0 - 1, y = yc + cr.cy0 - 1, x = xc + cr.cx0 - 1;
    int v = 0;
    if ((unsigned)z < (unsigned)cr.Z0 && (unsigned)y < (unsigned)cr.Y0 && (unsigned)x < (unsigned)cr.X0) {
      if (!denoise) {
        v = u8_value(img, ((uint64_t)z * cr.Y0 + y) * cr.X0 + x);
      } else {
        // box mean over in-bounds neighbours, truncated (numba float->uint8 cast)
        int sum = 0, cnt = 0;
        for (int k = -1; k <= 1; ++k)
          for (int l = -1; l <= 1; ++l)
            for (int m = -1; m <= 1; ++m) {
              const int zz = z + k, yy = y + l, xx = x + m;
              if ((unsigned)zz < (unsigned)cr.Z0 && (unsigned)yy < (unsigned)cr.Y0 && (unsigned)xx < (unsigned)cr.X0) {
                sum += u8_value(img, ((uint64_t)zz * cr.Y0 + yy) * cr.X0 + xx);
                ++cnt;
              }
            }
        v = sum / cnt;
      }
    }
    work[i] = (uint8_t)v;
  }
}

// float data domain: (x - mn) / range * 255 in binary32, as numpy does
// (biomedisa/interpolation.py:141-144).
template <typename T>
__device__ __forceinline__ float norm_value(const T* img, uint64_t i, float mn, float range) {
  const float v = to_float<T>(img[i]);
  return __fmul_rn(__fdiv_rn(__fsub_rn(v, mn), range), 255.0f);
}

template <typename T>
__global__ void __launch_bounds__(256) prepare_f32_kernel(const T* __restrict__ img, Crop cr, float mn, float range,
                                                          int denoise, float* __restrict__ work) {
  const uint64_t n = (uint64_t)cr.Zc * cr.Yc * cr.Xc;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int xc = (int)(i % cr.Xc);
    const uint64_t zy = i / cr.Xc;
    const int yc = (int)(zy % cr.Yc);
    const int zc = (int)(zy / cr.Yc);
    const int z = zc + cr.cz0 - 1, y = yc + cr.cy0 - 1, x = xc + cr.cx0 - 1;
    float v = 0.0f;
    if ((unsigned)z < (unsigned)cr.Z0 && (unsigned)y < (unsigned)cr.Y0 && (unsigned)x < (unsigned)cr.X0) {
      if (!denoise) {
        v = norm_value(img, ((uint64_t)z * cr.Y0 + y) * cr.X0 + x, mn, range);
      } else {
        // numba accumulates in float64 in (k, l, m) order, then divides
        double sum = 0.0;
        int cnt = 0;
        for (int k = -1; k <= 1; ++k)
          for (int l = -1; l <= 1; ++l)
            for (int m = -1; m <= 1; ++m) {
              const int zz = z + k, yy = y + l, xx = x + m;
              if ((unsigned)zz < (unsigned)cr.Z0 && (unsigned)yy < (unsigned)cr.Y0 && (unsigned)xx < (unsigned)cr.X0) {
                sum = __dadd_rn(sum, (double)norm_value(img, ((uint64_t)zz * cr.Y0 + yy) * cr.X0 + xx, mn, range));
                ++cnt;
              }
            }
        v = __double2float_rn(__ddiv_rn(sum, (double)cnt));
      }
    }
    work[i] = v;
  }
}

inline int grid_for(uint64_t n, int block) {
  const uint64_t want = (n + block - 1) / block;
  const uint64_t cap = (uint64_t)sm_count() * 16;
  return (int)(want < cap ? (want > 0 ? want : 1) : cap);
}

}  // namespace
}  // namespace si

using namespace si;

extern "C" int si_label_histogram(const void* labels, int dtype, uint64_t n, unsigned long long* hist, void* stream) {
  clear_error();
  if (!labels || !hist) return set_error(SI_ERR_ARG, "si_label_histogram: null pointer");
  if (n == 0) return SI_OK;
  const int block = 256, grid = grid_for(n, block);
  cudaStream_t st = as_stream(stream);
  switch (dtype) {
    case SI_U8:
      label_hist_kernel<<<grid, block, 0, st>>>(static_cast<const uint8_t*>(labels), n, hist);
      break;
    case SI_I16:
      label_hist_kernel<<<grid, block, 0, st>>>(static_cast<const int16_t*>(labels), n, hist);
      break;
    case SI_I32:
      label_hist_kernel<<<grid, block, 0, st>>>(static_cast<const int32_t*>(labels), n, hist);
      break;
    default:
      return set_error(SI_ERR_ARG, "si_label_histogram: unsupported label dtype %d", dtype);
  }
  return check_launch("si_label_histogram");
}

extern "C" int si_slice_flags(const void* labels, int dtype, int Z0, int Y0, int X0, const uint8_t* nz_lut,
                              int allaxis, uint8_t* flags_z, uint8_t* flags_y, uint8_t* flags_x, int32_t* bbox,
                              void* stream) {
  clear_error();
  if (!labels || !nz_lut || !flags_z || !bbox) return set_error(SI_ERR_ARG, "si_slice_flags: null pointer");
  if (allaxis < 0 || allaxis > 2) return set_error(SI_ERR_ARG, "si_slice_flags: allaxis must be 0, 1 or 2");
  if (allaxis && (!flags_y || !flags_x)) return set_error(SI_ERR_ARG, "si_slice_flags: allaxis needs flags_y/flags_x");
  if (Z0 <= 0 || Y0 <= 0 || X0 <= 0) return set_error(SI_ERR_ARG, "si_slice_flags: bad dims");
  const uint64_t n = (uint64_t)Z0 * Y0 * X0;
  const int block = 256, grid = grid_for(n, block);
  cudaStream_t st = as_stream(stream);
  switch (dtype) {
    case SI_U8:
      slice_flags_kernel<<<grid, block, 0, st>>>(static_cast<const uint8_t*>(labels), Z0, Y0, X0, nz_lut, allaxis,
                                                 flags_z, flags_y, flags_x, bbox);
      break;
    case SI_I16:
      slice_flags_kernel<<<grid, block, 0, st>>>(static_cast<const int16_t*>(labels), Z0, Y0, X0, nz_lut, allaxis,
                                                 flags_z, flags_y, flags_x, bbox);
      break;
    case SI_I32:
      slice_flags_kernel<<<grid, block, 0, st>>>(static_cast<const int32_t*>(labels), Z0, Y0, X0, nz_lut, allaxis,
                                                 flags_z, flags_y, flags_x, bbox);
      break;
    default:
      return set_error(SI_ERR_ARG, "si_slice_flags: unsupported label dtype %d", dtype);
  }
  return check_launch("si_slice_flags");
}

extern "C" int si_image_minmax(const void* img, int dtype, uint64_t n, float* mm, void* stream) {
  clear_error();
  if (!img || !mm) return set_error(SI_ERR_ARG, "si_image_minmax: null pointer");
  if (n == 0) return SI_OK;
  const int block = 256, grid = grid_for(n, block);
  cudaStream_t st = as_stream(stream);
  switch (dtype) {
    case SI_U16:
      minmax_kernel<<<grid, block, 0, st>>>(static_cast<const uint16_t*>(img), n, mm);
      break;
    case SI_I16:
      minmax_kernel<<<grid, block, 0, st>>>(static_cast<const int16_t*>(img), n, mm);
      break;
    case SI_I32:
      minmax_kernel<<<grid, block, 0, st>>>(static_cast<const int32_t*>(img), n, mm);
      break;
    case SI_F32:
      minmax_kernel<<<grid, block, 0, st>>>(static_cast<const float*>(img), n, mm);
      break;
    default:
      return set_error(SI_ERR_ARG, "si_image_minmax: unsupported image dtype %d", dtype);
  }
  return check_launch("si_image_minmax");
}

extern "C" int si_prepare_image(const void* img, int dtype, int Z0, int Y0, int X0, int cz0, int cy0, int cx0,
                                int Zc, int Yc, int Xc, float norm_min, float norm_range, int denoise, void* work,
                                void* stream) {
  clear_error();
  if (!img || !work) return set_error(SI_ERR_ARG, "si_prepare_image: null pointer");
  if (Z0 <= 0 || Y0 <= 0 || X0 <= 0 || Zc < 3 || Yc < 3 || Xc < 3)
    return set_error(SI_ERR_ARG, "si_prepare_image: bad dims");
  if (cz0 < 0 || cy0 < 0 || cx0 < 0 || cz0 + Zc > Z0 + 2 || cy0 + Yc > Y0 + 2 || cx0 + Xc > X0 + 2)
    return set_error(SI_ERR_ARG, "si_prepare_image: crop outside the padded frame");
  const Crop cr{Z0, Y0, X0, cz0, cy0, cx0, Zc, Yc, Xc};
  const uint64_t n = (uint64_t)Zc * Yc * Xc;
  const int block = 256, grid = grid_for(n, block);
  cudaStream_t st = as_stream(stream);
  switch (dtype) {
    case SI_U8:
      prepare_u8_kernel<<<grid, block, 0, st>>>(static_cast<const uint8_t*>(img), cr, denoise,
                                                static_cast<uint8_t*>(work));
      break;
    case SI_I8:
      prepare_u8_kernel<<<grid, block, 0, st>>>(static_cast<const int8_t*>(img), cr, denoise,
                                                static_cast<uint8_t*>(work));
      break;
    case SI_U16:
      prepare_f32_kernel<<<grid, block, 0, st>>>(static_cast<const uint16_t*>(img), cr, norm_min, norm_range,
                                                 denoise, static_cast<float*>(work));
      break;
    case SI_I16:
      prepare_f32_kernel<<<grid, block, 0, st>>>(static_cast<const int16_t*>(img), cr, norm_min, norm_range,
                                                 denoise, static_cast<float*>(work));
      break;
    case SI_I32:
      prepare_f32_kernel<<<grid, block, 0, st>>>(static_cast<const int32_t*>(img), cr, norm_min, norm_range,
                                                 denoise, static_cast<float*>(work));
      break;
    case SI_F32:
      prepare_f32_kernel<<<grid, block, 0, st>>>(static_cast<const float*>(img), cr, norm_min, norm_range,
                                                 denoise, static_cast<float*>(work));
      break;
    default:
      return set_error(SI_ERR_ARG, "si_prepare_image: unsupported image dtype %d", dtype);
  }
  return check_launch("si_prepare_image");
}
