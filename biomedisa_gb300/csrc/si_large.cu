// The reference large path's adaptive seed filter (pycuda_large.py:513-533,
// and for all axes pycuda_large_allx.py:513-533 / :683-703): a seed walks iff
// (row + column) % 4 == 0 or its in-slice window [-100, 100]^2, clipped to the
// interior rows/columns 1..n-2 of its slice plane, holds a label that is
// neither the seed's own nor -1. Rows and columns are the plane's: z-slices
// (y, x), y-slices (z, x), x-slices (z, y). Labels outside the plane's box
// (reduceBlocksize, pycuda_large.py:39-58 / pycuda_large_allx.py:37-57; one
// box per axis) read as -1.
//
// "Some window label differs from `own`" is evaluated as min/max over the
// window of the labels other than -1 (the seed itself is in its window, so
// min == max == own exactly when none differs): a row pass (window along x,
// row in shared memory) then a column pass (window along y) over the taken
// slices, int16 values (labels below -32767 saturate, which keeps them
// different from every own label and from -1).
#include <algorithm>
#include <cstdint>

#include "si_common.cuh"
#include "si_internal.h"

namespace si {
namespace {

constexpr int kWin = 100;
constexpr int16_t kNoMin = 32767, kNoMax = -32768;

struct LargeGeom {
  int Z0, Y0, X0, cz0, cy0, cx0, Zc, Yc, Xc;
  int box[3][4];  // per axis, [r0, r1) x [c0, c1) of the slice plane
  int pairs;      // slice entries are (axis, index) pairs; 0: z indices
  int64_t plane;  // scratch elements per slice entry
};

__device__ __forceinline__ int rows_of(const LargeGeom& g, int axis) { return axis == 0 ? g.Yc : g.Zc; }
__device__ __forceinline__ int cols_of(const LargeGeom& g, int axis) { return axis == 2 ? g.Yc : g.Xc; }
__device__ __forceinline__ int lut_off(const LargeGeom& g, int axis) {
  return axis == 0 ? 0 : axis == 1 ? g.Zc : g.Zc + g.Yc;
}

__device__ __forceinline__ void slice_entry(const int32_t* slices, int pairs, int e, int& axis, int& s) {
  axis = pairs ? slices[2 * e] : 0;
  s = pairs ? slices[2 * e + 1] : slices[e];
}

// (slice s, row r, column c) of an axis -> crop coordinates: z-slices (y, x),
// y-slices (z, x), x-slices (z, y).
__device__ __forceinline__ void to_crop(int axis, int s, int r, int c, int& z, int& y, int& x) {
  if (axis == 0) {
    z = s; y = r; x = c;
  } else if (axis == 1) {
    z = r; y = s; x = c;
  } else {
    z = r; y = c; x = s;
  }
}

// label at (row r, column c) of slice s of an axis, as the large walker's
// slice stack of that axis holds it
template <typename T>
__device__ __forceinline__ int stack_label(const T* lab, const LargeGeom& g, const int16_t* slot_lut,
                                           const uint8_t* slot_label, int axis, int s, int r, int c) {
  const int* b = g.box[axis];
  if (r < b[0] || r >= b[1] || c < b[2] || c >= b[3]) return -1;
  int z, y, x;
  to_crop(axis, s, r, c, z, y, x);
  const int oz = z + g.cz0 - 1, oy = y + g.cy0 - 1, ox = x + g.cx0 - 1;
  int v = 0;
  if ((unsigned)oz < (unsigned)g.Z0 && (unsigned)oy < (unsigned)g.Y0 && (unsigned)ox < (unsigned)g.X0)
    v = static_cast<int>(lab[((int64_t)oz * g.Y0 + oy) * g.X0 + ox]);
  if (v < 0) return v < -32767 ? -32767 : v;
  if (v > 255) return 0;
  const int sl = slot_lut[v];
  return sl >= 0 ? slot_label[sl] : 0;
}

template <typename T>
__global__ void __launch_bounds__(256) window_rows_kernel(const T* __restrict__ lab, LargeGeom g,
                                                          const int16_t* __restrict__ slot_lut,
                                                          const uint8_t* __restrict__ slot_label,
                                                          const int32_t* __restrict__ slices,
                                                          int16_t* __restrict__ rmin, int16_t* __restrict__ rmax) {
  extern __shared__ int16_t row[];
  const int r = blockIdx.x, e = blockIdx.y;
  int axis, s;
  slice_entry(slices, g.pairs, e, axis, s);
  const int R = rows_of(g, axis), C = cols_of(g, axis);
  if (r < 1 || r > R - 2) return;  // uniform: only interior rows enter a window
  for (int c = threadIdx.x; c < C; c += blockDim.x)
    row[c] = (int16_t)stack_label(lab, g, slot_lut, slot_label, axis, s, r, c);
  __syncthreads();
  const int64_t base = (int64_t)e * g.plane + (int64_t)r * C;
  for (int c = 1 + threadIdx.x; c <= C - 2; c += blockDim.x) {
    const int lo = max(1, c - kWin), hi = min(C - 2, c + kWin);
    int mn = kNoMin, mx = kNoMax;
    for (int cc = lo; cc <= hi; ++cc) {
      const int v = row[cc];
      if (v != -1) {
        mn = min(mn, v);
        mx = max(mx, v);
      }
    }
    rmin[base + c] = (int16_t)mn;
    rmax[base + c] = (int16_t)mx;
  }
}

__global__ void __launch_bounds__(256) window_cols_kernel(LargeGeom g, const int32_t* __restrict__ slices,
                                                          const int16_t* __restrict__ rmin,
                                                          const int16_t* __restrict__ rmax, int16_t* __restrict__ wmin,
                                                          int16_t* __restrict__ wmax) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y, e = blockIdx.z;
  int axis, s;
  slice_entry(slices, g.pairs, e, axis, s);
  const int R = rows_of(g, axis), C = cols_of(g, axis);
  if (c < 1 || c > C - 2 || r < 1 || r > R - 2) return;
  const int lo = max(1, r - kWin), hi = min(R - 2, r + kWin);
  const int64_t plane = (int64_t)e * g.plane;
  int mn = kNoMin, mx = kNoMax;
  for (int rr = lo; rr <= hi; ++rr) {
    mn = min(mn, (int)rmin[plane + (int64_t)rr * C + c]);
    mx = max(mx, (int)rmax[plane + (int64_t)rr * C + c]);
  }
  wmin[plane + (int64_t)r * C + c] = (int16_t)mn;
  wmax[plane + (int64_t)r * C + c] = (int16_t)mx;
}

__global__ void slice_lut_kernel(LargeGeom g, const int32_t* __restrict__ slices, int n, int32_t* __restrict__ lut) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    int axis, s;
    slice_entry(slices, g.pairs, e, axis, s);
    const int len = axis == 0 ? g.Zc : axis == 1 ? g.Yc : g.Xc;
    if ((unsigned)s < (unsigned)len) lut[lut_off(g, axis) + s] = e;
  }
}

__global__ void __launch_bounds__(256) filter_kernel(const SeedRec* __restrict__ in, const uint32_t* __restrict__ n_in,
                                                     LargeGeom g, const int32_t* __restrict__ lut,
                                                     const int16_t* __restrict__ wmin,
                                                     const int16_t* __restrict__ wmax, SeedRec* __restrict__ out,
                                                     uint32_t* __restrict__ n_out) {
  const uint32_t n = *n_in;
  const int64_t F = (int64_t)g.Yc * g.Xc;
  const int lane = threadIdx.x & 31;
  // whole warps iterate together (warp-aggregated compaction)
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t nw = (n + 31u) & ~31u;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += stride) {
    bool keep = false;
    SeedRec rec;
    if (i < n) {
      rec = in[i];
      const int64_t pos = rec.pos;
      const int z = (int)(pos / F), y = (int)((pos / g.Xc) % g.Yc), x = (int)(pos % g.Xc);
      const int own = (int)((rec.meta >> 16) & 0xFFu);
      const int axis = g.pairs ? (int)((rec.meta >> 8) & 3u) : 0;
      const int s = axis == 0 ? z : axis == 1 ? y : x;
      const int r = axis == 0 ? y : z, c = axis == 2 ? y : x;
      const int e = axis < 3 ? lut[lut_off(g, axis) + s] : -1;
      if (((r + c) & 3) == 0) {
        keep = true;
      } else if (e >= 0) {
        const int64_t w = (int64_t)e * g.plane + (int64_t)r * (axis == 2 ? g.Yc : g.Xc) + c;
        keep = wmin[w] != own || wmax[w] != own;
      }
    }
    const unsigned ballot = __ballot_sync(0xffffffffu, keep);
    uint32_t base = 0;
    if (lane == 0 && ballot) base = atomicAdd(n_out, (uint32_t)__popc(ballot));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (keep) out[base + __popc(ballot & ((1u << lane) - 1u))] = rec;
  }
}

}  // namespace
}  // namespace si

using namespace si;

static uint64_t align256(uint64_t v) { return (v + 255) & ~255ull; }

static uint64_t plane_elems(int Zc, int Yc, int Xc, int pairs) {
  uint64_t p = (uint64_t)Yc * Xc;
  if (pairs) {
    p = std::max<uint64_t>(p, (uint64_t)Zc * Xc);
    p = std::max<uint64_t>(p, (uint64_t)Zc * Yc);
  }
  return p;
}

static uint64_t scratch_bytes(int Zc, int Yc, int Xc, int n_slices, int pairs) {
  const uint64_t plane = (uint64_t)n_slices * plane_elems(Zc, Yc, Xc, pairs) * sizeof(int16_t);
  return 4 * align256(plane) + align256(((uint64_t)Zc + Yc + Xc) * sizeof(int32_t));
}

extern "C" int si_adaptive_scratch_bytes(int Zc, int Yc, int Xc, int n_slices, uint64_t* bytes) {
  clear_error();
  if (!bytes || Zc < 1 || Yc < 1 || Xc < 1 || n_slices < 0)
    return set_error(SI_ERR_ARG, "si_adaptive_scratch_bytes: bad arguments");
  *bytes = scratch_bytes(Zc, Yc, Xc, n_slices, 0);
  return 0;
}

extern "C" int si_adaptive_scratch_bytes_allx(int Zc, int Yc, int Xc, int n_slices, uint64_t* bytes) {
  clear_error();
  if (!bytes || Zc < 1 || Yc < 1 || Xc < 1 || n_slices < 0)
    return set_error(SI_ERR_ARG, "si_adaptive_scratch_bytes_allx: bad arguments");
  *bytes = scratch_bytes(Zc, Yc, Xc, n_slices, 1);
  return 0;
}

static int adaptive_filter_impl(const char* who, const void* labels, int dtype, int Z0, int Y0, int X0, int cz0,
                                int cy0, int cx0, int Zc, int Yc, int Xc, const int16_t* slot_lut,
                                const uint8_t* slot_label, const int32_t* slices, int pairs, int n_slices,
                                const int32_t* boxes, const si_seed_t* seeds_in, const uint32_t* n_in,
                                uint32_t max_in, si_seed_t* seeds_out, uint32_t* n_out, void* scratch,
                                uint64_t scratch_bytes_given, void* stream) {
  if (!labels || !slot_lut || !slot_label || !seeds_in || !n_in || !seeds_out || !n_out || !scratch || !boxes)
    return set_error(SI_ERR_ARG, "%s: null pointer", who);
  if (n_slices < 0 || (n_slices > 0 && !slices) || n_slices > 65535)
    return set_error(SI_ERR_ARG, "%s: bad slice list", who);
  if (Zc < 3 || Yc < 3 || Xc < 3 || Yc > 65535 || (pairs && Zc > 65535))
    return set_error(SI_ERR_ARG, "%s: bad crop", who);
  const int max_cols = pairs ? std::max(Xc, Yc) : Xc;
  const int max_rows = pairs ? std::max(Yc, Zc) : Yc;
  if (max_cols > 24576) return set_error(SI_ERR_LIMIT, "%s: rows wider than 24576 voxels", who);
  if (scratch_bytes_given < scratch_bytes(Zc, Yc, Xc, n_slices, pairs) || (uintptr_t)scratch % 256)
    return set_error(SI_ERR_ARG, "%s: scratch too small or misaligned", who);
  cudaStream_t st = as_stream(stream);
  if (cudaMemsetAsync(n_out, 0, sizeof(uint32_t), st) != cudaSuccess)
    return set_error(SI_ERR_CUDA, "%s: memset failed", who);
  if (n_slices == 0 || max_in == 0) return check_launch(who);
  LargeGeom g{Z0, Y0, X0, cz0, cy0, cx0, Zc, Yc, Xc, {}, pairs, (int64_t)plane_elems(Zc, Yc, Xc, pairs)};
  for (int a = 0; a < 3; ++a)
    for (int k = 0; k < 4; ++k) g.box[a][k] = boxes[4 * a + k];
  const uint64_t plane = align256((uint64_t)n_slices * g.plane * sizeof(int16_t));
  uint8_t* base = static_cast<uint8_t*>(scratch);
  int16_t* rmin = reinterpret_cast<int16_t*>(base);
  int16_t* rmax = reinterpret_cast<int16_t*>(base + plane);
  int16_t* wmin = reinterpret_cast<int16_t*>(base + 2 * plane);
  int16_t* wmax = reinterpret_cast<int16_t*>(base + 3 * plane);
  int32_t* lut = reinterpret_cast<int32_t*>(base + 4 * plane);
  if (cudaMemsetAsync(lut, 0xFF, ((size_t)Zc + Yc + Xc) * sizeof(int32_t), st) != cudaSuccess)
    return set_error(SI_ERR_CUDA, "%s: memset failed", who);
  slice_lut_kernel<<<(n_slices + 255) / 256, 256, 0, st>>>(g, slices, n_slices, lut);
  const dim3 rgrid(max_rows, n_slices);
  const size_t smem = (size_t)max_cols * sizeof(int16_t);
  if (smem > 48 * 1024) {
#define SI_SMEM_ATTR(T)                                                                                     \
  cudaFuncSetAttribute(window_rows_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
    SI_SMEM_ATTR(uint8_t);
    SI_SMEM_ATTR(int16_t);
    SI_SMEM_ATTR(int32_t);
#undef SI_SMEM_ATTR
  }
  switch (dtype) {
    case SI_U8:
      window_rows_kernel<uint8_t><<<rgrid, 256, smem, st>>>(static_cast<const uint8_t*>(labels), g, slot_lut,
                                                             slot_label, slices, rmin, rmax);
      break;
    case SI_I16:
      window_rows_kernel<int16_t><<<rgrid, 256, smem, st>>>(static_cast<const int16_t*>(labels), g, slot_lut,
                                                             slot_label, slices, rmin, rmax);
      break;
    case SI_I32:
      window_rows_kernel<int32_t><<<rgrid, 256, smem, st>>>(static_cast<const int32_t*>(labels), g, slot_lut,
                                                             slot_label, slices, rmin, rmax);
      break;
    default:
      return set_error(SI_ERR_ARG, "%s: unsupported label dtype %d", who, dtype);
  }
  window_cols_kernel<<<dim3((max_cols + 255) / 256, max_rows, n_slices), 256, 0, st>>>(g, slices, rmin, rmax, wmin,
                                                                                      wmax);
  const int fgrid = (int)std::min<uint64_t>((max_in + 255) / 256, (uint64_t)sm_count() * 16);
  filter_kernel<<<fgrid > 0 ? fgrid : 1, 256, 0, st>>>(reinterpret_cast<const SeedRec*>(seeds_in), n_in, g, lut,
                                                       wmin, wmax, reinterpret_cast<SeedRec*>(seeds_out), n_out);
  return check_launch(who);
}

extern "C" int si_adaptive_seed_filter(const void* labels, int dtype, int Z0, int Y0, int X0, int cz0, int cy0,
                                       int cx0, int Zc, int Yc, int Xc, const int16_t* slot_lut,
                                       const uint8_t* slot_label, const int32_t* slice_z, int n_slices, int box_y0,
                                       int box_y1, int box_x0, int box_x1, const si_seed_t* seeds_in,
                                       const uint32_t* n_in, uint32_t max_in, si_seed_t* seeds_out,
                                       uint32_t* n_out, void* scratch, uint64_t scratch_bytes, void* stream) {
  clear_error();
  const int32_t boxes[12] = {box_y0, box_y1, box_x0, box_x1, 0, Zc, 0, Xc, 0, Zc, 0, Yc};
  return adaptive_filter_impl("si_adaptive_seed_filter", labels, dtype, Z0, Y0, X0, cz0, cy0, cx0, Zc, Yc, Xc,
                              slot_lut, slot_label, slice_z, 0, n_slices, boxes, seeds_in, n_in, max_in, seeds_out,
                              n_out, scratch, scratch_bytes, stream);
}

extern "C" int si_adaptive_seed_filter_allx(const void* labels, int dtype, int Z0, int Y0, int X0, int cz0, int cy0,
                                            int cx0, int Zc, int Yc, int Xc, const int16_t* slot_lut,
                                            const uint8_t* slot_label, const int32_t* slice_list, int n_slices,
                                            const int32_t* boxes, const si_seed_t* seeds_in, const uint32_t* n_in,
                                            uint32_t max_in, si_seed_t* seeds_out, uint32_t* n_out, void* scratch,
                                            uint64_t scratch_bytes, void* stream) {
  clear_error();
  return adaptive_filter_impl("si_adaptive_seed_filter_allx", labels, dtype, Z0, Y0, X0, cz0, cy0, cx0, Zc, Yc,
                              Xc, slot_lut, slot_label, slice_list, 1, n_slices, boxes, seeds_in, n_in, max_in,
                              seeds_out, n_out, scratch, scratch_bytes, stream);
}
