// The reference large path's adaptive seed filter (pycuda_large.py:513-533):
// a seed of a taken z-slice walks iff (row + column) % 4 == 0 or its in-slice
// window [-100, 100]^2, clipped to the interior rows/columns 1..n-2 of the
// crop, holds a label that is neither the seed's own nor -1. Labels outside
// the in-plane box of pycuda_large.py:39-58 read as -1.
//
// "Some window label differs from `own`" is evaluated as min/max over the
// window of the labels other than -1 (the seed itself is in its window, so
// min == max == own exactly when none differs): a row pass (window along x,
// row in shared memory) then a column pass (window along y) over the taken
// slices, int16 values (labels below -32767 saturate, which keeps them
// different from every own label and from -1).
#include <cstdint>

#include "si_common.cuh"
#include "si_internal.h"

namespace si {
namespace {

constexpr int kWin = 100;
constexpr int16_t kNoMin = 32767, kNoMax = -32768;

struct LargeGeom {
  int Z0, Y0, X0, cz0, cy0, cx0, Zc, Yc, Xc;
  int by0, by1, bx0, bx1;
};

// label at crop (z, y, x) as the large walker's slice stack holds it
template <typename T>
__device__ __forceinline__ int stack_label(const T* lab, const LargeGeom& g, const int16_t* slot_lut,
                                           const uint8_t* slot_label, int z, int y, int x) {
  if (y < g.by0 || y >= g.by1 || x < g.bx0 || x >= g.bx1) return -1;
  const int oz = z + g.cz0 - 1, oy = y + g.cy0 - 1, ox = x + g.cx0 - 1;
  int v = 0;
  if ((unsigned)oz < (unsigned)g.Z0 && (unsigned)oy < (unsigned)g.Y0 && (unsigned)ox < (unsigned)g.X0)
    v = static_cast<int>(lab[((int64_t)oz * g.Y0 + oy) * g.X0 + ox]);
  if (v < 0) return v < -32767 ? -32767 : v;
  if (v > 255) return 0;
  const int s = slot_lut[v];
  return s >= 0 ? slot_label[s] : 0;
}

template <typename T>
__global__ void __launch_bounds__(256) window_rows_kernel(const T* __restrict__ lab, LargeGeom g,
                                                          const int16_t* __restrict__ slot_lut,
                                                          const uint8_t* __restrict__ slot_label,
                                                          const int32_t* __restrict__ slice_z,
                                                          int16_t* __restrict__ rmin, int16_t* __restrict__ rmax) {
  extern __shared__ int16_t row[];
  const int y = blockIdx.x, s = blockIdx.y;
  if (y < 1 || y > g.Yc - 2) return;  // uniform: only interior rows enter a window
  const int z = slice_z[s];
  for (int x = threadIdx.x; x < g.Xc; x += blockDim.x)
    row[x] = (int16_t)stack_label(lab, g, slot_lut, slot_label, z, y, x);
  __syncthreads();
  const int64_t base = ((int64_t)s * g.Yc + y) * g.Xc;
  for (int x = 1 + threadIdx.x; x <= g.Xc - 2; x += blockDim.x) {
    const int lo = max(1, x - kWin), hi = min(g.Xc - 2, x + kWin);
    int mn = kNoMin, mx = kNoMax;
    for (int xx = lo; xx <= hi; ++xx) {
      const int v = row[xx];
      if (v != -1) {
        mn = min(mn, v);
        mx = max(mx, v);
      }
    }
    rmin[base + x] = (int16_t)mn;
    rmax[base + x] = (int16_t)mx;
  }
}

__global__ void __launch_bounds__(256) window_cols_kernel(int Yc, int Xc, const int16_t* __restrict__ rmin,
                                                          const int16_t* __restrict__ rmax, int16_t* __restrict__ wmin,
                                                          int16_t* __restrict__ wmax) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, s = blockIdx.z;
  if (x < 1 || x > Xc - 2 || y < 1 || y > Yc - 2) return;
  const int lo = max(1, y - kWin), hi = min(Yc - 2, y + kWin);
  const int64_t plane = (int64_t)s * Yc * Xc;
  int mn = kNoMin, mx = kNoMax;
  for (int yy = lo; yy <= hi; ++yy) {
    mn = min(mn, (int)rmin[plane + (int64_t)yy * Xc + x]);
    mx = max(mx, (int)rmax[plane + (int64_t)yy * Xc + x]);
  }
  wmin[plane + (int64_t)y * Xc + x] = (int16_t)mn;
  wmax[plane + (int64_t)y * Xc + x] = (int16_t)mx;
}

__global__ void zlut_kernel(const int32_t* __restrict__ slice_z, int n, int Zc, int32_t* __restrict__ zlut) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if ((unsigned)slice_z[i] < (unsigned)Zc) zlut[slice_z[i]] = i;
}

__global__ void __launch_bounds__(256) filter_kernel(const SeedRec* __restrict__ in, const uint32_t* __restrict__ n_in,
                                                     int Yc, int Xc, const int32_t* __restrict__ zlut,
                                                     const int16_t* __restrict__ wmin,
                                                     const int16_t* __restrict__ wmax, SeedRec* __restrict__ out,
                                                     uint32_t* __restrict__ n_out) {
  const uint32_t n = *n_in;
  const int64_t F = (int64_t)Yc * Xc;
  const int lane = threadIdx.x & 31;
  // whole warps iterate together (warp-aggregated compaction)
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t nw = (n + 31u) & ~31u;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += stride) {
    bool keep = false;
    SeedRec r;
    if (i < n) {
      r = in[i];
      const int64_t pos = r.pos;
      const int z = (int)(pos / F), y = (int)((pos / Xc) % Yc), x = (int)(pos % Xc);
      const int own = (int)((r.meta >> 16) & 0xFFu);
      const int s = zlut[z];
      if (((y + x) & 3) == 0) {
        keep = true;
      } else if (s >= 0) {
        const int64_t w = ((int64_t)s * Yc + y) * Xc + x;
        keep = wmin[w] != own || wmax[w] != own;
      }
    }
    const unsigned ballot = __ballot_sync(0xffffffffu, keep);
    uint32_t base = 0;
    if (lane == 0 && ballot) base = atomicAdd(n_out, (uint32_t)__popc(ballot));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (keep) out[base + __popc(ballot & ((1u << lane) - 1u))] = r;
  }
}

}  // namespace
}  // namespace si

using namespace si;

static uint64_t align256(uint64_t v) { return (v + 255) & ~255ull; }

extern "C" int si_adaptive_scratch_bytes(int Zc, int Yc, int Xc, int n_slices, uint64_t* bytes) {
  clear_error();
  if (!bytes || Zc < 1 || Yc < 1 || Xc < 1 || n_slices < 0)
    return set_error(SI_ERR_ARG, "si_adaptive_scratch_bytes: bad arguments");
  const uint64_t plane = (uint64_t)n_slices * Yc * Xc * sizeof(int16_t);
  *bytes = 4 * align256(plane) + align256((uint64_t)Zc * sizeof(int32_t));
  return 0;
}

extern "C" int si_adaptive_seed_filter(const void* labels, int dtype, int Z0, int Y0, int X0, int cz0, int cy0,
                                       int cx0, int Zc, int Yc, int Xc, const int16_t* slot_lut,
                                       const uint8_t* slot_label, const int32_t* slice_z, int n_slices, int box_y0,
                                       int box_y1, int box_x0, int box_x1, const si_seed_t* seeds_in,
                                       const uint32_t* n_in, uint32_t max_in, si_seed_t* seeds_out,
                                       uint32_t* n_out, void* scratch, uint64_t scratch_bytes, void* stream) {
  clear_error();
  if (!labels || !slot_lut || !slot_label || !seeds_in || !n_in || !seeds_out || !n_out || !scratch)
    return set_error(SI_ERR_ARG, "si_adaptive_seed_filter: null pointer");
  if (n_slices < 0 || (n_slices > 0 && !slice_z) || n_slices > 65535)
    return set_error(SI_ERR_ARG, "si_adaptive_seed_filter: bad slice list");
  if (Zc < 3 || Yc < 3 || Xc < 3 || Yc > 65535) return set_error(SI_ERR_ARG, "si_adaptive_seed_filter: bad crop");
  if (Xc > 24576) return set_error(SI_ERR_LIMIT, "si_adaptive_seed_filter: rows wider than 24576 voxels");
  uint64_t need = 0;
  si_adaptive_scratch_bytes(Zc, Yc, Xc, n_slices, &need);
  if (scratch_bytes < need || (uintptr_t)scratch % 256)
    return set_error(SI_ERR_ARG, "si_adaptive_seed_filter: scratch too small or misaligned");
  cudaStream_t st = as_stream(stream);
  if (cudaMemsetAsync(n_out, 0, sizeof(uint32_t), st) != cudaSuccess)
    return set_error(SI_ERR_CUDA, "si_adaptive_seed_filter: memset failed");
  if (n_slices == 0 || max_in == 0) return check_launch("si_adaptive_seed_filter");
  const uint64_t plane = align256((uint64_t)n_slices * Yc * Xc * sizeof(int16_t));
  uint8_t* base = static_cast<uint8_t*>(scratch);
  int16_t* rmin = reinterpret_cast<int16_t*>(base);
  int16_t* rmax = reinterpret_cast<int16_t*>(base + plane);
  int16_t* wmin = reinterpret_cast<int16_t*>(base + 2 * plane);
  int16_t* wmax = reinterpret_cast<int16_t*>(base + 3 * plane);
  int32_t* zlut = reinterpret_cast<int32_t*>(base + 4 * plane);
  if (cudaMemsetAsync(zlut, 0xFF, (size_t)Zc * sizeof(int32_t), st) != cudaSuccess)
    return set_error(SI_ERR_CUDA, "si_adaptive_seed_filter: memset failed");
  zlut_kernel<<<(n_slices + 255) / 256, 256, 0, st>>>(slice_z, n_slices, Zc, zlut);
  const LargeGeom g{Z0, Y0, X0, cz0, cy0, cx0, Zc, Yc, Xc, box_y0, box_y1, box_x0, box_x1};
  const dim3 rgrid(Yc, n_slices);
  const size_t smem = (size_t)Xc * sizeof(int16_t);
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
                                                             slot_label, slice_z, rmin, rmax);
      break;
    case SI_I16:
      window_rows_kernel<int16_t><<<rgrid, 256, smem, st>>>(static_cast<const int16_t*>(labels), g, slot_lut,
                                                             slot_label, slice_z, rmin, rmax);
      break;
    case SI_I32:
      window_rows_kernel<int32_t><<<rgrid, 256, smem, st>>>(static_cast<const int32_t*>(labels), g, slot_lut,
                                                             slot_label, slice_z, rmin, rmax);
      break;
    default:
      return set_error(SI_ERR_ARG, "si_adaptive_seed_filter: unsupported label dtype %d", dtype);
  }
  window_cols_kernel<<<dim3((Xc + 255) / 256, Yc, n_slices), 256, 0, st>>>(Yc, Xc, rmin, rmax, wmin, wmax);
  const int fgrid = (int)std::min<uint64_t>((max_in + 255) / 256, (uint64_t)sm_count() * 16);
  filter_kernel<<<fgrid > 0 ? fgrid : 1, 256, 0, st>>>(reinterpret_cast<const SeedRec*>(seeds_in), n_in, Yc, Xc,
                                                       zlut, wmin, wmax, reinterpret_cast<SeedRec*>(seeds_out),
                                                       n_out);
  return check_launch("si_adaptive_seed_filter");
}
