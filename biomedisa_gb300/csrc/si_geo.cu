// Geodesic raster-scan interpolation (biomedisa/geodis.py): image
// normalisation, per-label seed masks, the forward/backward raster scans and
// the per-voxel label selection.
//
// The reference scan (geodis.py:44-76) is an in-place Gauss-Seidel sweep: a
// voxel takes the minimum over itself and 13 neighbours that come EARLIER in
// the pass's raster order. With t = x + 2y + 4z every one of the 13 forward
// offsets lowers t (by 1..7) and every backward offset raises it, so all voxels
// of one t read only finished values. Three schedules reproduce the
// sequential sweep exactly:
//   * tiled (default): tiles in skewed coordinates (p, q, r) = (t, y + 2z, z),
//     one launch per tile-wavefront, each tile worked plane by plane in
//     shared memory (geo_tile_kernel);
//   * wavefronts: one launch per wavefront t, in increasing t (forward) or
//     decreasing t (backward) (geo_wave_kernel);
//   * cluster: every wavefront inside one launch, a thread-block cluster per
//     label synchronised by the cluster barrier (geo_cluster_scan_kernel).
// All labels share each launch. The tiled and wavefront launches can be
// replayed from cached CUDA graphs.
//
// Arithmetic (numba's typing of the reference, see the scan kernel): the
// intensity difference and its square are binary32, the cost sum and the
// comparison binary64, the store rounds to binary32.
#include <atomic>
#include <cmath>
#include <mutex>
#include <vector>

#include "si_common.cuh"
#include "si_internal.h"

namespace si {
namespace {

// Forward offsets (dz, dy, dx) in the reference's order (geodis.py:12-26); the
// backward scan uses their negations in the same order (:28-42).
constexpr int kGeoOff[13][3] = {
    {-1, -1, -1}, {-1, -1, 0}, {-1, -1, 1}, {-1, 0, -1}, {-1, 0, 0}, {-1, 0, 1}, {-1, 1, -1},
    {-1, 1, 0},   {-1, 1, 1},  {0, -1, -1}, {0, -1, 0},  {0, -1, 1}, {0, 0, -1},
};

__host__ __device__ inline int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }
__host__ __device__ inline int ceil_div(int a, int b) { return -floor_div(-a, b); }
__host__ __device__ inline int imax(int a, int b) { return a > b ? a : b; }
__host__ __device__ inline int imin(int a, int b) { return a < b ? a : b; }

// The voxels of wavefront t: x = t - 2y - 4z inside the pass's domain
// (forward z = 1..Z-1, backward z = 0..Z-2; both y = 1..Y-2, x = 1..X-2).
// Thread (zi, j) of a launch takes z = zlo + zi (zi < nz) and the j-th valid y
// of that plane (j < jmax = the most y values any plane can have).
struct GeoWave {
  int t, zlo, nz, jmax;
};

__host__ __device__ inline GeoWave geo_wave(int Z, int Y, int X, int fwd, int t) {
  GeoWave w{t, 0, 0, (X - 1) / 2};
  const int zmin = fwd ? 1 : 0, zmax = fwd ? Z - 1 : Z - 2;
  // 1 <= x = t - 2y - 4z <= X-2 and 1 <= y <= Y-2 bound 4z to [t-(X-2)-2(Y-2), t-3]
  const int zlo = imax(zmin, ceil_div(t - (X - 2) - 2 * (Y - 2), 4));
  const int zhi = imin(zmax, floor_div(t - 3, 4));
  w.zlo = zlo;
  w.nz = zhi >= zlo ? zhi - zlo + 1 : 0;
  return w;
}

__host__ __device__ inline bool geo_wave_voxel(int Y, int X, const GeoWave& w, int zi, int j, int* z, int* y,
                                               int* x) {
  const int zz = w.zlo + zi;
  const int r = w.t - 4 * zz;
  const int ylo = imax(1, ceil_div(r - (X - 2), 2));
  const int yhi = imin(Y - 2, floor_div(r - 1, 2));
  const int yy = ylo + j;
  if (yy > yhi) return false;
  *z = zz;
  *y = yy;
  *x = r - 2 * yy;
  return true;
}

// Wavefront ranges of one pass: first, last (inclusive) and step.
__host__ __device__ inline void geo_t_range(int Z, int Y, int X, int fwd, int* t0, int* t1, int* step) {
  if (fwd) {
    *t0 = 1 + 2 + 4;
    *t1 = (X - 2) + 2 * (Y - 2) + 4 * (Z - 1);
    *step = 1;
  } else {
    *t0 = (X - 2) + 2 * (Y - 2) + 4 * (Z - 2);
    *t1 = 1 + 2 + 0;
    *step = -1;
  }
}

inline bool geo_has_interior(int Z, int Y, int X) { return Z >= 2 && Y >= 3 && X >= 3; }

struct GeoScanArgs {
  float* c;
  const float* img;
  int Z, Y, X, nol;
  long long V;
  long long off[13];  // forward linear offsets
  int box_off[13];    // the same offsets in the tiled kernel's shared-memory box
  double w[13];       // (1 - lamb) * |offset|
  double lamb;
};

// Update of voxel v of one distance map cl. kLamb1: lamb == 1.0, where the
// reference's float64 cost c[q] + 0.0 + 1.0*sq equals the binary64 sum of two
// binary32 values; rounding that sum to binary32 equals the binary32 sum
// (double rounding is innocuous for addition when 53 >= 2*24 + 2), and
// rounding is monotone, so the stored minimum is the binary32 minimum of the
// binary32 sums. Otherwise the float64 expression is evaluated as written.
// kL2: distance loads bypass L1 (ld.global.cg), for the cluster scan whose
// CTAs exchange values through L2 inside one launch.
template <bool kLamb1, bool kL2>
__device__ __forceinline__ void geo_update(const GeoScanArgs& a, float* cl, long long v, int fwd) {
  const float iv = a.img[v];
  if (kLamb1) {
    float best = kL2 ? __ldcg(cl + v) : cl[v];
#pragma unroll
    for (int n = 0; n < 13; ++n) {
      const long long q = fwd ? v + a.off[n] : v - a.off[n];
      const float diff = __fsub_rn(iv, a.img[q]);
      const float cq = kL2 ? __ldcg(cl + q) : cl[q];
      const float cost = __fadd_rn(cq, __fmul_rn(diff, diff));
      if (cost < best) best = cost;
    }
    cl[v] = best;
  } else {
    double best = (double)(kL2 ? __ldcg(cl + v) : cl[v]);
#pragma unroll
    for (int n = 0; n < 13; ++n) {
      const long long q = fwd ? v + a.off[n] : v - a.off[n];
      const float diff = __fsub_rn(iv, a.img[q]);
      const double sq = (double)__fmul_rn(diff, diff);
      const float cq = kL2 ? __ldcg(cl + q) : cl[q];
      const double cost = __dadd_rn(__dadd_rn((double)cq, a.w[n]), __dmul_rn(a.lamb, sq));
      if (cost < best) best = cost;
    }
    cl[v] = __double2float_rn(best);
  }
}

// Wavefront mode: one launch per wavefront t, one thread per (label, voxel).
template <bool kLamb1>
__global__ void __launch_bounds__(256) geo_wave_kernel(GeoScanArgs a, GeoWave w, int fwd) {
  const long long per_label = (long long)w.nz * w.jmax;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= per_label * a.nol) return;
  const int k = (int)(i / per_label);
  const long long r = i - (long long)k * per_label;
  const int zi = (int)(r / w.jmax);
  const int j = (int)(r - (long long)zi * w.jmax);
  int z, y, x;
  if (!geo_wave_voxel(a.Y, a.X, w, zi, j, &z, &y, &x)) return;
  geo_update<kLamb1, false>(a, a.c + (long long)k * a.V, ((long long)z * a.Y + y) * a.X + x, fwd);
}

// ---------------------------------------------------------------------------
// Tiled mode. In the skewed coordinates p = s(x + 2y + 4z), q = s(y + 2z),
// r = s z (s = +1 forward, -1 backward) every neighbour a voxel reads lies at
// (p + dp, q + dq, r + dr) with dp in [-7, -1], dq in [-3, 0], dr in [-1, 0]
// (the same 13 offsets for both passes). Rectangular tiles of kTileP x kTileQ
// x kTileR in (p, q, r) are therefore legal: a voxel's neighbours lie in its
// own tile or in tiles whose indices are all <= and one <, i.e. in an earlier
// tile-wavefront S = ip + iq + ir. One launch per S; a CTA takes one tile of
// one label, stages the tile and its halo (7 in p, 3 in q, 1 in r) of the
// distance map and the image in shared memory, updates its voxels plane by
// plane in p with a CTA barrier between planes (planes of equal p are
// independent), and writes the tile back.
// ---------------------------------------------------------------------------
constexpr int kTileP = 32, kTileQ = 32, kTileR = 8;
constexpr int kBoxP = kTileP + 7, kBoxQ = kTileQ + 3, kBoxR = kTileR + 1;
constexpr int kBoxCells = kBoxP * kBoxQ * kBoxR;
constexpr int kTileThreads = kTileQ * kTileR;
constexpr size_t kTileSmem = 2 * sizeof(float) * kBoxCells;
constexpr int kStageBatch = 8;
constexpr int kStageRounds = (kBoxCells + kTileThreads - 1) / kTileThreads;  // cells per thread, rounded up

struct GeoTiling {
  int s;             // +1 forward, -1 backward
  int zlo, zhi;      // z range of the pass
  int pb, qb, rb;    // smallest transformed coordinates over the pass's domain
  int ntp, ntq, ntr;  // tiles along p, q, r
};

__host__ __device__ inline GeoTiling geo_tiling(int Z, int Y, int X, int fwd) {
  GeoTiling g;
  g.s = fwd ? 1 : -1;
  g.zlo = fwd ? 1 : 0;
  g.zhi = fwd ? Z - 1 : Z - 2;
  const int pmin = 1 + 2 + 4 * g.zlo, pmax = (X - 2) + 2 * (Y - 2) + 4 * g.zhi;
  const int qmin = 1 + 2 * g.zlo, qmax = (Y - 2) + 2 * g.zhi;
  g.pb = fwd ? pmin : -pmax;
  g.qb = fwd ? qmin : -qmax;
  g.rb = fwd ? g.zlo : -g.zhi;
  g.ntp = (pmax - pmin + kTileP) / kTileP;
  g.ntq = (qmax - qmin + kTileQ) / kTileQ;
  g.ntr = (g.zhi - g.zlo + kTileR) / kTileR;
  return g;
}

// Volume coordinates of transformed (p, q, r).
__host__ __device__ inline void geo_unskew(const GeoTiling& g, int p, int q, int r, int* z, int* y, int* x) {
  *z = g.s * r;
  *y = g.s * q - 2 * *z;
  *x = g.s * p - 2 * *y - 4 * *z;
}

// Voxel at step k of column (cq, cr) of tile (ip, iq, ir); false when it is
// outside the pass's domain.
__host__ __device__ inline bool geo_tile_voxel(const GeoTiling& g, int Y, int X, int ip, int iq, int ir, int cq,
                                               int cr, int k, int* z, int* y, int* x) {
  geo_unskew(g, g.pb + ip * kTileP + k, g.qb + iq * kTileQ + cq, g.rb + ir * kTileR + cr, z, y, x);
  return *z >= g.zlo && *z <= g.zhi && *y >= 1 && *y <= Y - 2 && *x >= 1 && *x <= X - 2;
}

// Shared-memory box cell of transformed offset (dp, dq, dr) from the tile's
// corner cell (7, 3, 1).
__host__ __device__ constexpr int geo_box_cell(int bp, int bq, int br) { return (br * kBoxQ + bq) * kBoxP + bp; }

// Box offset of neighbour n: (dp, dq, dr) = (dx + 2dy + 4dz, dy + 2dz, dz).
inline int geo_box_offset(int n) {
  const int dz = kGeoOff[n][0], dy = kGeoOff[n][1], dx = kGeoOff[n][2];
  return geo_box_cell(dx + 2 * dy + 4 * dz, dy + 2 * dz, dz);
}

template <bool kLamb1>
__global__ void __launch_bounds__(kTileThreads) geo_tile_kernel(GeoScanArgs a, GeoTiling g, int S) {
  extern __shared__ float smem[];
  float* sc = smem;              // distances of the box
  float* si = smem + kBoxCells;  // image of the box
  const int iq = blockIdx.x % g.ntq, ir = blockIdx.x / g.ntq;
  const int ip = S - iq - ir;
  if (ip < 0 || ip >= g.ntp || ir >= g.ntr) return;  // uniform over the CTA
  float* cl = a.c + (long long)blockIdx.y * a.V;
  const int cq = threadIdx.x % kTileQ, cr = threadIdx.x / kTileQ;
  bool any = false;
  for (int k = 0; k < kTileP; ++k) {
    int z, y, x;
    any = any || geo_tile_voxel(g, a.Y, a.X, ip, iq, ir, cq, cr, k, &z, &y, &x);
  }
  if (!__syncthreads_or(any)) return;  // no voxel of the domain in this tile
  const int p0 = g.pb + ip * kTileP - 7, q0 = g.qb + iq * kTileQ - 3, r0 = g.rb + ir * kTileR - 1;
  // staging in batches of kStageBatch cells per thread: all loads of a batch
  // are issued before the first shared-memory store waits for one
  for (int b = 0; b < kStageRounds; b += kStageBatch) {
    float vc[kStageBatch], vi[kStageBatch];
#pragma unroll
    for (int u = 0; u < kStageBatch; ++u) {
      const int cell = threadIdx.x + (b + u) * kTileThreads;
      vc[u] = __uint_as_float(0x7f800000u);
      vi[u] = 0.0f;
      if (cell < kBoxCells) {
        const int bp = cell % kBoxP, bq = (cell / kBoxP) % kBoxQ, br = cell / (kBoxP * kBoxQ);
        int z, y, x;
        geo_unskew(g, p0 + bp, q0 + bq, r0 + br, &z, &y, &x);
        if (z >= 0 && z < a.Z && y >= 0 && y < a.Y && x >= 0 && x < a.X) {
          const long long v = ((long long)z * a.Y + y) * a.X + x;
          vc[u] = cl[v];
          vi[u] = a.img[v];
        }
      }
    }
#pragma unroll
    for (int u = 0; u < kStageBatch; ++u) {
      const int cell = threadIdx.x + (b + u) * kTileThreads;
      if (cell < kBoxCells) {
        sc[cell] = vc[u];
        si[cell] = vi[u];
      }
    }
  }
  __syncthreads();
  for (int k = 0; k < kTileP; ++k) {
    int z, y, x;
    if (geo_tile_voxel(g, a.Y, a.X, ip, iq, ir, cq, cr, k, &z, &y, &x)) {
      const int own = geo_box_cell(k + 7, cq + 3, cr + 1);
      const float iv = si[own];
      if (kLamb1) {
        float best = sc[own];
#pragma unroll
        for (int n = 0; n < 13; ++n) {
          const int nb = own + a.box_off[n];
          const float diff = __fsub_rn(iv, si[nb]);
          const float cost = __fadd_rn(sc[nb], __fmul_rn(diff, diff));
          if (cost < best) best = cost;
        }
        sc[own] = best;
      } else {
        double best = (double)sc[own];
#pragma unroll
        for (int n = 0; n < 13; ++n) {
          const int nb = own + a.box_off[n];
          const float diff = __fsub_rn(iv, si[nb]);
          const double sq = (double)__fmul_rn(diff, diff);
          const double cost = __dadd_rn(__dadd_rn((double)sc[nb], a.w[n]), __dmul_rn(a.lamb, sq));
          if (cost < best) best = cost;
        }
        sc[own] = __double2float_rn(best);
      }
    }
    __syncthreads();
  }
  for (int k = 0; k < kTileP; ++k) {
    int z, y, x;
    if (geo_tile_voxel(g, a.Y, a.X, ip, iq, ir, cq, cr, k, &z, &y, &x))
      cl[((long long)z * a.Y + y) * a.X + x] = sc[geo_box_cell(k + 7, cq + 3, cr + 1)];
  }
}

// Cluster mode: one thread-block cluster of kGeoCluster CTAs per label runs
// every pass and wavefront of the scan in one launch; the cluster's hardware
// barrier (release/acquire at cluster scope) separates the wavefronts. Every
// thread runs the same loop bounds (they depend on t only) and reaches every
// barrier; no thread leaves early.
constexpr int kGeoCluster = 8;
constexpr int kGeoClusterThreads = 1024;

__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

template <bool kLamb1>
__global__ void __launch_bounds__(kGeoClusterThreads, 1) geo_cluster_scan_kernel(GeoScanArgs a, int iterations) {
  const int k = blockIdx.x / kGeoCluster;
  const int tid = (blockIdx.x % kGeoCluster) * kGeoClusterThreads + threadIdx.x;
  const int nthr = kGeoCluster * kGeoClusterThreads;
  float* cl = a.c + (long long)k * a.V;
  for (int it = 0; it < iterations; ++it) {
    for (int fwd = 1; fwd >= 0; --fwd) {
      int t0, t1, step;
      geo_t_range(a.Z, a.Y, a.X, fwd, &t0, &t1, &step);
      for (int t = t0; step > 0 ? t <= t1 : t >= t1; t += step) {
        const GeoWave w = geo_wave(a.Z, a.Y, a.X, fwd, t);
        if (w.nz == 0) continue;  // uniform across the cluster
        const int per = w.nz * w.jmax;
        for (int i = tid; i < per; i += nthr) {
          const int zi = i / w.jmax, j = i - zi * w.jmax;
          int z, y, x;
          if (geo_wave_voxel(a.Y, a.X, w, zi, j, &z, &y, &x))
            geo_update<kLamb1, true>(a, cl, ((long long)z * a.Y + y) * a.X + x, fwd);
        }
        cluster_barrier();
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Normalisation (geodis.py:86-88): image.astype(float32); image -= amin;
// image /= amax. amin/amax follow numpy: a NaN anywhere makes them NaN.
// Rounding is monotone, so amax of (image - amin) is fl(max - amin).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t ord_key(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__device__ __forceinline__ float ord_value(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

template <typename T>
__device__ __forceinline__ float to_f32(T v) {
  return (float)v;  // exact for 8/16-bit integers and float
}
template <>
__device__ __forceinline__ float to_f32<int32_t>(int32_t v) {
  return __int2float_rn(v);
}

template <typename T>
__global__ void __launch_bounds__(256) geo_convert_minmax_kernel(const T* __restrict__ img, uint64_t n,
                                                                 float* __restrict__ out, uint32_t* mm) {
  uint32_t lo = 0xffffffffu, hi = 0u, nan = 0u;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float f = to_f32(img[i]);
    out[i] = f;
    if (f != f) {
      nan = 1u;
    } else {
      const uint32_t k = ord_key(f);
      lo = k < lo ? k : lo;
      hi = k > hi ? k : hi;
    }
  }
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  nan = __reduce_or_sync(0xffffffffu, nan);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&mm[0], lo);
    atomicMax(&mm[1], hi);
    if (nan) atomicOr(&mm[2], 1u);
  }
}

__global__ void geo_minmax_init_kernel(uint32_t* mm) {
  if (threadIdx.x == 0) {
    mm[0] = 0xffffffffu;
    mm[1] = 0u;
    mm[2] = 0u;
  }
}

__global__ void __launch_bounds__(256) geo_normalize_kernel(float* __restrict__ out, uint64_t n,
                                                            const uint32_t* __restrict__ mm) {
  float mn = ord_value(mm[0]);
  float amax = __fsub_rn(ord_value(mm[1]), mn);
  // numpy: NaN in the image, or an infinite minimum (inf - inf inside image - amin), gives NaN everywhere
  if (mm[2] || isinf(mn)) {
    mn = __uint_as_float(0x7fffffffu);
    amax = mn;
  }
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = __fdiv_rn(__fsub_rn(out[i], mn), amax);
}

// mask.fill(inf); mask[labels == label] = 0 for every label slot at once
// (geodis.py:95-96). slot_lut[v] = slot of label value v (0..255) or -1.
template <typename T>
__global__ void __launch_bounds__(256) geo_masks_kernel(const T* __restrict__ lab, uint64_t n,
                                                        const int16_t* __restrict__ slot_lut, int nol,
                                                        float* __restrict__ c) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int v = (int)lab[i];
    const int s = (v >= 0 && v <= 255) ? (int)slot_lut[v] : -1;
    for (int k = 0; k < nol; ++k) c[(uint64_t)k * n + i] = (s == k) ? 0.0f : __uint_as_float(0x7f800000u);
  }
}

// The label loop of geodis.py:94-103: slot 0 only initialises the running
// minimum (its voxels keep result 0); a later slot wins where its distance is
// strictly smaller.
__global__ void __launch_bounds__(256) geo_select_kernel(const float* __restrict__ c, int nol, uint64_t n,
                                                         const uint8_t* __restrict__ slot_label,
                                                         uint8_t* __restrict__ out) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    float m = c[i];
    uint8_t r = 0;
    for (int k = 1; k < nol; ++k) {
      const float d = c[(uint64_t)k * n + i];
      if (d < m) {
        m = d;
        r = slot_label[k];
      }
    }
    out[i] = r;
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

extern "C" int si_geo_normalize(const void* img, int dtype, uint64_t n, float* out, uint32_t* mm, void* stream) {
  clear_error();
  if (!img || !out || !mm) return set_error(SI_ERR_ARG, "si_geo_normalize: null pointer");
  if (n == 0) return set_error(SI_ERR_ARG, "si_geo_normalize: empty image (numpy's amin has no identity)");
  if (dtype_size(dtype) == 0) return set_error(SI_ERR_ARG, "si_geo_normalize: unsupported image dtype %d", dtype);
  cudaStream_t st = as_stream(stream);
  geo_minmax_init_kernel<<<1, 32, 0, st>>>(mm);
  const int block = 256, grid = grid_for(n, block);
  switch (dtype) {
    case SI_U8:
      geo_convert_minmax_kernel<<<grid, block, 0, st>>>(static_cast<const uint8_t*>(img), n, out, mm);
      break;
    case SI_I8:
      geo_convert_minmax_kernel<<<grid, block, 0, st>>>(static_cast<const int8_t*>(img), n, out, mm);
      break;
    case SI_U16:
      geo_convert_minmax_kernel<<<grid, block, 0, st>>>(static_cast<const uint16_t*>(img), n, out, mm);
      break;
    case SI_I16:
      geo_convert_minmax_kernel<<<grid, block, 0, st>>>(static_cast<const int16_t*>(img), n, out, mm);
      break;
    case SI_I32:
      geo_convert_minmax_kernel<<<grid, block, 0, st>>>(static_cast<const int32_t*>(img), n, out, mm);
      break;
    case SI_F32:
      geo_convert_minmax_kernel<<<grid, block, 0, st>>>(static_cast<const float*>(img), n, out, mm);
      break;
    default:
      return set_error(SI_ERR_ARG, "si_geo_normalize: unsupported image dtype %d", dtype);
  }
  geo_normalize_kernel<<<grid, block, 0, st>>>(out, n, mm);
  return check_launch("si_geo_normalize");
}

extern "C" int si_geo_masks(const void* labels, int dtype, uint64_t n, const int16_t* slot_lut, int nol, float* c,
                            void* stream) {
  clear_error();
  if (!labels || !slot_lut || !c) return set_error(SI_ERR_ARG, "si_geo_masks: null pointer");
  if (nol < 1 || nol > 256) return set_error(SI_ERR_ARG, "si_geo_masks: nol must be 1..256");
  if (n == 0) return SI_OK;
  const int block = 256, grid = grid_for(n, block);
  cudaStream_t st = as_stream(stream);
  switch (dtype) {
    case SI_U8:
      geo_masks_kernel<<<grid, block, 0, st>>>(static_cast<const uint8_t*>(labels), n, slot_lut, nol, c);
      break;
    case SI_I16:
      geo_masks_kernel<<<grid, block, 0, st>>>(static_cast<const int16_t*>(labels), n, slot_lut, nol, c);
      break;
    case SI_I32:
      geo_masks_kernel<<<grid, block, 0, st>>>(static_cast<const int32_t*>(labels), n, slot_lut, nol, c);
      break;
    default:
      return set_error(SI_ERR_ARG, "si_geo_masks: unsupported label dtype %d", dtype);
  }
  return check_launch("si_geo_masks");
}

namespace si {
namespace {

// Clusters of the scan kernel that fit on the current device at once (0 if
// the cluster launch is not possible), cached per device.
int geo_cluster_capacity(bool lamb1) {
  static std::atomic<int> cache[2][64];  // capacity + 1; 0 = not yet queried
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  const int known = cache[lamb1][dev].load(std::memory_order_relaxed);
  if (known) return known - 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kGeoCluster);
  cfg.blockDim = dim3(kGeoClusterThreads);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kGeoCluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  const cudaError_t e =
      lamb1 ? cudaOccupancyMaxActiveClusters(&n, geo_cluster_scan_kernel<true>, &cfg)
            : cudaOccupancyMaxActiveClusters(&n, geo_cluster_scan_kernel<false>, &cfg);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    n = 0;
  }
  cache[lamb1][dev].store(n + 1, std::memory_order_relaxed);
  return n;
}

// Largest wavefront of either pass (voxels of one label).
long long geo_max_wave(int Z, int Y, int X) {
  long long m = 0;
  for (int fwd = 1; fwd >= 0; --fwd) {
    int t0, t1, step;
    geo_t_range(Z, Y, X, fwd, &t0, &t1, &step);
    for (int t = t0; step > 0 ? t <= t1 : t >= t1; t += step) {
      const GeoWave w = geo_wave(Z, Y, X, fwd, t);
      const long long n = (long long)w.nz * w.jmax;
      m = n > m ? n : m;
    }
  }
  return m;
}

// Scan mode of one call: the cluster scan (mode 2) or wavefront launches.
int geo_resolve_mode(int Z, int Y, int X, bool lamb1, int mode, bool* cluster) {
  const long long max_wave = geo_max_wave(Z, Y, X);
  if (max_wave >= 0x7fffffffLL) return set_error(SI_ERR_LIMIT, "si_geo_scan: wavefront too large");
  if (mode == 2 && geo_cluster_capacity(lamb1) < 1)
    return set_error(SI_ERR_CUDA, "si_geo_scan: a cluster of %d CTAs x %d threads cannot be launched here",
                     kGeoCluster, kGeoClusterThreads);
  *cluster = (mode == 2);
  return SI_OK;
}

// Opt-in shared memory of the tiled kernel (once per device, outside any capture).
int geo_tile_prepare() {
  static std::atomic<bool> done[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return check_launch("si_geo_scan (device)");
  if (done[dev].load(std::memory_order_acquire)) return SI_OK;
  if (cudaFuncSetAttribute(geo_tile_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTileSmem) !=
          cudaSuccess ||
      cudaFuncSetAttribute(geo_tile_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTileSmem) !=
          cudaSuccess)
    return check_launch("si_geo_scan (tile shared memory)");
  done[dev].store(true, std::memory_order_release);
  return SI_OK;
}

// All launches of a scan, in order, on stream st: one per tile-wavefront
// (tiled) or one per wavefront.
int geo_launch_scan(const GeoScanArgs& a, bool lamb1, int iterations, bool tiled, cudaStream_t st) {
  if (tiled) {
    for (int it = 0; it < iterations; ++it)
      for (int fwd = 1; fwd >= 0; --fwd) {
        const GeoTiling g = geo_tiling(a.Z, a.Y, a.X, fwd);
        const long long ncta = (long long)g.ntq * g.ntr;
        if (ncta > 0x7fffffffLL) return set_error(SI_ERR_LIMIT, "si_geo_scan: too many tiles");
        const dim3 grid((unsigned)ncta, (unsigned)a.nol);
        for (int S = 0; S <= g.ntp + g.ntq + g.ntr - 3; ++S) {
          if (lamb1)
            geo_tile_kernel<true><<<grid, kTileThreads, kTileSmem, st>>>(a, g, S);
          else
            geo_tile_kernel<false><<<grid, kTileThreads, kTileSmem, st>>>(a, g, S);
        }
      }
    return SI_OK;
  }
  const int block = 256;
  for (int it = 0; it < iterations; ++it) {
    for (int fwd = 1; fwd >= 0; --fwd) {
      int t0, t1, step;
      geo_t_range(a.Z, a.Y, a.X, fwd, &t0, &t1, &step);
      for (int t = t0; step > 0 ? t <= t1 : t >= t1; t += step) {
        const GeoWave w = geo_wave(a.Z, a.Y, a.X, fwd, t);
        if (w.nz == 0) continue;
        const long long threads = (long long)w.nz * w.jmax * a.nol;
        const long long blocks = (threads + block - 1) / block;
        if (blocks > 0x7fffffffLL) return set_error(SI_ERR_LIMIT, "si_geo_scan: wavefront too large");
        if (lamb1)
          geo_wave_kernel<true><<<(unsigned)blocks, block, 0, st>>>(a, w, fwd);
        else
          geo_wave_kernel<false><<<(unsigned)blocks, block, 0, st>>>(a, w, fwd);
      }
    }
  }
  return SI_OK;
}

// Instantiated CUDA graphs of whole scans (the wavefront launches of one
// call, parameters included), keyed by every argument that enters them.
// Mode 0 captures a scan the second time the same arguments come; mode 3 the
// first time. At most kGeoGraphs graphs are kept (least recently used go).
struct GeoGraphKey {
  int dev;
  const float* c;
  const float* img;
  int Z, Y, X, nol, iterations, tiled;
  double lamb;
  bool operator==(const GeoGraphKey& o) const {
    return dev == o.dev && c == o.c && img == o.img && Z == o.Z && Y == o.Y && X == o.X && nol == o.nol &&
           iterations == o.iterations && tiled == o.tiled && lamb == o.lamb;
  }
};

struct GeoGraph {
  GeoGraphKey key;
  cudaGraphExec_t exec;
  unsigned long long used;
};

constexpr size_t kGeoGraphs = 8;
constexpr size_t kGeoSeen = 64;
std::mutex g_geo_mu;
std::vector<GeoGraph> g_geo_graphs;
std::vector<GeoGraphKey> g_geo_seen;
unsigned long long g_geo_clock = 0;
cudaStream_t g_geo_capture[64];

// Runs the scan through a cached graph; *done = false when the caller should
// launch the wavefronts directly (mode 0, first call with these arguments).
int geo_scan_graph(const GeoScanArgs& a, bool lamb1, int iterations, bool tiled, bool capture_first,
                   cudaStream_t st, bool* done) {
  *done = false;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return SI_OK;
  const GeoGraphKey key{dev, a.c, a.img, a.Z, a.Y, a.X, a.nol, iterations, tiled ? 1 : 0, a.lamb};
  std::lock_guard<std::mutex> lock(g_geo_mu);
  for (GeoGraph& g : g_geo_graphs)
    if (g.key == key) {
      g.used = ++g_geo_clock;
      if (cudaGraphLaunch(g.exec, st) != cudaSuccess) return check_launch("si_geo_scan (graph launch)");
      *done = true;
      return SI_OK;
    }
  if (!capture_first) {
    bool seen = false;
    for (const GeoGraphKey& k : g_geo_seen) seen = seen || (k == key);
    if (!seen) {
      if (g_geo_seen.size() >= kGeoSeen) g_geo_seen.erase(g_geo_seen.begin());
      g_geo_seen.push_back(key);
      return SI_OK;
    }
  }
  if (!g_geo_capture[dev] && cudaStreamCreateWithFlags(&g_geo_capture[dev], cudaStreamNonBlocking) != cudaSuccess)
    return check_launch("si_geo_scan (capture stream)");
  cudaStream_t cs = g_geo_capture[dev];
  if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return check_launch("si_geo_scan (begin capture)");
  const int rc = geo_launch_scan(a, lamb1, iterations, tiled, cs);
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(cs, &graph);
  if (rc || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    (void)cudaGetLastError();
    return rc ? rc : set_error(SI_ERR_CUDA, "si_geo_scan: capture failed: %s", cudaGetErrorString(e));
  }
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess) {
    (void)cudaGetLastError();
    return set_error(SI_ERR_CUDA, "si_geo_scan: graph instantiation failed: %s", cudaGetErrorString(ei));
  }
  if (g_geo_graphs.size() >= kGeoGraphs) {
    size_t old = 0;
    for (size_t i = 1; i < g_geo_graphs.size(); ++i)
      if (g_geo_graphs[i].used < g_geo_graphs[old].used) old = i;
    cudaGraphExecDestroy(g_geo_graphs[old].exec);  // an in-flight graph is freed when it completes
    g_geo_graphs.erase(g_geo_graphs.begin() + old);
  }
  g_geo_graphs.push_back(GeoGraph{key, exec, ++g_geo_clock});
  if (cudaGraphLaunch(exec, st) != cudaSuccess) return check_launch("si_geo_scan (graph launch)");
  *done = true;
  return SI_OK;
}

}  // namespace
}  // namespace si

extern "C" int si_geo_scan_launches(int Z, int Y, int X, double lamb, int iterations, int mode,
                                    long long* launches) {
  clear_error();
  if (!launches || Z < 1 || Y < 1 || X < 1 || iterations < 0 || mode < 0 || mode > 5)
    return set_error(SI_ERR_ARG, "si_geo_scan_launches: bad arguments");
  *launches = 0;
  if (!geo_has_interior(Z, Y, X) || iterations == 0) return SI_OK;
  bool cluster = false;
  const int rc = geo_resolve_mode(Z, Y, X, lamb == 1.0, mode, &cluster);
  if (rc) return rc;
  if (cluster) {
    *launches = 1;
    return SI_OK;
  }
  long long n = 0;
  for (int fwd = 1; fwd >= 0; --fwd) {
    if (mode == 0 || mode == 4 || mode == 5) {
      const GeoTiling g = geo_tiling(Z, Y, X, fwd);
      n += g.ntp + g.ntq + g.ntr - 2;
      continue;
    }
    int t0, t1, step;
    geo_t_range(Z, Y, X, fwd, &t0, &t1, &step);
    for (int t = t0; step > 0 ? t <= t1 : t >= t1; t += step) n += geo_wave(Z, Y, X, fwd, t).nz > 0;
  }
  *launches = n * iterations;
  return SI_OK;
}

extern "C" int si_geo_scan(float* c, const float* img, int Z, int Y, int X, int nol, double lamb, int iterations,
                           int mode, void* stream) {
  clear_error();
  if (!c || !img) return set_error(SI_ERR_ARG, "si_geo_scan: null pointer");
  if (Z < 1 || Y < 1 || X < 1 || nol < 1 || iterations < 0 || mode < 0 || mode > 5)
    return set_error(SI_ERR_ARG, "si_geo_scan: bad arguments");
  if ((long long)X + 2LL * Y + 4LL * Z > 0x7fffffffLL) return set_error(SI_ERR_LIMIT, "si_geo_scan: volume too large");
  if (!geo_has_interior(Z, Y, X) || iterations == 0) return SI_OK;
  GeoScanArgs a{};
  a.c = c;
  a.img = img;
  a.Z = Z;
  a.Y = Y;
  a.X = X;
  a.nol = nol;
  a.V = (long long)Z * Y * X;
  a.lamb = lamb;
  const long long YX = (long long)Y * X;
  for (int n = 0; n < 13; ++n) {
    a.off[n] = kGeoOff[n][0] * YX + (long long)kGeoOff[n][1] * X + kGeoOff[n][2];
    a.box_off[n] = geo_box_offset(n);
    const int nzc = (kGeoOff[n][0] != 0) + (kGeoOff[n][1] != 0) + (kGeoOff[n][2] != 0);
    const double d = nzc == 3 ? std::sqrt(3.0) : nzc == 2 ? std::sqrt(2.0) : 1.0;
    a.w[n] = (1.0 - lamb) * d;
  }
  const bool lamb1 = (lamb == 1.0);
  cudaStream_t st = as_stream(stream);
  bool cluster = false;
  const int rc_mode = geo_resolve_mode(Z, Y, X, lamb1, mode, &cluster);
  if (rc_mode) return rc_mode;
  if (cluster) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(kGeoCluster * nol));
    cfg.blockDim = dim3(kGeoClusterThreads);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kGeoCluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = lamb1 ? cudaLaunchKernelEx(&cfg, geo_cluster_scan_kernel<true>, a, iterations)
                                : cudaLaunchKernelEx(&cfg, geo_cluster_scan_kernel<false>, a, iterations);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return set_error(SI_ERR_CUDA, "si_geo_scan: cluster launch failed: %s", cudaGetErrorString(e));
    }
    return check_launch("si_geo_scan");
  }
  const bool tiled = (mode == 0 || mode == 4 || mode == 5);
  if (tiled) {
    const int rc = geo_tile_prepare();
    if (rc) return rc;
  }
  if (mode == 0 || mode == 3 || mode == 5) {
    bool done = false;
    const int rc = geo_scan_graph(a, lamb1, iterations, tiled, mode != 0, st, &done);
    if (rc || done) return rc;
  }
  const int rc = geo_launch_scan(a, lamb1, iterations, tiled, st);
  return rc ? rc : check_launch("si_geo_scan");
}

extern "C" int si_geo_select(const float* c, int nol, uint64_t n, const uint8_t* slot_label, uint8_t* out,
                             void* stream) {
  clear_error();
  if (!c || !slot_label || !out) return set_error(SI_ERR_ARG, "si_geo_select: null pointer");
  if (nol < 1 || nol > 256) return set_error(SI_ERR_ARG, "si_geo_select: nol must be 1..256");
  if (n == 0) return SI_OK;
  const int block = 256, grid = grid_for(n, block);
  geo_select_kernel<<<grid, block, 0, as_stream(stream)>>>(c, nol, n, slot_label, out);
  return check_launch("si_geo_select");
}

extern "C" int si_geo_visit_order(int Z, int Y, int X, int fwd, int32_t* t_of_voxel) {
  clear_error();
  if (!t_of_voxel || Z < 1 || Y < 1 || X < 1) return set_error(SI_ERR_ARG, "si_geo_visit_order: bad arguments");
  const long long V = (long long)Z * Y * X;
  for (long long v = 0; v < V; ++v) t_of_voxel[v] = -1;
  if (!geo_has_interior(Z, Y, X)) return SI_OK;
  int t0, t1, step;
  geo_t_range(Z, Y, X, fwd ? 1 : 0, &t0, &t1, &step);
  for (int t = t0; step > 0 ? t <= t1 : t >= t1; t += step) {
    const GeoWave w = geo_wave(Z, Y, X, fwd ? 1 : 0, t);
    for (int zi = 0; zi < w.nz; ++zi)
      for (int j = 0; j < w.jmax; ++j) {
        int z, y, x;
        if (!geo_wave_voxel(Y, X, w, zi, j, &z, &y, &x)) continue;
        if (z < 0 || z >= Z || y < 0 || y >= Y || x < 0 || x >= X)
          return set_error(SI_ERR_LIMIT, "si_geo_visit_order: voxel (%d,%d,%d) outside the volume", z, y, x);
        const long long v = ((long long)z * Y + y) * X + x;
        if (t_of_voxel[v] != -1)
          return set_error(SI_ERR_LIMIT, "si_geo_visit_order: voxel (%d,%d,%d) visited twice", z, y, x);
        t_of_voxel[v] = t;
      }
  }
  return SI_OK;
}

extern "C" int si_geo_tile_visit_order(int Z, int Y, int X, int fwd, int32_t* wave, int32_t* tile, int32_t* step) {
  clear_error();
  if (!wave || !tile || !step || Z < 1 || Y < 1 || X < 1)
    return set_error(SI_ERR_ARG, "si_geo_tile_visit_order: bad arguments");
  const long long V = (long long)Z * Y * X;
  for (long long v = 0; v < V; ++v) wave[v] = tile[v] = step[v] = -1;
  if (!geo_has_interior(Z, Y, X)) return SI_OK;
  const GeoTiling g = geo_tiling(Z, Y, X, fwd ? 1 : 0);
  for (int S = 0; S <= g.ntp + g.ntq + g.ntr - 3; ++S)
    for (int ir = 0; ir < g.ntr; ++ir)
      for (int iq = 0; iq < g.ntq; ++iq) {
        const int ip = S - iq - ir;
        if (ip < 0 || ip >= g.ntp) continue;
        const int p0 = g.pb + ip * kTileP - 7, q0 = g.qb + iq * kTileQ - 3, r0 = g.rb + ir * kTileR - 1;
        for (int cr = 0; cr < kTileR; ++cr)
          for (int cq = 0; cq < kTileQ; ++cq)
            for (int k = 0; k < kTileP; ++k) {
              int z, y, x;
              if (!geo_tile_voxel(g, Y, X, ip, iq, ir, cq, cr, k, &z, &y, &x)) continue;
              const long long v = ((long long)z * Y + y) * X + x;
              if (wave[v] != -1)
                return set_error(SI_ERR_LIMIT, "si_geo_tile_visit_order: voxel (%d,%d,%d) visited twice", z, y, x);
              wave[v] = S;
              tile[v] = (ip * g.ntr + ir) * g.ntq + iq;
              step[v] = k;
              // every neighbour the kernel reads: inside the box, and the voxel the scan reads
              const int own = geo_box_cell(k + 7, cq + 3, cr + 1);
              for (int n = 0; n < 13; ++n) {
                const int cell = own + geo_box_offset(n);
                if (cell < 0 || cell >= kBoxCells)
                  return set_error(SI_ERR_LIMIT, "si_geo_tile_visit_order: neighbour %d outside the box", n);
                const int bp = cell % kBoxP, bq = (cell / kBoxP) % kBoxQ, br = cell / (kBoxP * kBoxQ);
                int nz, ny, nx;
                geo_unskew(g, p0 + bp, q0 + bq, r0 + br, &nz, &ny, &nx);
                const int sg = fwd ? 1 : -1;
                if (nz != z + sg * kGeoOff[n][0] || ny != y + sg * kGeoOff[n][1] || nx != x + sg * kGeoOff[n][2])
                  return set_error(SI_ERR_LIMIT, "si_geo_tile_visit_order: box neighbour %d is not the scan's", n);
              }
            }
      }
  return SI_OK;
}
