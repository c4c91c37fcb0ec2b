// Post-walk kernels: per-voxel argmax (+ optional uncertainty), label remap
// and curvature smoothing.
#include "si_common.cuh"
#include "si_internal.h"

namespace si {
namespace {

struct PostGeom {
  int Zc, Yc, Xc;
  int cz0, cy0, cx0;
  int Z0, Y0, X0;
};

// ---------------------------------------------------------------------------
// argmax over labels, ties -> lowest index (np.argmax, rw_small.py:200), fused
// with the top-3 uncertainty of gpu_kernels.py:54-116 (strict '>' updates in
// label order; uq = 1 - (1 - m0/m2)(1 - m1/m2), m2 == 0 -> 1; then
// uint8(uq * 255) as rw_small.py:172). Crop-border voxels get uq = 0 (the
// reference leaves the last label's hit count there, which is always 0 on the
// border because walkers never enter it).
// ---------------------------------------------------------------------------
template <bool kFloat>
__global__ void __launch_bounds__(256) argmax_kernel(const void* __restrict__ maps_v, int nol, PostGeom g,
                                                     uint8_t* __restrict__ out, uint32_t* __restrict__ presence,
                                                     uint8_t* __restrict__ uq) {
  const size_t F = (size_t)g.Yc * g.Xc;
  const size_t V = F * g.Zc;
  uint32_t pres_lo = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < V; i += stride) {
    const int xc = (int)(i % g.Xc);
    const uint64_t zy = i / g.Xc;
    const int yc = (int)(zy % g.Yc);
    const int zc = (int)(zy / g.Yc);
    int idx = 0;
    float m0 = 0.0f, m1 = 0.0f, m2 = 0.0f;
    if (kFloat) {
      const float* m = static_cast<const float*>(maps_v);
      float best = m[i];
      for (int l = 1; l < nol; ++l) {
        const float v = m[(size_t)l * V + i];
        if (v > best) {
          best = v;
          idx = l;
        }
      }
    } else {
      const uint32_t* m = static_cast<const uint32_t*>(maps_v);
      uint32_t best = m[i];
      if (uq) m2 = __uint2float_rn(best);
      for (int l = 1; l < nol; ++l) {
        const uint32_t v = m[(size_t)l * V + i];
        if (v > best) {
          best = v;
          idx = l;
        }
        if (uq) {
          const float tmp = __uint2float_rn(v);
          if (tmp > m2) {
            m0 = m1; m1 = m2; m2 = tmp;
          } else if (tmp > m1) {
            m0 = m1; m1 = tmp;
          } else if (tmp > m0) {
            m0 = tmp;
          }
        }
      }
    }
    if (idx < 32)
      pres_lo |= 1u << idx;
    else
      atomicOr(&presence[idx >> 5], 1u << (idx & 31));
    const int oz = zc + g.cz0 - 1, oy = yc + g.cy0 - 1, ox = xc + g.cx0 - 1;
    if ((unsigned)oz < (unsigned)g.Z0 && (unsigned)oy < (unsigned)g.Y0 && (unsigned)ox < (unsigned)g.X0) {
      const size_t o = ((size_t)oz * g.Y0 + oy) * g.X0 + ox;
      out[o] = (uint8_t)idx;
      if (uq) {
        uint8_t q = 0;
        if (zc > 0 && yc > 0 && xc > 0 && zc < g.Zc - 1 && yc < g.Yc - 1 && xc < g.Xc - 1) {
          const float mx = m2 == 0.0f ? 1.0f : m2;
          const float t0 = __fdiv_rn(m0, mx);
          const float t1 = __fdiv_rn(m1, mx);
          const float a = __fsub_rn(1.0f, __fmul_rn(__fsub_rn(1.0f, t0), __fsub_rn(1.0f, t1)));
          q = (uint8_t)(int)__fmul_rn(a, 255.0f);
        }
        uq[o] = q;
      }
    }
  }
  pres_lo = __reduce_or_sync(0xffffffffu, pres_lo);
  if ((threadIdx.x & 31) == 0 && pres_lo) atomicOr(&presence[0], pres_lo);
}

// The first label in the uncertainty top-3 is seeded from map 0 above
// (m2 = value of label 0 when it is > 0), exactly what the sequential update
// gives for the first label since m0 = m1 = m2 = 0 before it.

// ---------------------------------------------------------------------------
// get_labels (biomedisa_helper.py:1209-1213): index k -> all_labels[k] for
// every index present except the smallest one present, which stays 0.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) remap_kernel(uint8_t* __restrict__ out, PostGeom g,
                                                    const uint32_t* __restrict__ presence,
                                                    const uint8_t* __restrict__ all_labels, int nol) {
  __shared__ uint8_t lut[256];
  __shared__ int kmin;
  if (threadIdx.x == 0) {
    kmin = 256;
    for (int w = 0; w < 8 && kmin == 256; ++w)
      if (presence[w]) kmin = w * 32 + __ffs(presence[w]) - 1;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < 256; k += blockDim.x) lut[k] = (k < nol && k != kmin) ? all_labels[k] : 0;
  __syncthreads();
  // crop region intersected with the original frame
  const int z0 = max(g.cz0 - 1, 0), z1 = min(g.cz0 - 1 + g.Zc, g.Z0);
  const int y0 = max(g.cy0 - 1, 0), y1 = min(g.cy0 - 1 + g.Yc, g.Y0);
  const int x0 = max(g.cx0 - 1, 0), x1 = min(g.cx0 - 1 + g.Xc, g.X0);
  if (z1 <= z0 || y1 <= y0 || x1 <= x0) return;
  const int nx = x1 - x0, ny = y1 - y0;
  const uint64_t n = (uint64_t)(z1 - z0) * ny * nx;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int x = x0 + (int)(i % nx);
    const uint64_t zy = i / nx;
    const int y = y0 + (int)(zy % ny);
    const int z = z0 + (int)(zy / ny);
    const size_t o = ((size_t)z * g.Y0 + y) * g.X0 + x;
    out[o] = lut[out[o]];
  }
}

// ---------------------------------------------------------------------------
// Curvature smoothing step (gpu_kernels.py:118-183): on interior voxels
//   dst = phi + 0.01 * kappa(phi), kappa the level-set mean-curvature term
// with central differences (sign convention x-1 minus x+1 as in the
// reference); border voxels copy phi. Every operation is a binary32
// round-to-nearest operation in the order of the reference expression;
// /2.0 and /4.0 are exact scalings.
// ---------------------------------------------------------------------------
template <bool kSrcU32>
__device__ __forceinline__ float ld(const void* p, size_t i) {
  if (kSrcU32) return __uint2float_rn(static_cast<const uint32_t*>(p)[i]);
  return static_cast<const float*>(p)[i];
}

// 2.5-D tiled smoothing step: a 32x8 tile of threads marches
// along z over a chunk of planes, keeping planes z-1, z, z+1 of the tile plus a
// one-voxel halo in shared memory, so every value is read from global memory
// about 1.3 times per iteration instead of being gathered 19 times.
constexpr int kTX = 32, kTY = 8, kZChunk = 16;

template <bool kSrcU32>
__global__ void __launch_bounds__(kTX * kTY) smooth_tile_kernel(const void* __restrict__ src, float* __restrict__ dst,
                                                               int Zc, int Yc, int Xc) {
  __shared__ float pl[3][kTY + 2][kTX + 2];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY;
  const int zb = blockIdx.z * kZChunk;
  const int ze = min(zb + kZChunk, Zc);
  const size_t X = (size_t)Xc, F = (size_t)Yc * Xc;
  const int x = x0 + tx, y = y0 + ty;
  const int tid = ty * kTX + tx;
  // Each thread fills at most two halo-tile entries per plane; their tile and
  // in-plane offsets are fixed for the whole z-loop (kLoads: ceil(340 / 256)).
  constexpr int kTile = (kTY + 2) * (kTX + 2), kLoads = (kTile + kTX * kTY - 1) / (kTX * kTY);
  int tile_idx[kLoads];
  int64_t plane_off[kLoads];  // -1: outside the plane (or no entry)
#pragma unroll
  for (int k = 0; k < kLoads; ++k) {
    const int i = tid + k * kTX * kTY;
    tile_idx[k] = i;
    plane_off[k] = -1;
    if (i < kTile) {
      const int ly = i / (kTX + 2), lx = i - ly * (kTX + 2);
      const int gy = y0 + ly - 1, gx = x0 + lx - 1;
      if (gy >= 0 && gy < Yc && gx >= 0 && gx < Xc) plane_off[k] = (int64_t)gy * X + gx;
    }
  }
  // loads plane z (zero outside the volume; such values are never used) into
  // slot sidx and returns the OR of the bit patterns this thread stored
  auto load_plane = [&](int z, int sidx) -> uint32_t {
    float* dstp = &pl[sidx][0][0];
    const bool zin = z >= 0 && z < Zc;
    uint32_t orv = 0u;
#pragma unroll
    for (int k = 0; k < kLoads; ++k) {
      if (tile_idx[k] < kTile) {
        const float v = (zin && plane_off[k] >= 0) ? ld<kSrcU32>(src, (size_t)z * F + (size_t)plane_off[k]) : 0.0f;
        dstp[tile_idx[k]] = v;
        orv |= __float_as_uint(v);
      }
    }
    return orv;
  };
  // A plane flag is set when any value of the tile's (halo) plane is not +0.0.
  // When the three planes around z are all +0.0, every stencil of the tile
  // is +0 and stays exactly +0 (all differences 0, num = +0, +0 / (0 + 1e-10)
  // = +0), so the block writes the centre values and skips the arithmetic;
  // hit maps are +0 far from their label's region.
  int nzm = __syncthreads_or(load_plane(zb - 1, 0) != 0u);
  int nz0 = __syncthreads_or(load_plane(zb, 1) != 0u);
  int sm = 0, s0 = 1, sp = 2;
  for (int z = zb; z < ze; ++z) {
    const int nzp = __syncthreads_or(load_plane(z + 1, sp) != 0u);
    const bool quiet = !(nzm | nz0 | nzp);
    const int lx = tx + 1, ly = ty + 1;
    const bool inside = x < Xc && y < Yc;
    const bool interior = inside && z > 0 && y > 0 && x > 0 && z < Zc - 1 && y < Yc - 1 && x < Xc - 1;
    if (inside) {
      const float c = pl[s0][ly][lx];
      const size_t i = (size_t)z * F + (size_t)y * X + x;
      if (quiet || !interior) {
        dst[i] = c;
      } else {
        const float c2 = __fmul_rn(2.0f, c);
        const float xm = pl[s0][ly][lx - 1], xp = pl[s0][ly][lx + 1];
        const float ym = pl[s0][ly - 1][lx], yp = pl[s0][ly + 1][lx];
        const float zm = pl[sm][ly][lx], zp = pl[sp][ly][lx];
        const float dx = __fmul_rn(__fsub_rn(xm, xp), 0.5f);
        const float dxx = __fadd_rn(__fsub_rn(xm, c2), xp);
        const float dx2 = __fmul_rn(dx, dx);
        const float dy = __fmul_rn(__fsub_rn(ym, yp), 0.5f);
        const float dyy = __fadd_rn(__fsub_rn(ym, c2), yp);
        const float dy2 = __fmul_rn(dy, dy);
        const float dz = __fmul_rn(__fsub_rn(zm, zp), 0.5f);
        const float dzz = __fadd_rn(__fsub_rn(zm, c2), zp);
        const float dz2 = __fmul_rn(dz, dz);
        const float dxy = __fmul_rn(
            __fsub_rn(__fsub_rn(__fadd_rn(pl[s0][ly - 1][lx - 1], pl[s0][ly + 1][lx + 1]), pl[s0][ly - 1][lx + 1]),
                      pl[s0][ly + 1][lx - 1]),
            0.25f);
        const float dxz = __fmul_rn(
            __fsub_rn(__fsub_rn(__fadd_rn(pl[sp][ly][lx - 1], pl[sm][ly][lx + 1]), pl[sp][ly][lx + 1]),
                      pl[sm][ly][lx - 1]),
            0.25f);
        const float dyz = __fmul_rn(
            __fsub_rn(__fsub_rn(__fadd_rn(pl[sp][ly - 1][lx], pl[sm][ly + 1][lx]), pl[sp][ly + 1][lx]),
                      pl[sm][ly - 1][lx]),
            0.25f);
        float num = __fadd_rn(__fmul_rn(dxx, __fadd_rn(dy2, dz2)), __fmul_rn(dyy, __fadd_rn(dx2, dz2)));
        num = __fadd_rn(num, __fmul_rn(dzz, __fadd_rn(dx2, dy2)));
        num = __fsub_rn(num, __fmul_rn(__fmul_rn(__fmul_rn(2.0f, dx), dy), dxy));
        num = __fsub_rn(num, __fmul_rn(__fmul_rn(__fmul_rn(2.0f, dx), dz), dxz));
        num = __fsub_rn(num, __fmul_rn(__fmul_rn(__fmul_rn(2.0f, dy), dz), dyz));
        const float den = __fadd_rn(__fadd_rn(__fadd_rn(dx2, dy2), dz2), 1e-10f);
        dst[i] = __fadd_rn(c, __fmul_rn(0.01f, __fdiv_rn(num, den)));
      }
    }
    __syncthreads();
    const int t = sm;
    sm = s0;
    s0 = sp;
    sp = t;
    nzm = nz0;
    nz0 = nzp;
  }
}

__global__ void __launch_bounds__(256) u32_to_f32_kernel(const uint32_t* __restrict__ src, float* __restrict__ dst,
                                                         size_t n) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    dst[i] = __uint2float_rn(src[i]);
}

inline int grid_for(uint64_t n, int block) {
  const uint64_t want = (n + block - 1) / block;
  const uint64_t cap = (uint64_t)sm_count() * 16;
  return (int)(want < cap ? (want > 0 ? want : 1) : cap);
}

}  // namespace
}  // namespace si

using namespace si;

extern "C" int si_argmax(const void* maps, int maps_are_float, int nol, int Zc, int Yc, int Xc, int cz0, int cy0,
                         int cx0, int Z0, int Y0, int X0, uint8_t* out, uint32_t* presence, uint8_t* uq,
                         void* stream) {
  clear_error();
  if (!maps || !out || !presence) return set_error(SI_ERR_ARG, "si_argmax: null pointer");
  if (nol < 1 || nol > 256) return set_error(SI_ERR_ARG, "si_argmax: nol must be 1..256");
  if (Zc < 1 || Yc < 1 || Xc < 1 || Z0 < 1 || Y0 < 1 || X0 < 1) return set_error(SI_ERR_ARG, "si_argmax: bad dims");
  if (maps_are_float && uq) return set_error(SI_ERR_ARG, "si_argmax: uncertainty is computed from hit counts only");
  const PostGeom g{Zc, Yc, Xc, cz0, cy0, cx0, Z0, Y0, X0};
  const uint64_t n = (uint64_t)Zc * Yc * Xc;
  const int block = 256, grid = grid_for(n, block);
  cudaStream_t st = as_stream(stream);
  if (maps_are_float)
    argmax_kernel<true><<<grid, block, 0, st>>>(maps, nol, g, out, presence, nullptr);
  else
    argmax_kernel<false><<<grid, block, 0, st>>>(maps, nol, g, out, presence, uq);
  return check_launch("si_argmax");
}

extern "C" int si_remap_labels(uint8_t* out, int Zc, int Yc, int Xc, int cz0, int cy0, int cx0, int Z0, int Y0,
                               int X0, const uint32_t* presence, const uint8_t* all_labels, int nol, void* stream) {
  clear_error();
  if (!out || !presence || !all_labels) return set_error(SI_ERR_ARG, "si_remap_labels: null pointer");
  if (nol < 1 || nol > 256) return set_error(SI_ERR_ARG, "si_remap_labels: nol must be 1..256");
  const PostGeom g{Zc, Yc, Xc, cz0, cy0, cx0, Z0, Y0, X0};
  const uint64_t n = (uint64_t)Zc * Yc * Xc;
  const int block = 256, grid = grid_for(n, block);
  remap_kernel<<<grid, block, 0, as_stream(stream)>>>(out, g, presence, all_labels, nol);
  return check_launch("si_remap_labels");
}

extern "C" int si_smooth(uint32_t* maps, float* tmp0, float* tmp1, int nol, int Zc, int Yc, int Xc, int iters,
                         void* stream) {
  clear_error();
  if (!maps || !tmp0 || !tmp1) return set_error(SI_ERR_ARG, "si_smooth: null pointer");
  if (nol < 1 || nol > 256) return set_error(SI_ERR_ARG, "si_smooth: nol must be 1..256");
  if (Zc < 1 || Yc < 1 || Xc < 1 || iters < 0) return set_error(SI_ERR_ARG, "si_smooth: bad arguments");
  const size_t V = (size_t)Zc * Yc * Xc;
  const int block = 256, grid = grid_for(V, block);
  const dim3 tblock(kTX, kTY);
  const dim3 tgrid((Xc + kTX - 1) / kTX, (Yc + kTY - 1) / kTY, (Zc + kZChunk - 1) / kZChunk);
  cudaStream_t st = as_stream(stream);
  for (int l = 0; l < nol; ++l) {
    uint32_t* m = maps + (size_t)l * V;
    float* mf = reinterpret_cast<float*>(m);
    if (iters == 0) {
      u32_to_f32_kernel<<<grid, block, 0, st>>>(m, mf, V);
      continue;
    }
    // iteration 1 reads the uint32 hits; later ones ping-pong; the last one
    // writes into the map itself (its hits were consumed by iteration 1).
    float* bufs[2] = {tmp0, tmp1};
    const void* src = m;
    for (int it = 1; it <= iters; ++it) {
      float* dst = (it == iters && it > 1) ? mf : bufs[it & 1];
      if (it == 1)
        smooth_tile_kernel<true><<<tgrid, tblock, 0, st>>>(src, dst, Zc, Yc, Xc);
      else
        smooth_tile_kernel<false><<<tgrid, tblock, 0, st>>>(src, dst, Zc, Yc, Xc);
      src = dst;
    }
    if (iters == 1) {
      if (cudaMemcpyAsync(mf, src, V * sizeof(float), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return set_error(SI_ERR_CUDA, "si_smooth: copy failed");
    }
  }
  return check_launch("si_smooth");
}

extern "C" int si_smooth_f32(float* maps, float* tmp0, float* tmp1, int nol, int Zc, int Yc, int Xc, int iters,
                             void* stream) {
  clear_error();
  if (!maps || !tmp0 || !tmp1) return set_error(SI_ERR_ARG, "si_smooth_f32: null pointer");
  if (nol < 1 || nol > 256) return set_error(SI_ERR_ARG, "si_smooth_f32: nol must be 1..256");
  if (Zc < 1 || Yc < 1 || Xc < 1 || iters < 0) return set_error(SI_ERR_ARG, "si_smooth_f32: bad arguments");
  const size_t V = (size_t)Zc * Yc * Xc;
  const dim3 tblock(kTX, kTY);
  const dim3 tgrid((Xc + kTX - 1) / kTX, (Yc + kTY - 1) / kTY, (Zc + kZChunk - 1) / kZChunk);
  cudaStream_t st = as_stream(stream);
  for (int l = 0; l < nol && iters > 0; ++l) {
    float* m = maps + (size_t)l * V;
    float* bufs[2] = {tmp0, tmp1};
    const float* src = m;
    for (int it = 1; it <= iters; ++it) {
      float* dst = (it == iters && it > 1) ? m : bufs[it & 1];
      smooth_tile_kernel<false><<<tgrid, tblock, 0, st>>>(src, dst, Zc, Yc, Xc);
      src = dst;
    }
    if (iters == 1 && cudaMemcpyAsync(m, src, V * sizeof(float), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return set_error(SI_ERR_CUDA, "si_smooth_f32: copy failed");
  }
  return check_launch("si_smooth_f32");
}
