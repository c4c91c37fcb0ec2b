// Post-walk kernels: per-voxel argmax (+ optional uncertainty), label remap
// and curvature smoothing.
#include <algorithm>
#include <atomic>
#include <cstring>

#include "si_common.cuh"
#include "si_internal.h"
#include "si_tma.cuh"

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
// reference); border voxels copy phi. kappa is evaluated with binary32
// round-to-nearest operations in the order of the reference expression
// (/2.0 and /4.0 are exact scalings). The update is either binary32
// (phi + RN(0.01f * kappa), the default) or the reference's own arithmetic:
// `phi += 0.01 * curvature` multiplies by the binary64 literal 0.01 and adds
// in binary64 before the store rounds to binary32 (gpu_kernels.py:133).
//
// Layout: the source of every step is a pitched float32 volume (row pitch
// Xp = Xc rounded up to 4, so that rows start on 16 bytes), read by TMA
// tensor copies; the destination may have any row pitch.
//
// Schedule: a CTA of 256 threads owns a 64 x 8 column of voxels and marches
// through kSZ planes in z. Planes arrive in a ring of four shared-memory slots
// by TMA (one 72 x 10 box per plane: x from x0 - 4 so the copy starts on 16
// bytes, y from y0 - 1; out-of-volume parts read as zero), issued by one
// thread two planes ahead of use and completed on per-slot mbarriers. Each
// thread computes voxels x0 + tx and x0 + 32 + tx of its row as one pair on
// the packed binary32 pipe (add/sub/mul.rn.f32x2: per lane the same IEEE
// operation as the scalar form). Of the 19 stencil values a voxel needs, the
// 10 of planes z-1 and z are carried in registers from the previous plane, so
// a plane step loads 9 values per voxel from shared memory.
//
// Support box: values outside the box of non-(+0) source values grown by
// one voxel per iteration are exactly +0 (all differences +0, kappa =
// +0 / (0 + 1e-10) = +0, phi + 0.01 * 0 = +0), so CTAs whose column lies
// outside it do nothing (or write zeros, when their destination may hold
// older values).
// ---------------------------------------------------------------------------
// kP packed pairs per thread: the CTA's column is 64 * kP voxels wide
// (voxels x0 + tx + 32 j, j < 2 kP; pair p = columns 2p and 2p + 1).
constexpr int kSY = 8, kSZ = 32;
template <int kP>
struct SmoothTile {
  static constexpr int kSX = 64 * kP;
  static constexpr int kBoxX = kSX + 8, kBoxY = kSY + 2;
  static constexpr int kPlaneFloats = kBoxX * kBoxY;                  // floats per plane box
  static constexpr int kSlotFloats = (kPlaneFloats + 31) / 32 * 32;  // slots 128-byte aligned
};
constexpr int kSlots = 4;
constexpr int kHeadFloats = 64;              // before the pitched volume in tmp1: the support box

// Sticky status of the smoothing kernels (bit 0: a TMA wait gave up); read
// and cleared by si_smooth_status.
__device__ uint32_t g_smooth_status;

// Packed pairs per smoothing thread (si_smooth_set_pairs): 1 = 64-wide
// columns (default; measured faster on hit maps, whose support box skips
// more of the finer columns), 2 = 128-wide (faster on dense maps).
std::atomic<int> g_smooth_pairs{1};

inline int pitch4(int x) { return (x + 3) & ~3; }

// Support box of one map: b[0..2] = 0x7FFFFFFF - min(z, y, x), b[3..5] =
// max(z, y, x) + 1, all 0 when the map is all +0 (so one memset empties it).
__device__ __forceinline__ bool box_outside(const int* __restrict__ b, int grow, int z0, int z1, int y0, int y1,
                                            int x0, int x1) {
  if (b[3] == 0) return true;
  const int bz0 = 0x7FFFFFFF - b[0] - grow, by0 = 0x7FFFFFFF - b[1] - grow, bx0 = 0x7FFFFFFF - b[2] - grow;
  const int bz1 = b[3] - 1 + grow, by1 = b[4] - 1 + grow, bx1 = b[5] - 1 + grow;
  return z1 < bz0 || z0 > bz1 || y1 < by0 || y0 > by1 || x1 < bx0 || x0 > bx1;
}

// src map (uint32 hits or float32) -> pitched float32 copy, and the support
// box of its non-(+0) values. A warp takes one row at a time.
template <bool kSrcU32>
__global__ void __launch_bounds__(256) smooth_convert_kernel(const void* __restrict__ src, float* __restrict__ dst,
                                                             int Zc, int Yc, int Xc, int Xp, int* __restrict__ box) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  int zmin = 0x7FFFFFFF, ymin = 0x7FFFFFFF, xmin = 0x7FFFFFFF, zmax = -1, ymax = -1, xmax = -1;
  const int rows = Zc * Yc;
  for (int r = warp; r < rows; r += nwarps) {
    const size_t si = (size_t)r * Xc, di = (size_t)r * Xp;
    int rxmin = 0x7FFFFFFF, rxmax = -1;
    for (int x = lane; x < Xc; x += 32) {
      float v;
      if (kSrcU32) v = __uint2float_rn(static_cast<const uint32_t*>(src)[si + x]);
      else v = static_cast<const float*>(src)[si + x];
      dst[di + x] = v;
      if (__float_as_uint(v) != 0u) {
        rxmin = min(rxmin, x);
        rxmax = max(rxmax, x);
      }
    }
    if (rxmax >= 0) {
      const int z = r / Yc, y = r - (r / Yc) * Yc;
      zmin = min(zmin, z); zmax = max(zmax, z);
      ymin = min(ymin, y); ymax = max(ymax, y);
      xmin = min(xmin, rxmin); xmax = max(xmax, rxmax);
    }
  }
  zmin = __reduce_min_sync(0xffffffffu, zmin); ymin = __reduce_min_sync(0xffffffffu, ymin);
  xmin = __reduce_min_sync(0xffffffffu, xmin); zmax = __reduce_max_sync(0xffffffffu, zmax);
  ymax = __reduce_max_sync(0xffffffffu, ymax); xmax = __reduce_max_sync(0xffffffffu, xmax);
  if (lane == 0 && zmax >= 0) {
    atomicMax(&box[0], 0x7FFFFFFF - zmin); atomicMax(&box[1], 0x7FFFFFFF - ymin);
    atomicMax(&box[2], 0x7FFFFFFF - xmin); atomicMax(&box[3], zmax + 1);
    atomicMax(&box[4], ymax + 1); atomicMax(&box[5], xmax + 1);
  }
}

template <bool kF64, int kP>
__global__ void __launch_bounds__(256, kP == 1 ? 3 : 2) smooth_tma_kernel(const __grid_constant__ CUtensorMap src,
                                                                         float* __restrict__ dst, int dst_pitch,
                                                                         int Zc, int Yc, int Xc,
                                                                         const int* __restrict__ box, int grow,
                                                                         int write_outside, uint32_t wait_lim) {
  using T = SmoothTile<kP>;
  constexpr int kBoxX = T::kBoxX;
  __shared__ __align__(128) float pl[kSlots][T::kSlotFloats];
  __shared__ __align__(8) uint64_t bar[kSlots];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int x0 = blockIdx.x * T::kSX, y0 = blockIdx.y * kSY, zb = blockIdx.z * kSZ;
  const int ze = min(zb + kSZ, Zc);
  const int y = y0 + ty;
  const size_t dF = (size_t)Yc * dst_pitch;
  if (box_outside(box, grow, zb, ze - 1, y0, min(y0 + kSY, Yc) - 1, x0, min(x0 + T::kSX, Xc) - 1)) {
    if (write_outside && y < Yc) {
      for (int z = zb; z < ze; ++z) {
        float* row = dst + (size_t)z * dF + (size_t)y * dst_pitch;
#pragma unroll
        for (int j = 0; j < 2 * kP; ++j)
          if (x0 + tx + 32 * j < Xc) row[x0 + tx + 32 * j] = 0.0f;
      }
    }
    return;
  }
  const int nq = ze - zb + 2;  // planes zb-1 .. ze; plane zb-1+q sits in slot q & 3
  if (threadIdx.x == 0) {
    for (int s = 0; s < kSlots; ++s) mbar_init(&bar[s], 1);
    fence_barrier_init();
  }
  __syncthreads();
  int issued = 0;  // meaningful in thread 0 only
  if (threadIdx.x == 0) {
    fence_proxy_async_shared();
    for (; issued < kSlots && issued < nq; ++issued) {
      mbar_expect_tx(&bar[issued], T::kPlaneFloats * (uint32_t)sizeof(float));
      tma_load_box(pl[issued], &src, x0 - 4, y0 - 1, zb - 1 + issued, &bar[issued]);
    }
  }
  const int ly = ty + 1;
  const int i0 = ly * kBoxX + tx + 4;  // column j of the thread sits at i0 + 32 j
  auto cross = [&](const float* P, int p, uint64_t& cc, uint64_t& xm, uint64_t& xp, uint64_t& ym, uint64_t& yp) {
    const int ia = i0 + 64 * p, ib = ia + 32;
    cc = f2_pack(P[ia], P[ib]);
    xm = f2_pack(P[ia - 1], P[ib - 1]);
    xp = f2_pack(P[ia + 1], P[ib + 1]);
    ym = f2_pack(P[ia - kBoxX], P[ib - kBoxX]);
    yp = f2_pack(P[ia + kBoxX], P[ib + kBoxX]);
  };
  auto wait_q = [&](int q) { return mbar_wait_bounded(&bar[q & 3], (uint32_t)(q >> 2) & 1u, wait_lim); };

  uint64_t m_c[kP], m_xm[kP], m_xp[kP], m_ym[kP], m_yp[kP];  // plane z-1
  uint64_t c_c[kP], c_xm[kP], c_xp[kP], c_ym[kP], c_yp[kP];  // plane z
#pragma unroll
  for (int p = 0; p < kP; ++p) m_c[p] = m_xm[p] = m_xp[p] = m_ym[p] = m_yp[p] = c_c[p] = c_xm[p] = c_xp[p] = c_ym[p] =
      c_yp[p] = 0;
  bool ok = wait_q(0);
  ok = ok && wait_q(1);
  if (ok) {
#pragma unroll
    for (int p = 0; p < kP; ++p) {
      cross(pl[0], p, m_c[p], m_xm[p], m_xp[p], m_ym[p], m_yp[p]);
      cross(pl[1], p, c_c[p], c_xm[p], c_xp[p], c_ym[p], c_yp[p]);
    }
  }
  const uint64_t two = f2_splat(2.0f), half = f2_splat(0.5f), quarter = f2_splat(0.25f);
  const uint64_t eps = f2_splat(1e-10f), hundredth = f2_splat(0.01f);
  const uint64_t nz = f2_negzero();  // products as fma(a, b, -0): never fused into a later sum
  const bool row_in = y < Yc, row_interior = y > 0 && y < Yc - 1;
  for (int k = 0; k < ze - zb; ++k) {
    const int z = zb + k;
    ok = ok && wait_q(k + 2);
    if (ok) {
      const float* C = pl[(k + 1) & 3];
      const float* Pn = pl[(k + 2) & 3];
      const bool z_int = z > 0 && z < Zc - 1;
      float* row = dst + (size_t)z * dF + (size_t)y * dst_pitch;
#pragma unroll
      for (int p = 0; p < kP; ++p) {
        const int ia = i0 + 64 * p, ib = ia + 32;
        const uint64_t k_mm = f2_pack(C[ia - kBoxX - 1], C[ib - kBoxX - 1]);
        const uint64_t k_pp = f2_pack(C[ia + kBoxX + 1], C[ib + kBoxX + 1]);
        const uint64_t k_mp = f2_pack(C[ia - kBoxX + 1], C[ib - kBoxX + 1]);
        const uint64_t k_pm = f2_pack(C[ia + kBoxX - 1], C[ib + kBoxX - 1]);
        uint64_t p_c, p_xm, p_xp, p_ym, p_yp;  // plane z+1
        cross(Pn, p, p_c, p_xm, p_xp, p_ym, p_yp);
        const uint64_t c2 = f2_mul(two, c_c[p], nz);
        const uint64_t dx = f2_mul(f2_sub(c_xm[p], c_xp[p]), half, nz);
        const uint64_t dxx = f2_add(f2_sub(c_xm[p], c2), c_xp[p]);
        const uint64_t dx2 = f2_mul(dx, dx, nz);
        const uint64_t dy = f2_mul(f2_sub(c_ym[p], c_yp[p]), half, nz);
        const uint64_t dyy = f2_add(f2_sub(c_ym[p], c2), c_yp[p]);
        const uint64_t dy2 = f2_mul(dy, dy, nz);
        const uint64_t dz = f2_mul(f2_sub(m_c[p], p_c), half, nz);
        const uint64_t dzz = f2_add(f2_sub(m_c[p], c2), p_c);
        const uint64_t dz2 = f2_mul(dz, dz, nz);
        const uint64_t dxy = f2_mul(f2_sub(f2_sub(f2_add(k_mm, k_pp), k_mp), k_pm), quarter, nz);
        const uint64_t dxz = f2_mul(f2_sub(f2_sub(f2_add(p_xm, m_xp[p]), p_xp), m_xm[p]), quarter, nz);
        const uint64_t dyz = f2_mul(f2_sub(f2_sub(f2_add(p_ym, m_yp[p]), p_yp), m_ym[p]), quarter, nz);
        uint64_t num = f2_add(f2_mul(dxx, f2_add(dy2, dz2), nz), f2_mul(dyy, f2_add(dx2, dz2), nz));
        num = f2_add(num, f2_mul(dzz, f2_add(dx2, dy2), nz));
        num = f2_sub(num, f2_mul(f2_mul(f2_mul(two, dx, nz), dy, nz), dxy, nz));
        num = f2_sub(num, f2_mul(f2_mul(f2_mul(two, dx, nz), dz, nz), dxz, nz));
        num = f2_sub(num, f2_mul(f2_mul(f2_mul(two, dy, nz), dz, nz), dyz, nz));
        const uint64_t den = f2_add(f2_add(f2_add(dx2, dy2), dz2), eps);
        float na, nb, da, db, ca, cb;
        f2_unpack(num, na, nb);
        f2_unpack(den, da, db);
        f2_unpack(c_c[p], ca, cb);
        // den >= 1e-10 > 0, so a zero numerator gives kappa = num (its sign
        // kept) exactly; flat neighbourhoods (zero regions of a hit map) skip
        // the division
        float ka = na, kb = nb;
        if (na != 0.0f || nb != 0.0f) {
          ka = __fdiv_rn(na, da);
          kb = __fdiv_rn(nb, db);
        }
        float oa, ob;
        if (kF64) {
          oa = __double2float_rn(__dadd_rn((double)ca, __dmul_rn(0.01, (double)ka)));
          ob = __double2float_rn(__dadd_rn((double)cb, __dmul_rn(0.01, (double)kb)));
        } else {
          f2_unpack(f2_add(c_c[p], f2_mul(hundredth, f2_pack(ka, kb), nz)), oa, ob);
        }
        const int xa = x0 + tx + 64 * p, xb = xa + 32;
        if (row_in && xa < Xc) row[xa] = (z_int && row_interior && xa > 0 && xa < Xc - 1) ? oa : ca;
        if (row_in && xb < Xc) row[xb] = (z_int && row_interior && xb > 0 && xb < Xc - 1) ? ob : cb;
        m_c[p] = c_c[p]; m_xm[p] = c_xm[p]; m_xp[p] = c_xp[p]; m_ym[p] = c_ym[p]; m_yp[p] = c_yp[p];
        c_c[p] = p_c; c_xm[p] = p_xm; c_xp[p] = p_xp; c_ym[p] = p_ym; c_yp[p] = p_yp;
      }
    }
    if (__syncthreads_or(!ok)) {
      // a wait gave up: let the copies still in flight land (bounded) before
      // the CTA's shared memory goes away, then report
      if (threadIdx.x == 0) {
        for (int q = issued > kSlots ? issued - kSlots : 0; q < issued; ++q)
          mbar_wait_bounded(&bar[q & 3], (uint32_t)(q >> 2) & 1u, kDrainWaitLimit);
        atomicOr(&g_smooth_status, 1u);
      }
      return;
    }
    // the slot of plane q = k was last read in step k - 1 (or the prologue): refill it
    if (threadIdx.x == 0 && issued < nq) {
      fence_proxy_async_shared();
      mbar_expect_tx(&bar[issued & 3], T::kPlaneFloats * (uint32_t)sizeof(float));
      tma_load_box(pl[issued & 3], &src, x0 - 4, y0 - 1, zb - 1 + issued, &bar[issued & 3]);
      ++issued;
    }
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

namespace si {
namespace {

// Tensor map over a pitched float32 volume (Zc, Yc, Xp) with logical extents
// (Zc, Yc, Xc): reads beyond Xc, Yc, Zc or below 0 return zero.
int encode_volume_map(CUtensorMap* map, float* base, int Zc, int Yc, int Xc, int box_x, const char* what) {
  const EncodeTiledFn enc = encode_fn();
  if (!enc) return set_error(SI_ERR_CUDA, "%s: cuTensorMapEncodeTiled unavailable", what);
  std::memset(map, 0, sizeof(*map));
  const int Xp = pitch4(Xc);
  const cuuint64_t dims[3] = {(cuuint64_t)Xc, (cuuint64_t)Yc, (cuuint64_t)Zc};
  const cuuint64_t strides[2] = {(cuuint64_t)Xp * sizeof(float), (cuuint64_t)Xp * Yc * sizeof(float)};
  const cuuint32_t boxd[3] = {(cuuint32_t)box_x, (cuuint32_t)(kSY + 2), 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult cr = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, boxd, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) return set_error(SI_ERR_CUDA, "%s: tensor map encoding failed (%d)", what, (int)cr);
  return SI_OK;
}

// Smoothing of nol maps (uint32 hits when kSrcU32, else float32) of
// Zc*Yc*Xc voxels; results as float32 in place. tmp0 holds the pitched
// source of odd iterations, tmp1 its 64-float head (the support box) and the
// pitched source of even iterations.
template <bool kSrcU32>
int smooth_maps(void* maps, float* tmp0, float* tmp1, int nol, int Zc, int Yc, int Xc, int iters, int update,
                cudaStream_t st, const char* what) {
  const size_t V = (size_t)Zc * Yc * Xc;
  const int Xp = pitch4(Xc);
  int* box = reinterpret_cast<int*>(tmp1);
  float* tmp1v = tmp1 + kHeadFloats;
  if (iters > 0 && ((reinterpret_cast<uintptr_t>(tmp0) | reinterpret_cast<uintptr_t>(tmp1)) & 15u))
    return set_error(SI_ERR_ARG, "%s: tmp0/tmp1 must be 16-byte aligned", what);
  // pairs per thread: 128-wide columns only when selected and the rows are long enough
  const int kp = g_smooth_pairs.load(std::memory_order_relaxed) == 1 || Xc <= 64 ? 1 : 2;
  const int sx = 64 * kp;
  CUtensorMap map0, map1;
  if (iters > 0) {
    int rc = encode_volume_map(&map0, tmp0, Zc, Yc, Xc, sx + 8, what);
    if (rc) return rc;
    rc = encode_volume_map(&map1, tmp1v, Zc, Yc, Xc, sx + 8, what);
    if (rc) return rc;
  }
  const dim3 grid((Xc + sx - 1) / sx, (Yc + kSY - 1) / kSY, (Zc + kSZ - 1) / kSZ);
  const int cgrid = std::max(1, std::min(sm_count() * 8, (Zc * Yc + 7) / 8));
  const uint32_t wl = wait_limit();
  for (int l = 0; l < nol; ++l) {
    void* m = static_cast<uint8_t*>(maps) + (size_t)l * V * 4;
    float* mf = static_cast<float*>(m);
    if (iters == 0) {
      if (kSrcU32) u32_to_f32_kernel<<<grid_for(V, 256), 256, 0, st>>>(static_cast<uint32_t*>(m), mf, V);
      continue;
    }
    if (cudaMemsetAsync(box, 0, 6 * sizeof(int), st) != cudaSuccess)
      return set_error(SI_ERR_CUDA, "%s: memset failed", what);
    smooth_convert_kernel<kSrcU32><<<cgrid, 256, 0, st>>>(m, tmp0, Zc, Yc, Xc, Xp, box);
    for (int it = 1; it <= iters; ++it) {
      const bool last = it == iters;
      const CUtensorMap& sm = (it & 1) ? map0 : map1;
      float* dst = last ? mf : ((it & 1) ? tmp1v : tmp0);
      const int pitch = last ? Xc : Xp;
      // only iteration 1's destination (tmp1) may hold another map's values
      // outside the support; every later destination is +0 there already
      const int write_outside = (it == 1 && !last) ? 1 : 0;
#define SI_SMOOTH(F64, P) \
  smooth_tma_kernel<F64, P><<<grid, 256, 0, st>>>(sm, dst, pitch, Zc, Yc, Xc, box, it, write_outside, wl)
      if (update) {
        if (kp == 2)
          SI_SMOOTH(true, 2);
        else
          SI_SMOOTH(true, 1);
      } else {
        if (kp == 2)
          SI_SMOOTH(false, 2);
        else
          SI_SMOOTH(false, 1);
      }
#undef SI_SMOOTH
    }
  }
  return check_launch(what);
}

int smooth_args(const void* maps, const float* tmp0, const float* tmp1, int nol, int Zc, int Yc, int Xc, int iters,
                int update, const char* what) {
  if (!maps || !tmp0 || !tmp1) return set_error(SI_ERR_ARG, "%s: null pointer", what);
  if (nol < 1 || nol > 256) return set_error(SI_ERR_ARG, "%s: nol must be 1..256", what);
  if (Zc < 1 || Yc < 1 || Xc < 1 || iters < 0) return set_error(SI_ERR_ARG, "%s: bad arguments", what);
  if (update != SI_SMOOTH_F32 && update != SI_SMOOTH_REF_F64)
    return set_error(SI_ERR_ARG, "%s: update must be SI_SMOOTH_F32 or SI_SMOOTH_REF_F64", what);
  if ((unsigned long long)Zc * Yc * pitch4(Xc) >= (1ull << 40))
    return set_error(SI_ERR_LIMIT, "%s: volume too large", what);
  return SI_OK;
}

}  // namespace
}  // namespace si

extern "C" int si_smooth_tmp_floats(int Zc, int Yc, int Xc, unsigned long long* n) {
  clear_error();
  if (!n || Zc < 1 || Yc < 1 || Xc < 1) return set_error(SI_ERR_ARG, "si_smooth_tmp_floats: bad arguments");
  *n = (unsigned long long)Zc * Yc * pitch4(Xc) + kHeadFloats;
  return SI_OK;
}

extern "C" int si_smooth(uint32_t* maps, float* tmp0, float* tmp1, int nol, int Zc, int Yc, int Xc, int iters,
                         int update, void* stream) {
  clear_error();
  const int rc = smooth_args(maps, tmp0, tmp1, nol, Zc, Yc, Xc, iters, update, "si_smooth");
  if (rc) return rc;
  return smooth_maps<true>(maps, tmp0, tmp1, nol, Zc, Yc, Xc, iters, update, as_stream(stream), "si_smooth");
}

extern "C" int si_smooth_f32(float* maps, float* tmp0, float* tmp1, int nol, int Zc, int Yc, int Xc, int iters,
                             int update, void* stream) {
  clear_error();
  const int rc = smooth_args(maps, tmp0, tmp1, nol, Zc, Yc, Xc, iters, update, "si_smooth_f32");
  if (rc) return rc;
  return smooth_maps<false>(maps, tmp0, tmp1, nol, Zc, Yc, Xc, iters, update, as_stream(stream), "si_smooth_f32");
}

extern "C" int si_smooth_set_pairs(int pairs) {
  clear_error();
  if (pairs < 1 || pairs > 2) return set_error(SI_ERR_ARG, "si_smooth_set_pairs: 1 or 2");
  g_smooth_pairs.store(pairs, std::memory_order_relaxed);
  return SI_OK;
}

extern "C" int si_smooth_status(int* status, void* stream) {
  clear_error();
  if (!status) return set_error(SI_ERR_ARG, "si_smooth_status: null pointer");
  cudaStream_t st = as_stream(stream);
  uint32_t v = 0;
  const uint32_t zero = 0;
  if (cudaMemcpyFromSymbolAsync(&v, g_smooth_status, sizeof(v), 0, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess ||
      cudaMemcpyToSymbolAsync(g_smooth_status, &zero, sizeof(zero), 0, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return set_error(SI_ERR_CUDA, "si_smooth_status: %s", cudaGetErrorString(cudaGetLastError()));
  *status = (int)v;
  if (v) return set_error(SI_ERR_CUDA, "smoothing: a TMA wait gave up (status %u)", v);
  return SI_OK;
}
