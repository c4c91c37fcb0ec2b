// Active-contour post-processing of a label volume on the device
// (biomedisa/features/active_contour.py:109-225 and curvop_numba.py:5-149):
//   * 'acwe': `steps` rounds of (label means -> evolution -> for every label
//     `smooth` erosion/dilation pairs);
//   * 'refined': a chamfer band around the labels (distance <= 10, by Jacobi
//     relaxation: see the refinement section), per-slice Gaussian likelihoods
//     from band histograms, and a per-slice lookup table that labels each band
//     voxel by its intensity.
// Both run on the reference's cropped volume: the image and labels padded by
// one zero voxel and cut to the labels' bounding box grown by 100 voxels
// (reduce_blocksize, active_contour.py:84-104), gathered in one pass.
//
// Layout: uint8 image D and labels L of the crop, C order. The 27-point
// stencils (evolution, erosion, dilation) stage three 34 x 10 byte planes of
// a 32 x 8 tile in shared memory and march 16 planes in z per CTA; every
// output voxel is written (non-interior voxels copy their input), so each
// pass is one read and one write of the crop.
#include <cfloat>
#include <cmath>
#include <cstdint>

#include "si_internal.h"

namespace si {
namespace {

constexpr int kTX = 32, kTY = 8, kZChunk = 16;
constexpr int kRowB = kTX + 2;          // bytes per staged row (1-voxel halo)
constexpr int kPlaneB = (kTY + 2) * kRowB;  // bytes per staged plane
constexpr uint32_t kAll27 = (1u << 27) - 1u;

// Offset index i = (dz+1)*9 + (dy+1)*3 + (dx+1): the reference's loop order
// (dz outer, dx inner). The nine 3x3 planes through the centre that erosion
// tests (curvop_numba.py:125-134): x = 0, y = 0, z = 0, y = x, y = -x, z = x,
// z = -x, z = y, z = -y.
__host__ __device__ constexpr uint32_t plane_mask(int which) {
  uint32_t m = 0;
  for (int i = 0; i < 27; ++i) {
    const int dz = i / 9 - 1, dy = (i / 3) % 3 - 1, dx = i % 3 - 1;
    bool in = false;
    switch (which) {
      case 0: in = dx == 0; break;
      case 1: in = dy == 0; break;
      case 2: in = dz == 0; break;
      case 3: in = dy == dx; break;
      case 4: in = dy == -dx; break;
      case 5: in = dz == dx; break;
      case 6: in = dz == -dx; break;
      case 7: in = dz == dy; break;
      default: in = dz == -dy; break;
    }
    if (in) m |= 1u << i;
  }
  return m;
}

enum StencilOp { kEvolution = 0, kErosion = 1, kDilation = 2 };

// Label cost of evolution (curvop_numba.py:13-24, numba's typing): the
// binary32 distance d = |mean - intensity| (float32 - uint8 is float32),
// times alpha in binary64 for label 0; the comparisons are binary64.
// Every cost but label 0's is a binary32 value, so costs are compared as
// keys (f, flag) without binary64 arithmetic in the loop: a binary32 cost d
// is (d, 0); label 0's binary64 cost c0 is (the smallest binary32 >= c0, -1
// if c0 is not a binary32 value else 0). For a binary32 d, c0 < d iff
// d >= ceil32(c0) and d < c0 iff d < ceil32(c0) when c0 is inexact, so the
// lexicographic order of the keys is the order of the binary64 costs (a NaN
// key compares false both ways, as NaN costs do).
struct EvoKey {
  float f;
  int flag;
};

__device__ __forceinline__ bool key_less(const EvoKey& a, const EvoKey& b) {
  return a.f < b.f || (a.f == b.f && a.flag < b.flag);
}

__device__ __forceinline__ EvoKey zero_key(const float* mean, float f, double alpha) {
  const double c0 = __dmul_rn(alpha, (double)fabsf(__fsub_rn(mean[0], f)));
  const float up = __double2float_ru(c0);
  return EvoKey{up, (double)up == c0 ? 0 : -1};
}

__device__ __forceinline__ EvoKey evo_key(const float* mean, int l, float f, const EvoKey& k0) {
  return l == 0 ? k0 : EvoKey{fabsf(__fsub_rn(mean[l], f)), 0};
}

// One pass of a 27-point stencil over the crop (Z, Y, X); dst must not alias
// src. kEvolution reads img and the label sums; kErosion / kDilation act on
// `label`.
template <int kOp>
__global__ void __launch_bounds__(kTX* kTY) acwe_stencil_kernel(const uint8_t* __restrict__ src,
                                                                 const uint8_t* __restrict__ img,
                                                                 const unsigned long long* __restrict__ sums,
                                                                 double alpha, int label, int Z, int Y, int X,
                                                                 uint8_t* __restrict__ dst) {
  __shared__ uint8_t s[3][kPlaneB];
  __shared__ float mean[256];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTX + tx;
  const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY, zs = blockIdx.z * kZChunk;
  const int ze = min(zs + kZChunk, Z);
  if (kOp == kEvolution) {
    // mean[k] = float32(float64 mean) for the labels present, 0 elsewhere
    // (active_contour.py:191-195); the float64 sum of integers is exact.
    for (int k = tid; k < 256; k += kTX * kTY) {
      const unsigned long long cnt = sums[k];
      mean[k] = cnt ? __double2float_rn(__ddiv_rn((double)sums[256 + k], (double)cnt)) : 0.0f;
    }
  }
  auto load_plane = [&](int z, int slot) {
    for (int i = tid; i < kPlaneB; i += kTX * kTY) {
      const int r = i / kRowB, c = i - r * kRowB;
      const int gy = y0 - 1 + r, gx = x0 - 1 + c;
      uint8_t v = 0;
      if ((unsigned)z < (unsigned)Z && (unsigned)gy < (unsigned)Y && (unsigned)gx < (unsigned)X)
        v = src[((size_t)z * Y + gy) * X + gx];
      s[slot][i] = v;
    }
  };
  load_plane(zs - 1, 0);
  load_plane(zs, 1);
  const int x = x0 + tx, y = y0 + ty;
  const bool in_xy = x < X && y < Y;
  const bool int_xy = x >= 1 && x <= X - 2 && y >= 1 && y <= Y - 2;
  const int cpos = (ty + 1) * kRowB + tx + 1;
  int sm = 0, sc = 1, sp = 2;
  for (int z = zs; z < ze; ++z) {
    load_plane(z + 1, sp);
    __syncthreads();
    if (in_xy) {
      const size_t v = ((size_t)z * Y + y) * X + x;
      const int c = s[sc][cpos];
      int out = c;
      if (int_xy && z >= 1 && z <= Z - 2) {
        const uint8_t* pl[3] = {s[sm], s[sc], s[sp]};
        if (kOp == kEvolution) {
          uint32_t same = 0;
#pragma unroll
          for (int i = 0; i < 27; ++i)
            same |= (uint32_t)(pl[i / 9][cpos + ((i / 3) % 3 - 1) * kRowB + (i % 3 - 1)] == c) << i;
          if (same != kAll27) {  // a voxel inside one label keeps it
            const float f = (float)img[v];
            const EvoKey k0 = zero_key(mean, f, alpha);
            EvoKey ref = evo_key(mean, c, f, k0);
#pragma unroll
            for (int i = 0; i < 27; ++i) {
              const int t = pl[i / 9][cpos + ((i / 3) % 3 - 1) * kRowB + (i % 3 - 1)];
              if (t != c) {
                const EvoKey val = evo_key(mean, t, f, k0);
                if (key_less(val, ref)) {
                  ref = val;
                  out = t;
                }
              }
            }
          }
        } else {
          uint32_t m = 0;
#pragma unroll
          for (int i = 0; i < 27; ++i)
            m |= (uint32_t)(pl[i / 9][cpos + ((i / 3) % 3 - 1) * kRowB + (i % 3 - 1)] == label) << i;
          if (kOp == kErosion) {
            if (c == label && m != kAll27) {
              bool keep = false;
#pragma unroll
              for (int t = 0; t < 9; ++t) keep |= (m & plane_mask(t)) == plane_mask(t);
              if (!keep) {
                // the last differing neighbour in scan order
                const int i = 31 - __clz(~m & kAll27);
                const int slot = i < 9 ? sm : (i < 18 ? sc : sp);
                out = s[slot][cpos + ((i / 3) % 3 - 1) * kRowB + (i % 3 - 1)];
              }
            }
          } else if (c != label && m != 0) {
            out = label;
          }
        }
      }
      dst[v] = (uint8_t)out;
    }
    __syncthreads();
    const int t = sm;
    sm = sc;
    sc = sp;
    sp = t;
  }
}

// ---------------------------------------------------------------------------
// curvop on bit masks. A label's mask is packed once per curvop, 32 voxels
// of a row per word: M[(z * Y + y) * W + w] bit j = (L[z][y][32 w + j] ==
// label), W = ceil(X / 32). Each erosion/dilation pass is one thread per
// word: the 27 neighbour masks are the 9 neighbouring rows' words shifted by
// one bit (carries from the adjacent words), the nine planes are ANDs of
// their members, and the pass writes the next mask word. Voxels change in
// place in L: dilation writes `label` (it reads masks only); erosion writes
// the last differing neighbour's value, read from L — a non-label voxel,
// which an erosion pass never changes, so the in-place update is race-free.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) acwe_pack_kernel(const uint8_t* __restrict__ L, int Z, int Y, int X, int W,
                                                        int label, uint32_t* __restrict__ M) {
  const int lane = threadIdx.x & 31;
  const int64_t rows = (int64_t)Z * Y;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < rows; r += nwarps) {
    const uint8_t* row = L + r * X;
    uint32_t* mrow = M + r * W;
    for (int w0 = 0; w0 < W; w0 += 32) {
      uint32_t mine = 0;  // lane i keeps word w0 + i
      const int nw = min(32, W - w0);
      for (int i = 0; i < nw; ++i) {
        const int x = 32 * (w0 + i) + lane;
        const bool hit = x < X && row[x] == label;
        const uint32_t word = __ballot_sync(0xffffffffu, hit);
        if (lane == i) mine = word;
      }
      if (lane < nw) mrow[w0 + lane] = mine;
    }
  }
}

template <bool kErode>
__global__ void __launch_bounds__(256) acwe_morph_bits_kernel(uint8_t* __restrict__ L,
                                                              const uint32_t* __restrict__ Min,
                                                              uint32_t* __restrict__ Mout, int Z, int Y, int X, int W,
                                                              int label) {
  const int64_t n = (int64_t)Z * Y * W;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int w = (int)(i % W);
    const int64_t zy = i / W;
    const int y = (int)(zy % Y), z = (int)(zy / Y);
    const uint32_t m = Min[i];
    if (z < 1 || z > Z - 2 || y < 1 || y > Y - 2) {
      Mout[i] = m;
      continue;
    }
    // interior columns 1..X-2 of this word
    const int xa = 32 * w;
    uint32_t inner = 0xffffffffu;
    if (xa == 0) inner &= ~1u;
    const int last = X - 2 - xa;  // highest interior bit
    if (last < 31) inner &= last >= 0 ? (0xffffffffu >> (31 - last)) : 0u;
    // neighbour masks S[k], k = (dz+1)*9 + (dy+1)*3 + (dx+1): bit j = voxel
    // (z+dz, y+dy, xa+j+dx) is the label
    uint32_t S[27];
#pragma unroll
    for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
      for (int dy = -1; dy <= 1; ++dy) {
        const int64_t r = ((int64_t)(z + dz) * Y + (y + dy)) * W;
        const uint32_t c = Min[r + w];
        const uint32_t p = w > 0 ? Min[r + w - 1] : 0u;
        const uint32_t q = w + 1 < W ? Min[r + w + 1] : 0u;
        const int k = (dz + 1) * 9 + (dy + 1) * 3;
        S[k] = (c << 1) | (p >> 31);
        S[k + 1] = c;
        S[k + 2] = (c >> 1) | (q << 31);
      }
    uint32_t cond;
    if (kErode) {
      uint32_t all = 0xffffffffu, keep = 0u;
#pragma unroll
      for (int k = 0; k < 27; ++k) all &= S[k];
#pragma unroll
      for (int t = 0; t < 9; ++t) {
        uint32_t full = 0xffffffffu;
#pragma unroll
        for (int k = 0; k < 27; ++k)
          if (plane_mask(t) >> k & 1u) full &= S[k];
        keep |= full;
      }
      cond = m & ~all & ~keep & inner;
      uint32_t todo = cond;
      while (todo) {
        const int j = __ffs(todo) - 1;
        todo &= todo - 1u;
        // the last neighbour in scan order that is not the label
        int k = 26;
        while (k > 0 && (S[k] >> j & 1u)) --k;
        const int dz = k / 9 - 1, dy = (k / 3) % 3 - 1, dx = k % 3 - 1;
        const uint8_t sub = L[((int64_t)(z + dz) * Y + (y + dy)) * X + (xa + j + dx)];
        L[((int64_t)z * Y + y) * X + xa + j] = sub;
      }
      Mout[i] = m & ~cond;
    } else {
      uint32_t any = 0u;
#pragma unroll
      for (int k = 0; k < 27; ++k) any |= S[k];
      cond = ~m & any & inner;
      uint32_t todo = cond;
      while (todo) {
        const int j = __ffs(todo) - 1;
        todo &= todo - 1u;
        L[((int64_t)z * Y + y) * X + xa + j] = (uint8_t)label;
      }
      Mout[i] = m | cond;
    }
  }
}

// ---------------------------------------------------------------------------
// Image conversion (img_to_uint8, biomedisa_helper.py:345-352) and gather.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ float to_f32(T v);
template <>
__device__ __forceinline__ float to_f32<uint8_t>(uint8_t v) { return (float)v; }
template <>
__device__ __forceinline__ float to_f32<int8_t>(int8_t v) { return (float)v; }
template <>
__device__ __forceinline__ float to_f32<uint16_t>(uint16_t v) { return __uint2float_rn(v); }
template <>
__device__ __forceinline__ float to_f32<int16_t>(int16_t v) { return __int2float_rn(v); }
template <>
__device__ __forceinline__ float to_f32<int32_t>(int32_t v) { return __int2float_rn(v); }
template <>
__device__ __forceinline__ float to_f32<float>(float v) { return v; }

__device__ __forceinline__ void atomic_min_f(float* addr, float v) {
  if (v >= 0.0f)
    atomicMin(reinterpret_cast<int*>(addr), __float_as_int(v));
  else
    atomicMax(reinterpret_cast<unsigned int*>(addr), __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float* addr, float v) {
  if (v >= 0.0f)
    atomicMax(reinterpret_cast<int*>(addr), __float_as_int(v));
  else
    atomicMin(reinterpret_cast<unsigned int*>(addr), __float_as_uint(v));
}

// Where an image array sits in the padded frame: voxel (a, b, c) of the
// (iZ, iY, iX) array is padded voxel (iz0 + a, iy0 + b, ix0 + c). The padded
// frame's interior is 1..Z, 1..Y, 1..X.
struct Frame {
  int iZ, iY, iX, iz0, iy0, ix0;
  int Z, Y, X;
};

template <typename T>
__global__ void __launch_bounds__(256) acwe_minmax_kernel(const T* __restrict__ img, Frame f, float* __restrict__ mm) {
  float lo = FLT_MAX, hi = -FLT_MAX;
  const uint64_t n = (uint64_t)f.iZ * f.iY * f.iX;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int c = (int)(i % f.iX);
    const uint64_t ab = i / f.iX;
    const int b = (int)(ab % f.iY), a = (int)(ab / f.iY);
    const int pz = f.iz0 + a, py = f.iy0 + b, px = f.ix0 + c;
    if (pz < 1 || pz > f.Z || py < 1 || py > f.Y || px < 1 || px > f.X) continue;
    const float v = to_f32<T>(img[i]);
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
  for (int o = 16; o; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_min_f(&mm[0], lo);
    atomic_max_f(&mm[1], hi);
  }
}

struct CropBox {
  int cz0, cy0, cx0, cZ, cY, cX;
};

// D and L of the crop. convert = 0: the image is uint8 and copied; 1: the
// value (0 outside the image array) is shifted by mn, divided by mx and scaled
// by 255 in binary32, then truncated (NaN -> 0). Padding voxels are 0.
template <typename T>
__global__ void __launch_bounds__(256) acwe_gather_kernel(const T* __restrict__ img, Frame f, int convert, float mn,
                                                          float mx, const uint8_t* __restrict__ labels, CropBox cb,
                                                          uint8_t* __restrict__ D, uint8_t* __restrict__ L) {
  const uint64_t n = (uint64_t)cb.cZ * cb.cY * cb.cX;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int xc = (int)(i % cb.cX);
    const uint64_t zy = i / cb.cX;
    const int yc = (int)(zy % cb.cY), zc = (int)(zy / cb.cY);
    const int pz = cb.cz0 + zc, py = cb.cy0 + yc, px = cb.cx0 + xc;
    uint8_t d = 0, l = 0;
    if (pz >= 1 && pz <= f.Z && py >= 1 && py <= f.Y && px >= 1 && px <= f.X) {
      l = labels[((size_t)(pz - 1) * f.Y + (py - 1)) * f.X + (px - 1)];
      const int a = pz - f.iz0, b = py - f.iy0, c = px - f.ix0;
      const bool inside = (unsigned)a < (unsigned)f.iZ && (unsigned)b < (unsigned)f.iY && (unsigned)c < (unsigned)f.iX;
      const T raw = inside ? img[((size_t)a * f.iY + b) * f.iX + c] : T(0);
      if (convert) {
        const float q = __fmul_rn(__fdiv_rn(__fsub_rn(to_f32<T>(raw), mn), mx), 255.0f);
        d = (uint8_t)__float2uint_rz(q == q ? q : 0.0f);
      } else {
        d = (uint8_t)raw;
      }
    }
    D[i] = d;
    L[i] = l;
  }
}

// Per-label voxel counts (sums[0..255]) and intensity sums (sums[256..511]).
// Each thread takes 16 consecutive voxels and folds runs of one label in
// registers before touching shared memory.
__global__ void __launch_bounds__(256) acwe_label_sums_kernel(const uint8_t* __restrict__ D,
                                                              const uint8_t* __restrict__ L, uint64_t n,
                                                              unsigned long long* __restrict__ sums) {
  __shared__ uint32_t cnt[256], sm[256];
  for (int k = threadIdx.x; k < 256; k += blockDim.x) cnt[k] = sm[k] = 0;
  __syncthreads();
  const uint64_t chunks = (n + 15) / 16;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t ch = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; ch < chunks; ch += stride) {
    const uint64_t b = ch * 16, e = b + 16 < n ? b + 16 : n;
    int cur = -1;
    uint32_t c = 0, s = 0;
    for (uint64_t i = b; i < e; ++i) {
      const int l = L[i];
      if (l != cur) {
        if (c) {
          atomicAdd(&cnt[cur], c);
          atomicAdd(&sm[cur], s);
        }
        cur = l;
        c = s = 0;
      }
      ++c;
      s += D[i];
    }
    if (c) {
      atomicAdd(&cnt[cur], c);
      atomicAdd(&sm[cur], s);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < 256; k += blockDim.x) {
    if (cnt[k]) {
      atomicAdd(&sums[k], (unsigned long long)cnt[k]);
      atomicAdd(&sums[256 + k], (unsigned long long)sm[k]);
    }
  }
}

// Crop -> output volume (Z, Y, X): voxel (z, y, x) is padded voxel
// (z+1, y+1, x+1); outside the crop it is 0.
__global__ void __launch_bounds__(256) acwe_scatter_kernel(const uint8_t* __restrict__ L, CropBox cb, int Z, int Y,
                                                           int X, uint8_t* __restrict__ out) {
  const uint64_t n = (uint64_t)Z * Y * X;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int x = (int)(i % X);
    const uint64_t zy = i / X;
    const int y = (int)(zy % Y), z = (int)(zy / Y);
    const int a = z + 1 - cb.cz0, b = y + 1 - cb.cy0, c = x + 1 - cb.cx0;
    uint8_t v = 0;
    if ((unsigned)a < (unsigned)cb.cZ && (unsigned)b < (unsigned)cb.cY && (unsigned)c < (unsigned)cb.cX)
      v = L[((size_t)a * cb.cY + b) * cb.cX + c];
    out[i] = v;
  }
}

// ---------------------------------------------------------------------------
// Refinement (active_contour.py:204-225).
//
// The band. The reference runs one forward and one backward chamfer raster
// scan (weights 1, sqrt2, sqrt3) from 0 on labels / 100 elsewhere and keeps
// distance <= 10. For every voxel whose band membership reaches the output,
// that scan gives the exact chamfer distance to the nearest label: an optimal
// path is monotone in each coordinate, so its moves sort into forward moves
// (the forward pass's neighbours) followed by backward moves, all inside the
// box of its ends and so inside both passes' domains. (The crop's boundary
// rows and columns, never updated by the reference, are never band here
// either; its first and last planes are padding, whose slices the result
// drops, or lie at least 100 voxels from any label.) The decision <= 10 does
// not depend on rounding: path lengths p + q sqrt2 + r sqrt3 within 10 moves
// are exactly 10 or differ from it by at least 0.0246, far beyond binary32
// rounding. So the band is computed by Jacobi relaxation instead of the
// sequential scan: pass k takes each interior voxel's minimum over itself and
// its 26 neighbours plus the move weights; after 10 passes every path of
// cost <= 10 (at most 10 moves) has been followed. Values are clamped to 11.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTX* kTY) acwe_chamfer_pass_kernel(const float* __restrict__ src, int Z, int Y,
                                                                     int X, float* __restrict__ dst) {
  constexpr int kRowF = kTX + 2, kPlaneF = (kTY + 2) * kRowF;
  __shared__ float s[3][kPlaneF];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTX + tx;
  const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY, zs = blockIdx.z * kZChunk;
  const int ze = min(zs + kZChunk, Z);
  auto load_plane = [&](int z, int slot) {
    for (int i = tid; i < kPlaneF; i += kTX * kTY) {
      const int r = i / kRowF, c = i - r * kRowF;
      const int gy = y0 - 1 + r, gx = x0 - 1 + c;
      float v = 11.0f;
      if ((unsigned)z < (unsigned)Z && (unsigned)gy < (unsigned)Y && (unsigned)gx < (unsigned)X)
        v = src[((size_t)z * Y + gy) * X + gx];
      s[slot][i] = v;
    }
  };
  load_plane(zs - 1, 0);
  load_plane(zs, 1);
  const int x = x0 + tx, y = y0 + ty;
  const bool in_xy = x < X && y < Y;
  const bool int_xy = x >= 1 && x <= X - 2 && y >= 1 && y <= Y - 2;
  const int cpos = (ty + 1) * kRowF + tx + 1;
  const float w1 = 1.0f, w2 = 1.41421356f, w3 = 1.73205081f;
  int sm = 0, sc = 1, sp = 2;
  for (int z = zs; z < ze; ++z) {
    load_plane(z + 1, sp);
    __syncthreads();
    if (in_xy) {
      float best = s[sc][cpos];
      if (int_xy) {  // every plane of the crop relaxes (see above); rows/columns 0 and n-1 keep their values
        const float* pl[3] = {s[sm], s[sc], s[sp]};
#pragma unroll
        for (int i = 0; i < 27; ++i) {
          const int dz = i / 9 - 1, dy = (i / 3) % 3 - 1, dx = i % 3 - 1;
          const int nzero = (dz != 0) + (dy != 0) + (dx != 0);
          if (nzero == 0 || (z + dz) < 0 || (z + dz) >= Z) continue;
          const float w = nzero == 1 ? w1 : (nzero == 2 ? w2 : w3);
          best = fminf(best, __fadd_rn(pl[dz + 1][cpos + dy * kRowF + dx], w));
        }
        best = fminf(best, 11.0f);
      }
      dst[((size_t)z * Y + y) * X + x] = best;
    }
    __syncthreads();
    const int t = sm;
    sm = sc;
    sc = sp;
    sp = t;
  }
}


__global__ void __launch_bounds__(256) acwe_dist_init_kernel(const uint8_t* __restrict__ L, uint64_t n,
                                                             float* __restrict__ dist) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    dist[i] = L[i] == 0 ? 100.0f : 0.0f;
}

// Band (distance <= 10) histograms per z-slice: hist[z][class][intensity],
// class = class_lut[label]. Blocks (bx, z); with use_smem the slice part is
// counted in shared memory (ncls * 256 counters) first.
__global__ void __launch_bounds__(256) acwe_band_hist_kernel(const float* __restrict__ dist,
                                                             const uint8_t* __restrict__ D,
                                                             const uint8_t* __restrict__ L,
                                                             const int16_t* __restrict__ class_lut, int ncls,
                                                             int Y, int X, int use_smem,
                                                             uint32_t* __restrict__ hist) {
  extern __shared__ uint32_t h[];
  const int z = blockIdx.y;
  uint32_t* gh = hist + (size_t)z * ncls * 256;
  if (use_smem) {
    for (int k = threadIdx.x; k < ncls * 256; k += blockDim.x) h[k] = 0;
    __syncthreads();
  }
  const uint64_t YX = (uint64_t)Y * X;
  const size_t base = (size_t)z * YX;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < YX; i += (uint64_t)gridDim.x * blockDim.x) {
    if (dist[base + i] <= 10.0f) {
      const int s = class_lut[L[base + i]];
      if (s < 0) continue;
      const int bin = s * 256 + D[base + i];
      if (use_smem)
        atomicAdd(&h[bin], 1u);
      else
        atomicAdd(&gh[bin], 1u);
    }
  }
  if (use_smem) {
    __syncthreads();
    for (int k = threadIdx.x; k < ncls * 256; k += blockDim.x)
      if (h[k]) atomicAdd(&gh[k], h[k]);
  }
}

template <typename V>
__device__ __forceinline__ V block_sum_256(V v, V* red) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  V t = 0;
  for (int k = 0; k < 8; ++k) t += red[k];  // fixed order: deterministic
  return t;
}

// One CTA of 256 threads per z-slice, thread = intensity v. Candidate j
// (label cand_label[j], histogram class j + 1; class 0 holds every other
// label) in order: where the band holds voxels of the label and of the rest,
// the Gaussian likelihoods p1 (label) and p2 (rest) of intensity v decide
// the slice's lookup entry; a later candidate overwrites the slice, as the
// reference's result[k] = ... does. lut[z][v] = label or 0.
__global__ void __launch_bounds__(256) acwe_refine_decide_kernel(const uint32_t* __restrict__ hist,
                                                                 const uint8_t* __restrict__ cand_label, int ncand,
                                                                 uint8_t* __restrict__ lut) {
  __shared__ unsigned long long red_u[8];
  __shared__ double red_d[8];
  const int z = blockIdx.x, v = threadIdx.x;
  const int ncls = ncand + 1;
  const uint32_t* hz = hist + (size_t)z * ncls * 256;
  uint32_t tot = 0;
  for (int s = 0; s < ncls; ++s) tot += hz[s * 256 + v];
  const unsigned long long n_tot = block_sum_256<unsigned long long>(tot, red_u);
  const unsigned long long s_tot = block_sum_256<unsigned long long>((unsigned long long)tot * v, red_u);
  int out = 0;
  const double dv = (double)v;
  const double two_pi = 6.283185307179586;  // 2 * pi in binary64 (2 * np.pi)
  for (int j = 0; j < ncand; ++j) {
    const uint32_t hin = hz[(j + 1) * 256 + v], hout = tot - hin;
    const unsigned long long n1 = block_sum_256<unsigned long long>(hin, red_u);
    const unsigned long long s1sum = block_sum_256<unsigned long long>((unsigned long long)hin * v, red_u);
    const unsigned long long n2 = n_tot - n1, s2sum = s_tot - s1sum;
    if (n1 == 0 || n2 == 0) continue;  // uniform over the block
    const double m1 = __ddiv_rn((double)s1sum, (double)n1), m2 = __ddiv_rn((double)s2sum, (double)n2);
    const double x1 = __dsub_rn(dv, m1), x2 = __dsub_rn(dv, m2);
    const double q1 = __dmul_rn(x1, x1), q2 = __dmul_rn(x2, x2);
    const double var1 = block_sum_256<double>(__dmul_rn((double)hin, q1), red_d);
    const double var2 = block_sum_256<double>(__dmul_rn((double)hout, q2), red_d);
    double sd1 = __dsqrt_rn(__ddiv_rn(var1, (double)n1)), sd2 = __dsqrt_rn(__ddiv_rn(var2, (double)n2));
    sd1 = sd1 > 1.0 ? sd1 : 1.0;
    sd2 = sd2 > 1.0 ? sd2 : 1.0;
    const double v1 = __dmul_rn(sd1, sd1), v2 = __dmul_rn(sd2, sd2);
    const double p1 = __ddiv_rn(exp(__ddiv_rn(-q1, __dmul_rn(2.0, v1))), __dsqrt_rn(__dmul_rn(two_pi, v1)));
    const double p2 = __ddiv_rn(exp(__ddiv_rn(-q2, __dmul_rn(2.0, v2))), __dsqrt_rn(__dmul_rn(two_pi, v2)));
    out = p1 > p2 ? cand_label[j] : 0;
  }
  lut[(size_t)z * 256 + v] = (uint8_t)out;
}

// Refined labels in the output volume (Z, Y, X): band voxels of the crop take
// their slice's lookup entry for their intensity; everything else is 0.
__global__ void __launch_bounds__(256) acwe_refine_apply_kernel(const float* __restrict__ dist,
                                                                const uint8_t* __restrict__ D,
                                                                const uint8_t* __restrict__ lut, CropBox cb, int Z,
                                                                int Y, int X, uint8_t* __restrict__ out) {
  const uint64_t n = (uint64_t)Z * Y * X;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int x = (int)(i % X);
    const uint64_t zy = i / X;
    const int y = (int)(zy % Y), z = (int)(zy / Y);
    const int a = z + 1 - cb.cz0, b = y + 1 - cb.cy0, c = x + 1 - cb.cx0;
    uint8_t v = 0;
    if ((unsigned)a < (unsigned)cb.cZ && (unsigned)b < (unsigned)cb.cY && (unsigned)c < (unsigned)cb.cX) {
      const size_t j = ((size_t)a * cb.cY + b) * cb.cX + c;
      if (dist[j] <= 10.0f) v = lut[(size_t)a * 256 + D[j]];
    }
    out[i] = v;
  }
}

inline int grid_n(uint64_t n, int block) {
  const uint64_t want = (n + block - 1) / block;
  const uint64_t cap = (uint64_t)sm_count() * 16;
  return (int)(want < cap ? (want > 0 ? want : 1) : cap);
}

inline bool crop_ok(const CropBox& cb) { return cb.cZ > 0 && cb.cY > 0 && cb.cX > 0; }

int stencil_pass(int op, const uint8_t* src, const uint8_t* img, const unsigned long long* sums, double alpha,
                 int label, int Z, int Y, int X, uint8_t* dst, cudaStream_t st) {
  const dim3 block(kTX, kTY);
  const dim3 grid((X + kTX - 1) / kTX, (Y + kTY - 1) / kTY, (Z + kZChunk - 1) / kZChunk);
  switch (op) {
    case kEvolution:
      acwe_stencil_kernel<kEvolution><<<grid, block, 0, st>>>(src, img, sums, alpha, label, Z, Y, X, dst);
      break;
    case kErosion:
      acwe_stencil_kernel<kErosion><<<grid, block, 0, st>>>(src, img, sums, alpha, label, Z, Y, X, dst);
      break;
    default:
      acwe_stencil_kernel<kDilation><<<grid, block, 0, st>>>(src, img, sums, alpha, label, Z, Y, X, dst);
      break;
  }
  return check_launch("si_acwe stencil");
}

inline bool dims_ok(int Z, int Y, int X) {
  return Z > 0 && Y > 0 && X > 0 && (uint64_t)(Z + kZChunk) / kZChunk < 65536u &&
         (uint64_t)(Y + kTY) / kTY < 65536u;
}

}  // namespace
}  // namespace si

using namespace si;

extern "C" int si_acwe_minmax(const void* img, int dtype, int iZ, int iY, int iX, int iz0, int iy0, int ix0, int Z,
                              int Y, int X, float* mm, void* stream) {
  clear_error();
  if (!img || !mm) return set_error(SI_ERR_ARG, "si_acwe_minmax: null pointer");
  if (iZ < 1 || iY < 1 || iX < 1 || Z < 1 || Y < 1 || X < 1)
    return set_error(SI_ERR_ARG, "si_acwe_minmax: bad dimensions");
  const Frame f{iZ, iY, iX, iz0, iy0, ix0, Z, Y, X};
  const uint64_t n = (uint64_t)iZ * iY * iX;
  const int grid = grid_n(n, 256);
  cudaStream_t st = as_stream(stream);
  switch (dtype) {
    case SI_U8: acwe_minmax_kernel<uint8_t><<<grid, 256, 0, st>>>((const uint8_t*)img, f, mm); break;
    case SI_I8: acwe_minmax_kernel<int8_t><<<grid, 256, 0, st>>>((const int8_t*)img, f, mm); break;
    case SI_U16: acwe_minmax_kernel<uint16_t><<<grid, 256, 0, st>>>((const uint16_t*)img, f, mm); break;
    case SI_I16: acwe_minmax_kernel<int16_t><<<grid, 256, 0, st>>>((const int16_t*)img, f, mm); break;
    case SI_I32: acwe_minmax_kernel<int32_t><<<grid, 256, 0, st>>>((const int32_t*)img, f, mm); break;
    case SI_F32: acwe_minmax_kernel<float><<<grid, 256, 0, st>>>((const float*)img, f, mm); break;
    default: return set_error(SI_ERR_ARG, "si_acwe_minmax: unsupported dtype %d", dtype);
  }
  return check_launch("si_acwe_minmax");
}

extern "C" int si_acwe_gather(const void* img, int dtype, int iZ, int iY, int iX, int iz0, int iy0, int ix0,
                              int convert, float mn, float mx, const uint8_t* labels, int Z, int Y, int X, int cz0,
                              int cy0, int cx0, int cZ, int cY, int cX, uint8_t* D, uint8_t* L, void* stream) {
  clear_error();
  if (!img || !labels || !D || !L) return set_error(SI_ERR_ARG, "si_acwe_gather: null pointer");
  const CropBox cb{cz0, cy0, cx0, cZ, cY, cX};
  if (iZ < 1 || iY < 1 || iX < 1 || Z < 1 || Y < 1 || X < 1 || !crop_ok(cb))
    return set_error(SI_ERR_ARG, "si_acwe_gather: bad dimensions");
  if (!convert && dtype != SI_U8) return set_error(SI_ERR_ARG, "si_acwe_gather: only uint8 images are copied");
  const Frame f{iZ, iY, iX, iz0, iy0, ix0, Z, Y, X};
  const int grid = grid_n((uint64_t)cZ * cY * cX, 256);
  cudaStream_t st = as_stream(stream);
  switch (dtype) {
    case SI_U8:
      acwe_gather_kernel<uint8_t><<<grid, 256, 0, st>>>((const uint8_t*)img, f, convert, mn, mx, labels, cb, D, L);
      break;
    case SI_I8:
      acwe_gather_kernel<int8_t><<<grid, 256, 0, st>>>((const int8_t*)img, f, convert, mn, mx, labels, cb, D, L);
      break;
    case SI_U16:
      acwe_gather_kernel<uint16_t><<<grid, 256, 0, st>>>((const uint16_t*)img, f, convert, mn, mx, labels, cb, D, L);
      break;
    case SI_I16:
      acwe_gather_kernel<int16_t><<<grid, 256, 0, st>>>((const int16_t*)img, f, convert, mn, mx, labels, cb, D, L);
      break;
    case SI_I32:
      acwe_gather_kernel<int32_t><<<grid, 256, 0, st>>>((const int32_t*)img, f, convert, mn, mx, labels, cb, D, L);
      break;
    case SI_F32:
      acwe_gather_kernel<float><<<grid, 256, 0, st>>>((const float*)img, f, convert, mn, mx, labels, cb, D, L);
      break;
    default: return set_error(SI_ERR_ARG, "si_acwe_gather: unsupported dtype %d", dtype);
  }
  return check_launch("si_acwe_gather");
}

extern "C" int si_acwe_label_sums(const uint8_t* D, const uint8_t* L, uint64_t n, unsigned long long* sums,
                                  void* stream) {
  clear_error();
  if (!D || !L || !sums) return set_error(SI_ERR_ARG, "si_acwe_label_sums: null pointer");
  if (n == 0) return SI_OK;
  // a CTA's 32-bit intensity sums hold at most 2^32 / 255 voxels
  uint64_t grid = (uint64_t)grid_n((n + 15) / 16, 256);
  const uint64_t per_cta_cap = 1ull << 24;
  if ((n + grid - 1) / grid > per_cta_cap) grid = (n + per_cta_cap - 1) / per_cta_cap;
  if (grid > 0x7fffffffull) return set_error(SI_ERR_LIMIT, "si_acwe_label_sums: volume too large");
  acwe_label_sums_kernel<<<(unsigned)grid, 256, 0, as_stream(stream)>>>(D, L, n, sums);
  return check_launch("si_acwe_label_sums");
}

extern "C" int si_acwe_evolution(const uint8_t* L, const uint8_t* D, const unsigned long long* sums, double alpha,
                                 int Z, int Y, int X, uint8_t* out, void* stream) {
  clear_error();
  if (!L || !D || !sums || !out) return set_error(SI_ERR_ARG, "si_acwe_evolution: null pointer");
  if (!dims_ok(Z, Y, X)) return set_error(SI_ERR_ARG, "si_acwe_evolution: bad dimensions");
  if (out == L) return set_error(SI_ERR_ARG, "si_acwe_evolution: out must not alias L");
  return stencil_pass(kEvolution, L, D, sums, alpha, 0, Z, Y, X, out, as_stream(stream));
}

extern "C" int si_acwe_morph(const uint8_t* src, int Z, int Y, int X, int label, int erode, uint8_t* dst,
                             void* stream) {
  clear_error();
  if (!src || !dst) return set_error(SI_ERR_ARG, "si_acwe_morph: null pointer");
  if (!dims_ok(Z, Y, X) || label < 0 || label > 255) return set_error(SI_ERR_ARG, "si_acwe_morph: bad arguments");
  if (src == dst) return set_error(SI_ERR_ARG, "si_acwe_morph: dst must not alias src");
  return stencil_pass(erode ? kErosion : kDilation, src, nullptr, nullptr, 0.0, label, Z, Y, X, dst,
                      as_stream(stream));
}

extern "C" int si_acwe_curvop(uint8_t* L, uint8_t* tmp, int Z, int Y, int X, int label, int steps, void* stream) {
  clear_error();
  if (!L || !tmp) return set_error(SI_ERR_ARG, "si_acwe_curvop: null pointer");
  if (!dims_ok(Z, Y, X) || label < 0 || label > 255 || steps < 0)
    return set_error(SI_ERR_ARG, "si_acwe_curvop: bad arguments");
  if (L == tmp) return set_error(SI_ERR_ARG, "si_acwe_curvop: tmp must not alias L");
  cudaStream_t st = as_stream(stream);
  if (steps == 0) return SI_OK;
  // bit masks when two of them fit in tmp (rows of at least ~8 voxels):
  // one pack, then every pass in place on L
  const int W = (X + 31) / 32;
  const size_t words = (size_t)Z * Y * W;
  const size_t mbytes = (words * sizeof(uint32_t) + 255) / 256 * 256;
  if (2 * mbytes <= (size_t)Z * Y * X && (reinterpret_cast<uintptr_t>(tmp) & 255u) == 0) {
    uint32_t* M[2] = {reinterpret_cast<uint32_t*>(tmp), reinterpret_cast<uint32_t*>(tmp + mbytes)};
    const int rows_grid = grid_n((uint64_t)Z * Y * 32, 256);
    acwe_pack_kernel<<<rows_grid, 256, 0, st>>>(L, Z, Y, X, W, label, M[0]);
    const int g = grid_n(words, 256);
    int p = 0;
    for (int k = 0; k < steps; ++k) {
      for (int h = 0; h < 2; ++h) {
        const bool erode = (k % 2 == 0) == (h == 0);
        if (erode)
          acwe_morph_bits_kernel<true><<<g, 256, 0, st>>>(L, M[p], M[p ^ 1], Z, Y, X, W, label);
        else
          acwe_morph_bits_kernel<false><<<g, 256, 0, st>>>(L, M[p], M[p ^ 1], Z, Y, X, W, label);
        p ^= 1;
      }
    }
    return check_launch("si_acwe_curvop");
  }
  uint8_t* buf[2] = {L, tmp};
  int p = 0;
  for (int k = 0; k < steps; ++k) {
    const int first = (k % 2 == 0) ? kErosion : kDilation;
    const int second = (k % 2 == 0) ? kDilation : kErosion;
    for (int op : {first, second}) {
      const int rc = stencil_pass(op, buf[p], nullptr, nullptr, 0.0, label, Z, Y, X, buf[p ^ 1], st);
      if (rc) return rc;
      p ^= 1;
    }
  }
  return SI_OK;  // an even number of passes: the result is back in L
}

extern "C" int si_acwe_scatter(const uint8_t* L, int cz0, int cy0, int cx0, int cZ, int cY, int cX, int Z, int Y,
                               int X, uint8_t* out, void* stream) {
  clear_error();
  if (!L || !out) return set_error(SI_ERR_ARG, "si_acwe_scatter: null pointer");
  const CropBox cb{cz0, cy0, cx0, cZ, cY, cX};
  if (Z < 1 || Y < 1 || X < 1 || !crop_ok(cb)) return set_error(SI_ERR_ARG, "si_acwe_scatter: bad dimensions");
  const uint64_t n = (uint64_t)Z * Y * X;
  acwe_scatter_kernel<<<grid_n(n, 256), 256, 0, as_stream(stream)>>>(L, cb, Z, Y, X, out);
  return check_launch("si_acwe_scatter");
}

extern "C" int si_acwe_dist_init(const uint8_t* L, uint64_t n, float* dist, void* stream) {
  clear_error();
  if (!L || !dist) return set_error(SI_ERR_ARG, "si_acwe_dist_init: null pointer");
  if (n == 0) return SI_OK;
  acwe_dist_init_kernel<<<grid_n(n, 256), 256, 0, as_stream(stream)>>>(L, n, dist);
  return check_launch("si_acwe_dist_init");
}

extern "C" int si_acwe_chamfer_band(float* dist, float* tmp, int Z, int Y, int X, void* stream) {
  clear_error();
  if (!dist || !tmp) return set_error(SI_ERR_ARG, "si_acwe_chamfer_band: null pointer");
  if (!dims_ok(Z, Y, X) || dist == tmp) return set_error(SI_ERR_ARG, "si_acwe_chamfer_band: bad arguments");
  cudaStream_t st = as_stream(stream);
  const dim3 block(kTX, kTY);
  const dim3 grid((X + kTX - 1) / kTX, (Y + kTY - 1) / kTY, (Z + kZChunk - 1) / kZChunk);
  float* buf[2] = {dist, tmp};
  for (int k = 0; k < 10; ++k)  // an even number of passes: the result is back in dist
    acwe_chamfer_pass_kernel<<<grid, block, 0, st>>>(buf[k & 1], Z, Y, X, buf[(k + 1) & 1]);
  return check_launch("si_acwe_chamfer_band");
}

extern "C" int si_acwe_refine_hist(const float* dist, const uint8_t* D, const uint8_t* L, const int16_t* class_lut,
                                   int ncls, int Z, int Y, int X, uint32_t* hist, void* stream) {
  clear_error();
  if (!dist || !D || !L || !class_lut || !hist) return set_error(SI_ERR_ARG, "si_acwe_refine_hist: null pointer");
  if (ncls < 1 || ncls > 257 || Z < 1 || Y < 1 || X < 1 || Z > 65535)
    return set_error(SI_ERR_ARG, "si_acwe_refine_hist: bad arguments");
  const uint64_t YX = (uint64_t)Y * X;
  const int use_smem = ncls <= 48;
  const size_t smem = use_smem ? (size_t)ncls * 256 * sizeof(uint32_t) : 0;
  uint64_t bx = (YX + 4095) / 4096;
  if (bx > 64) bx = 64;
  const dim3 grid((unsigned)bx, (unsigned)Z);
  acwe_band_hist_kernel<<<grid, 256, smem, as_stream(stream)>>>(dist, D, L, class_lut, ncls, Y, X, use_smem, hist);
  return check_launch("si_acwe_refine_hist");
}

extern "C" int si_acwe_refine_decide(const uint32_t* hist, const uint8_t* cand_label, int ncand, int Z,
                                     uint8_t* lut, void* stream) {
  clear_error();
  if (!hist || !lut || (ncand > 0 && !cand_label)) return set_error(SI_ERR_ARG, "si_acwe_refine_decide: null pointer");
  if (ncand < 0 || ncand > 256 || Z < 1) return set_error(SI_ERR_ARG, "si_acwe_refine_decide: bad arguments");
  acwe_refine_decide_kernel<<<Z, 256, 0, as_stream(stream)>>>(hist, cand_label, ncand, lut);
  return check_launch("si_acwe_refine_decide");
}

extern "C" int si_acwe_refine_apply(const float* dist, const uint8_t* D, const uint8_t* lut, int cz0, int cy0,
                                    int cx0, int cZ, int cY, int cX, int Z, int Y, int X, uint8_t* out,
                                    void* stream) {
  clear_error();
  if (!dist || !D || !lut || !out) return set_error(SI_ERR_ARG, "si_acwe_refine_apply: null pointer");
  const CropBox cb{cz0, cy0, cx0, cZ, cY, cX};
  if (Z < 1 || Y < 1 || X < 1 || !crop_ok(cb)) return set_error(SI_ERR_ARG, "si_acwe_refine_apply: bad dimensions");
  const uint64_t n = (uint64_t)Z * Y * X;
  acwe_refine_apply_kernel<<<grid_n(n, 256), 256, 0, as_stream(stream)>>>(dist, D, lut, cb, Z, Y, X, out);
  return check_launch("si_acwe_refine_apply");
}
