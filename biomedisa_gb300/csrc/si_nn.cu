// Kernels of the learned surrogate: a 3-D convolutional network over NDHWC
// bfloat16 activations with fp32 accumulation on the tensor cores
// (mma.sync m16n8k16 bf16), its backward pass, the soft-target
// cross-entropy loss, AdamW, and the feature/label plumbing of training and
// inference. Convolutions are 3x3x3, stride 1, zero padding = dilation
// ("same" size), written as implicit GEMMs:
//   forward   Y[v][co]  = sum_{tap, ci} X[v + d*off(tap)][ci] * W[tap][co][ci]
//   data grad dX = the same convolution of dY with W'[tap][ci][co] = W[26 - tap][co][ci]
//   weight    dW[tap][co][ci] = sum_v dY[v][co] * X[v + d*off(tap)][ci]
// Channel counts are multiples of 16 (padding channels carry zeros).
#include <cuda_bf16.h>

#include "si_common.cuh"
#include "si_internal.h"

namespace si {
namespace {

struct Vol5 {
  int N, D, H, W;
};

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// voxel index -> (n, z, y, x)
__device__ __forceinline__ void decomp(const Vol5& g, int64_t v, int& n, int& z, int& y, int& x) {
  x = (int)(v % g.W);
  int64_t t = v / g.W;
  y = (int)(t % g.H);
  t /= g.H;
  z = (int)(t % g.D);
  n = (int)(t / g.D);
}

// ---------------------------------------------------------------------------
// Forward convolution. A warp computes 16 voxels x kCout channels; a block of
// 4 warps 64 voxels. Epilogue: + bias, + residual, ReLU, store bf16 or fp32.
// ---------------------------------------------------------------------------
template <int kCout, bool kOutF32>
__global__ void __launch_bounds__(128) conv3d_fwd_kernel(const __nv_bfloat16* __restrict__ x,
                                                         const __nv_bfloat16* __restrict__ w,
                                                         const float* __restrict__ bias,
                                                         const __nv_bfloat16* __restrict__ residual, void* y_out,
                                                         Vol5 g, int cin, int dil, int relu) {
  constexpr int NT = kCout / 8;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = lane >> 2, tig = lane & 3;
  const int64_t V = (int64_t)g.N * g.D * g.H * g.W;
  const int64_t v0 = ((int64_t)blockIdx.x * 4 + warp) * 16;
  if (v0 >= V) return;
  const int64_t r0 = v0 + grp, r1 = v0 + grp + 8;
  int n0, z0, y0, x0, n1, z1, y1, x1;
  const bool ok0 = r0 < V, ok1 = r1 < V;
  decomp(g, ok0 ? r0 : 0, n0, z0, y0, x0);
  decomp(g, ok1 ? r1 : 0, n1, z1, y1, x1);
  float acc[NT][4];
#pragma unroll
  for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
  for (int tap = 0; tap < 27; ++tap) {
    const int dz = (tap / 9 - 1) * dil, dy = ((tap / 3) % 3 - 1) * dil, dx = (tap % 3 - 1) * dil;
    const int za = z0 + dz, ya = y0 + dy, xa = x0 + dx;
    const int zb = z1 + dz, yb = y1 + dy, xb = x1 + dx;
    const bool in0 = ok0 && (unsigned)za < (unsigned)g.D && (unsigned)ya < (unsigned)g.H && (unsigned)xa < (unsigned)g.W;
    const bool in1 = ok1 && (unsigned)zb < (unsigned)g.D && (unsigned)yb < (unsigned)g.H && (unsigned)xb < (unsigned)g.W;
    const __nv_bfloat16* p0 = x + ((((int64_t)n0 * g.D + za) * g.H + ya) * g.W + xa) * cin;
    const __nv_bfloat16* p1 = x + ((((int64_t)n1 * g.D + zb) * g.H + yb) * g.W + xb) * cin;
    const __nv_bfloat16* wt = w + (int64_t)tap * kCout * cin;
    for (int ci0 = 0; ci0 < cin; ci0 += 16) {
      uint32_t a[4];
      a[0] = in0 ? ld32(p0 + ci0 + tig * 2) : 0u;
      a[1] = in1 ? ld32(p1 + ci0 + tig * 2) : 0u;
      a[2] = in0 ? ld32(p0 + ci0 + tig * 2 + 8) : 0u;
      a[3] = in1 ? ld32(p1 + ci0 + tig * 2 + 8) : 0u;
#pragma unroll
      for (int j = 0; j < NT; ++j) {
        const __nv_bfloat16* wb = wt + (int64_t)(j * 8 + grp) * cin + ci0 + tig * 2;
        mma_bf16(acc[j], a, ld32(wb), ld32(wb + 8));
      }
    }
  }
#pragma unroll
  for (int j = 0; j < NT; ++j) {
    const int co = j * 8 + tig * 2;
    float b0 = bias ? bias[co] : 0.0f, b1 = bias ? bias[co + 1] : 0.0f;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t r = h ? r1 : r0;
      if (r >= V) continue;
      float u0 = acc[j][2 * h] + b0, u1 = acc[j][2 * h + 1] + b1;
      if (residual) {
        const __nv_bfloat162 rr = *reinterpret_cast<const __nv_bfloat162*>(residual + r * kCout + co);
        u0 += __bfloat162float(rr.x);
        u1 += __bfloat162float(rr.y);
      }
      if (relu) {
        u0 = fmaxf(u0, 0.0f);
        u1 = fmaxf(u1, 0.0f);
      }
      if (kOutF32) {
        *reinterpret_cast<float2*>(static_cast<float*>(y_out) + r * kCout + co) = make_float2(u0, u1);
      } else {
        *reinterpret_cast<__nv_bfloat162*>(static_cast<__nv_bfloat16*>(y_out) + r * kCout + co) =
            __floats2bfloat162_rn(u0, u1);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// 16 -> 16 channel forward convolution (the whole C = 16 network and its data
// gradient). A warp computes 64 consecutive voxels of one x-row (four 16-voxel
// m-tiles) x 16 output channels. The K order inside each m16n8k16 step is
// permuted so that a lane's four A values are four consecutive channels of
// one voxel: k = 2*tig + e -> channel 4*tig + e and k = 2*tig + 8 + e ->
// channel 4*tig + 2 + e (e = 0, 1). The same permutation applied to B makes
// both operands one 8-byte load each: A from global memory (the next tap's
// loads issued before this tap's MMAs), B from the weights staged in shared
// memory once per block.
// ---------------------------------------------------------------------------
constexpr int kC16Warps = 4;

template <bool kOutF32>
__global__ void __launch_bounds__(kC16Warps * 32, 4) conv16_kernel(const __nv_bfloat16* __restrict__ x,
                                                                const __nv_bfloat16* __restrict__ w,
                                                                const float* __restrict__ bias,
                                                                const __nv_bfloat16* __restrict__ residual,
                                                                void* y_out, Vol5 g, int dil, int relu, int xchunks) {
  __shared__ uint2 ws[27 * 16 * 4];  // [tap][co][tig]: channels 4*tig .. 4*tig + 3
  __shared__ float bs[16];
  for (int i = threadIdx.x; i < 27 * 16 * 4; i += blockDim.x) ws[i] = reinterpret_cast<const uint2*>(w)[i];
  if (threadIdx.x < 16) bs[threadIdx.x] = bias ? bias[threadIdx.x] : 0.0f;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = lane >> 2, tig = lane & 3;
  const int64_t rows = (int64_t)g.N * g.D * g.H * xchunks;
  const int64_t row = (int64_t)blockIdx.x * kC16Warps + warp;
  if (row >= rows) return;
  const int xc = (int)(row % xchunks);
  int64_t t = row / xchunks;
  const int yy = (int)(t % g.H);
  t /= g.H;
  const int zz = (int)(t % g.D);
  const int n = (int)(t / g.D);
  const int xb = xc * 64;

  float acc[4][2][4];
#pragma unroll
  for (int m = 0; m < 4; ++m)
#pragma unroll
    for (int j = 0; j < 2; ++j) acc[m][j][0] = acc[m][j][1] = acc[m][j][2] = acc[m][j][3] = 0.0f;

  uint2 A[2][4][2];
  auto load_tap = [&](uint2 (&dst)[4][2], int tap) {
    const int dz = (tap / 9 - 1) * dil, dy = ((tap / 3) % 3 - 1) * dil, dx = (tap % 3 - 1) * dil;
    const int zi = zz + dz, yi = yy + dy;
    const bool zy = (unsigned)zi < (unsigned)g.D && (unsigned)yi < (unsigned)g.H;
    const __nv_bfloat16* rowp =
        x + ((((int64_t)n * g.D + (zy ? zi : 0)) * g.H + (zy ? yi : 0)) * g.W) * 16 + 4 * tig;
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int xi = xb + 16 * m + 8 * h + grp + dx;
        dst[m][h] = (zy && (unsigned)xi < (unsigned)g.W) ? *reinterpret_cast<const uint2*>(rowp + (int64_t)xi * 16)
                                                         : make_uint2(0u, 0u);
      }
  };
  load_tap(A[0], 0);
#pragma unroll
  for (int tap = 0; tap < 27; ++tap) {
    if (tap + 1 < 27) load_tap(A[(tap + 1) & 1], tap + 1);
    const uint2 b0 = ws[(tap * 16 + grp) * 4 + tig];
    const uint2 b1 = ws[(tap * 16 + 8 + grp) * 4 + tig];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const uint2 lo = A[tap & 1][m][0], hi = A[tap & 1][m][1];
      const uint32_t a[4] = {lo.x, hi.x, lo.y, hi.y};
      mma_bf16(acc[m][0], a, b0.x, b0.y);
      mma_bf16(acc[m][1], a, b1.x, b1.y);
    }
  }
  const int64_t rbase = (((int64_t)n * g.D + zz) * g.H + yy) * g.W;
#pragma unroll
  for (int m = 0; m < 4; ++m)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int xo = xb + 16 * m + 8 * h + grp;
      if (xo >= g.W) continue;
      const int64_t r = rbase + xo;
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int co = j * 8 + tig * 2;
        float u0 = acc[m][j][2 * h] + bs[co], u1 = acc[m][j][2 * h + 1] + bs[co + 1];
        if (residual) {
          const __nv_bfloat162 rr = *reinterpret_cast<const __nv_bfloat162*>(residual + r * 16 + co);
          u0 += __bfloat162float(rr.x);
          u1 += __bfloat162float(rr.y);
        }
        if (relu) {
          u0 = fmaxf(u0, 0.0f);
          u1 = fmaxf(u1, 0.0f);
        }
        if (kOutF32)
          *reinterpret_cast<float2*>(static_cast<float*>(y_out) + r * 16 + co) = make_float2(u0, u1);
        else
          *reinterpret_cast<__nv_bfloat162*>(static_cast<__nv_bfloat16*>(y_out) + r * 16 + co) =
              __floats2bfloat162_rn(u0, u1);
      }
    }
}

// ---------------------------------------------------------------------------
// Weight gradient: per block a chunk of voxels, per warp a set of taps; the
// tap's [cout x cin] partial sums go to dW (fp32) with atomics.
// GEMM per tap: M = cout, N = cin, K = voxels; bf16 pairs along K are packed
// from two voxels.
// ---------------------------------------------------------------------------
constexpr int kWgradChunk = 512;

template <int kCout, int kCin>
__global__ void __launch_bounds__(128) conv3d_wgrad_kernel(const __nv_bfloat16* __restrict__ x,
                                                           const __nv_bfloat16* __restrict__ dy,
                                                           float* __restrict__ dw, Vol5 g, int dil) {
  constexpr int MT = kCout / 16, NT = kCin / 8;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = lane >> 2, tig = lane & 3;
  const int64_t V = (int64_t)g.N * g.D * g.H * g.W;
  const int64_t c0 = (int64_t)blockIdx.x * kWgradChunk;
  const int64_t c1 = c0 + kWgradChunk < V ? c0 + kWgradChunk : V;
  for (int tap = warp; tap < 27; tap += 4) {
    const int dz = (tap / 9 - 1) * dil, dyo = ((tap / 3) % 3 - 1) * dil, dx = (tap % 3 - 1) * dil;
    float acc[MT][NT][4];
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
      for (int j = 0; j < NT; ++j) acc[m][j][0] = acc[m][j][1] = acc[m][j][2] = acc[m][j][3] = 0.0f;
    for (int64_t k0 = c0; k0 < c1; k0 += 16) {
      // this thread's four voxels along K: k0 + tig*2 + {0, 1, 8, 9}
      __nv_bfloat16 const* xs[4];
      int64_t vk[4];
      bool okx[4], oky[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int64_t v = k0 + tig * 2 + (q & 1) + (q >> 1) * 8;
        vk[q] = v;
        oky[q] = v < c1;
        int n, z, yy, xx;
        decomp(g, oky[q] ? v : 0, n, z, yy, xx);
        z += dz;
        yy += dyo;
        xx += dx;
        okx[q] = oky[q] && (unsigned)z < (unsigned)g.D && (unsigned)yy < (unsigned)g.H && (unsigned)xx < (unsigned)g.W;
        xs[q] = x + ((((int64_t)n * g.D + z) * g.H + yy) * g.W + xx) * kCin;
      }
      const __nv_bfloat16 zero = __float2bfloat16(0.0f);
#pragma unroll
      for (int m = 0; m < MT; ++m) {
        // A[m = co][k = v] = dy[v][co]: rows grp and grp + 8 of the m-tile
        const int coa = m * 16 + grp, cob = coa + 8;
        uint32_t a[4];
        a[0] = pack2(oky[0] ? dy[vk[0] * kCout + coa] : zero, oky[1] ? dy[vk[1] * kCout + coa] : zero);
        a[1] = pack2(oky[0] ? dy[vk[0] * kCout + cob] : zero, oky[1] ? dy[vk[1] * kCout + cob] : zero);
        a[2] = pack2(oky[2] ? dy[vk[2] * kCout + coa] : zero, oky[3] ? dy[vk[3] * kCout + coa] : zero);
        a[3] = pack2(oky[2] ? dy[vk[2] * kCout + cob] : zero, oky[3] ? dy[vk[3] * kCout + cob] : zero);
#pragma unroll
        for (int j = 0; j < NT; ++j) {
          // B[k = v][n = ci] = x[v + off][ci], column grp of the n-tile
          const int ci = j * 8 + grp;
          const uint32_t b0 = pack2(okx[0] ? xs[0][ci] : zero, okx[1] ? xs[1][ci] : zero);
          const uint32_t b1 = pack2(okx[2] ? xs[2][ci] : zero, okx[3] ? xs[3][ci] : zero);
          mma_bf16(acc[m][j], a, b0, b1);
        }
      }
    }
    float* dwt = dw + (int64_t)tap * kCout * kCin;
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
      for (int j = 0; j < NT; ++j) {
        const int co = m * 16 + grp, ci = j * 8 + tig * 2;
        atomicAdd(&dwt[co * kCin + ci], acc[m][j][0]);
        atomicAdd(&dwt[co * kCin + ci + 1], acc[m][j][1]);
        atomicAdd(&dwt[(co + 8) * kCin + ci], acc[m][j][2]);
        atomicAdd(&dwt[(co + 8) * kCin + ci + 1], acc[m][j][3]);
      }
  }
}

// ---------------------------------------------------------------------------
// 16 x 16 weight gradient. A block of 4 warps walks a run of 64-voxel x-rows;
// per row the dY row is staged once in shared memory, and each warp handles
// the taps w, w + 4, ... : it stages the shifted X row (zeros outside the
// volume) and runs dW[tap] += dY^T X on the tensor cores, with both operands
// read K-major (K = voxels) by ldmatrix.trans. Rows are 32 bytes per voxel;
// the two 16-byte halves are swapped on every other group of four voxels so
// that the eight row addresses of one ldmatrix hit distinct banks. Each warp
// adds its fp32 partial sums to dW with atomics at the end.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int swz(int v, int h) { return (v * 2 + (h ^ ((v >> 2) & 1))) * 16; }

__device__ __forceinline__ void ldsm_x4_trans(uint32_t (&r)[4], uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}

__global__ void __launch_bounds__(128) wgrad16_kernel(const __nv_bfloat16* __restrict__ x,
                                                      const __nv_bfloat16* __restrict__ dy, float* __restrict__ dw,
                                                      float* __restrict__ partials, Vol5 g, int dil, int xchunks,
                                                      int64_t rows_per_block) {
  __shared__ __align__(16) uint8_t s_dy[64 * 32];
  __shared__ __align__(16) uint8_t s_x[4][64 * 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t rows = (int64_t)g.N * g.D * g.H * xchunks;
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_block;
  const int64_t r1 = r0 + rows_per_block < rows ? r0 + rows_per_block : rows;
  float acc[7][2][4];
#pragma unroll
  for (int i = 0; i < 7; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.0f;
  const uint32_t sdy = (uint32_t)__cvta_generic_to_shared(s_dy);
  const uint32_t sx = (uint32_t)__cvta_generic_to_shared(s_x[warp]);
  // ldmatrix row addresses: matrix q = lane / 8, row i = lane % 8.
  // A = dY^T (co x v): q0 (v 0-7, co 0-7), q1 (v 0-7, co 8-15), q2 (v 8-15, co 0-7), q3 (v 8-15, co 8-15)
  // B = X (v x ci):    q0 (v 0-7, ci 0-7), q1 (v 8-15, ci 0-7), q2 (v 0-7, ci 8-15), q3 (v 8-15, ci 8-15)
  const int q = lane >> 3, i8 = lane & 7;
  const int va = i8 + ((q >> 1) << 3), ha = q & 1;
  const int vb = i8 + ((q & 1) << 3), hb = q >> 1;
  for (int64_t row = r0; row < r1; ++row) {
    const int xc = (int)(row % xchunks);
    int64_t t = row / xchunks;
    const int yy = (int)(t % g.H);
    t /= g.H;
    const int zz = (int)(t % g.D);
    const int n = (int)(t / g.D);
    const int xb = xc * 64;
    const int64_t base = (((int64_t)n * g.D + zz) * g.H + yy) * g.W;
    __syncthreads();  // previous row's dY no longer read
    {
      const int qq = threadIdx.x;  // 128 threads x 16 bytes = one 64-voxel row of dY
      const int v = qq >> 1, h = qq & 1;
      uint4 val = make_uint4(0u, 0u, 0u, 0u);
      if (xb + v < g.W) val = *reinterpret_cast<const uint4*>(dy + (base + xb + v) * 16 + h * 8);
      *reinterpret_cast<uint4*>(s_dy + swz(v, h)) = val;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 7; ++i) {
      const int tap = warp + 4 * i;
      if (tap >= 27) break;
      const int dz = (tap / 9 - 1) * dil, dyo = ((tap / 3) % 3 - 1) * dil, dx = (tap % 3 - 1) * dil;
      const int zi = zz + dz, yi = yy + dyo;
      const bool zy = (unsigned)zi < (unsigned)g.D && (unsigned)yi < (unsigned)g.H;
      const __nv_bfloat16* xrow = x + (((int64_t)n * g.D + (zy ? zi : 0)) * g.H + (zy ? yi : 0)) * g.W * 16;
      __syncwarp();
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int qq = lane + 32 * k;
        const int v = qq >> 1, h = qq & 1;
        const int xi = xb + v + dx;
        uint4 val = make_uint4(0u, 0u, 0u, 0u);
        if (zy && xb + v < g.W && (unsigned)xi < (unsigned)g.W)
          val = *reinterpret_cast<const uint4*>(xrow + (int64_t)xi * 16 + h * 8);
        *reinterpret_cast<uint4*>(s_x[warp] + swz(v, h)) = val;
      }
      __syncwarp();
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) {
        uint32_t a[4], b[4];
        ldsm_x4_trans(a, sdy + swz(ks * 16 + va, ha));
        ldsm_x4_trans(b, sx + swz(ks * 16 + vb, hb));
        mma_bf16(acc[i][0], a, b[0], b[1]);
        mma_bf16(acc[i][1], a, b[2], b[3]);
      }
    }
  }
  const int grp = lane >> 2, tig = lane & 3;
#pragma unroll
  for (int i = 0; i < 7; ++i) {
    const int tap = warp + 4 * i;
    if (tap >= 27) break;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int ci = j * 8 + tig * 2;
      if (partials) {  // deterministic: this block's sums, reduced in block order by reduce_partials_kernel
        float* d = partials + ((int64_t)blockIdx.x * 27 + tap) * 256;
        *reinterpret_cast<float2*>(&d[grp * 16 + ci]) = make_float2(acc[i][j][0], acc[i][j][1]);
        *reinterpret_cast<float2*>(&d[(grp + 8) * 16 + ci]) = make_float2(acc[i][j][2], acc[i][j][3]);
      } else {
        float* d = dw + tap * 256;
        atomicAdd(&d[grp * 16 + ci], acc[i][j][0]);
        atomicAdd(&d[grp * 16 + ci + 1], acc[i][j][1]);
        atomicAdd(&d[(grp + 8) * 16 + ci], acc[i][j][2]);
        atomicAdd(&d[(grp + 8) * 16 + ci + 1], acc[i][j][3]);
      }
    }
  }
}

// W'[tap][ci][co] = W[26 - tap][co][ci]
__global__ void flip_weights_kernel(const __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ wf, int cout,
                                    int cin) {
  const int n = 27 * cout * cin;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int tap = i / (cout * cin);
    const int r = i - tap * cout * cin;
    const int co = r / cin, ci = r - co * cin;
    wf[((int64_t)tap * cin + ci) * cout + co] = w[((int64_t)(26 - tap) * cout + co) * cin + ci];
  }
}

// bias gradient: db[c] += sum_v dy[v][c]. Each thread sums a fixed set of
// voxels, warps reduce by shuffles and the block's warps in order; with
// `partials` the block writes its sums (reduced in block order afterwards),
// otherwise it adds them to db atomically.
template <int kC>
__global__ void __launch_bounds__(256) bias_grad_kernel(const __nv_bfloat16* __restrict__ dy, int64_t V,
                                                        float* __restrict__ db, float* __restrict__ partials) {
  __shared__ float s_sum[8][kC];
  float acc[kC];
#pragma unroll
  for (int c = 0; c < kC; ++c) acc[c] = 0.0f;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    const __nv_bfloat16* row = dy + v * kC;
#pragma unroll
    for (int c = 0; c < kC; ++c) acc[c] += __bfloat162float(row[c]);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < kC; ++c) {
    float s = acc[c];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) s_sum[warp][c] = s;
  }
  __syncthreads();
  if (threadIdx.x < kC) {
    float s = 0.0f;
    for (int w = 0; w < 8; ++w) s += s_sum[w][threadIdx.x];
    if (partials)
      partials[(int64_t)blockIdx.x * kC + threadIdx.x] = s;
    else
      atomicAdd(&db[threadIdx.x], s);
  }
}

// out[i] += sum_b partials[b][i] (n outputs, nb blocks). One warp per
// output: lane l sums b = l, l + 32, ... in order, then a fixed shuffle tree
// combines the lanes, so the result does not depend on scheduling.
__global__ void __launch_bounds__(256) reduce_partials_kernel(const float* __restrict__ partials, int nb, int n,
                                                              float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    float s = 0.0f;
    for (int b = lane; b < nb; b += 32) s += partials[(int64_t)b * n + i];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[i] += s;
  }
}

// g *= (y > 0); optionally also out = g_masked + add
__global__ void __launch_bounds__(256) relu_bwd_kernel(__nv_bfloat16* __restrict__ g,
                                                       const __nv_bfloat16* __restrict__ y,
                                                       const __nv_bfloat16* __restrict__ add, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float v = __bfloat162float(y[i]) > 0.0f ? __bfloat162float(g[i]) : 0.0f;
    if (add) v += __bfloat162float(add[i]);
    g[i] = __float2bfloat16(v);
  }
}

// Soft-target cross entropy over the first nol of C logit channels.
// loss += sum_v w_v * sum_l -p_l log softmax(z)_l ; dz = w_v * (softmax - p) * scale
__global__ void __launch_bounds__(256) xent_kernel(const float* __restrict__ logits, const float* __restrict__ target,
                                                   const float* __restrict__ weight, int64_t V, int C, int nol,
                                                   float scale, __nv_bfloat16* __restrict__ dlogits,
                                                   float* __restrict__ loss) {
  float local = 0.0f;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    const float* z = logits + v * C;
    const float* p = target + v * nol;
    const float wv = weight ? weight[v] : 1.0f;
    float m = -INFINITY;
    for (int l = 0; l < nol; ++l) m = fmaxf(m, z[l]);
    float s = 0.0f;
    for (int l = 0; l < nol; ++l) s += __expf(z[l] - m);
    const float lse = m + __logf(s);
    for (int l = 0; l < C; ++l) {
      float d = 0.0f;
      if (l < nol) {
        const float q = __expf(z[l] - lse);
        local += -wv * p[l] * (z[l] - lse);
        d = wv * (q - p[l]) * scale;
      }
      dlogits[v * C + l] = __float2bfloat16(d);
    }
  }
  for (int o = 16; o; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, local);
}

// AdamW on fp32 master weights; writes the bf16 working copy.
__global__ void __launch_bounds__(256) adamw_kernel(float* __restrict__ p, const float* __restrict__ g,
                                                    float* __restrict__ m, float* __restrict__ v,
                                                    __nv_bfloat16* __restrict__ p_bf16, int64_t n, float lr,
                                                    float b1, float b2, float eps, float wd, float bc1, float bc2) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float pi = p[i] * (1.0f - lr * wd);
    pi -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    p[i] = pi;
    if (p_bf16) p_bf16[i] = __float2bfloat16(pi);
  }
}

// Surrogate input features of a uint8 working volume (one crop), NDHWC bf16
// with 16 channels: [0] I / 255, [1] signed distance to the nearest labelled
// z-slice / 16 (clamped to [-1, 1]), [2] 1 on seed voxels, [3 + s] the linear
// interpolation along z of label slot s's seed indicator between the
// labelled z-slices below and above (s < kFeatSlots):
//   w_lo [slot(z_lo, y, x) == s] + (1 - w_lo) [slot(z_hi, y, x) == s].
// zinfo[z] = {distance, z_lo, z_hi, w_lo} (z_lo / z_hi = -1: none). Outside
// the crop: [1] = 1, all else 0.
constexpr int kFeatSlots = 13;

__global__ void __launch_bounds__(256) features_kernel(const uint8_t* __restrict__ img,
                                                       const int16_t* __restrict__ slot_map,
                                                       const float4* __restrict__ zinfo, int D, int H, int W,
                                                       int z0, int y0, int x0, int Dt, int Ht, int Wt,
                                                       __nv_bfloat16* __restrict__ out) {
  const int64_t n = (int64_t)Dt * Ht * Wt;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int xt = (int)(i % Wt);
    const int64_t t = i / Wt;
    const int yt = (int)(t % Ht);
    const int zt = (int)(t / Ht);
    const int z = z0 + zt, y = y0 + yt, x = x0 + xt;
    float f[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) f[c] = 0.0f;
    f[1] = 1.0f;
    if ((unsigned)z < (unsigned)D && (unsigned)y < (unsigned)H && (unsigned)x < (unsigned)W) {
      const int64_t p = ((int64_t)z * H + y) * W + x;
      const float4 zi = zinfo[z];
      f[0] = img[p] * (1.0f / 255.0f);
      f[1] = fminf(fmaxf(zi.x * (1.0f / 16.0f), -1.0f), 1.0f);
      if (slot_map[p] >= 0) f[2] = 1.0f;
      const int zlo = (int)zi.y, zhi = (int)zi.z;
      const int plo = zlo >= 0 ? slot_map[((int64_t)zlo * H + y) * W + x] : -1;
      const int phi = zhi >= 0 ? slot_map[((int64_t)zhi * H + y) * W + x] : -1;
#pragma unroll
      for (int s = 0; s < kFeatSlots; ++s) f[3 + s] = (plo == s ? zi.w : 0.0f) + (phi == s ? 1.0f - zi.w : 0.0f);
    }
    uint32_t wv[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) wv[c] = pack2(__float2bfloat16(f[2 * c]), __float2bfloat16(f[2 * c + 1]));
    uint4* o = reinterpret_cast<uint4*>(out + i * 16);
    o[0] = make_uint4(wv[0], wv[1], wv[2], wv[3]);
    o[1] = make_uint4(wv[4], wv[5], wv[6], wv[7]);
  }
}

// Softmax of fp32 logits [Ds][H*W][16] over the first nol channels, for slab
// planes [zb, ze), written planar: probs[l][zo + z - zb][y][x].
__global__ void __launch_bounds__(256) probs_kernel(const float* __restrict__ logits, int64_t plane, int zb, int ze,
                                                    int nol, float* __restrict__ probs, int64_t label_stride,
                                                    int zo) {
  const int64_t n = (int64_t)(ze - zb) * plane;
  const float* base = logits + (int64_t)zb * plane * 16;
  float* obase = probs + (int64_t)zo * plane;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float z[16];
    const float4* q = reinterpret_cast<const float4*>(base + i * 16);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float4 v = q[k];
      z[4 * k] = v.x;
      z[4 * k + 1] = v.y;
      z[4 * k + 2] = v.z;
      z[4 * k + 3] = v.w;
    }
    float m = -INFINITY;
#pragma unroll
    for (int l = 0; l < 16; ++l)
      if (l < nol) m = fmaxf(m, z[l]);
    float sum = 0.0f;
#pragma unroll
    for (int l = 0; l < 16; ++l)
      if (l < nol) {
        z[l] = expf(z[l] - m);
        sum += z[l];
      }
    const float inv = 1.0f / sum;
#pragma unroll
    for (int l = 0; l < 16; ++l)
      if (l < nol) obase[l * label_stride + i] = z[l] * inv;
  }
}

inline int egrid(int64_t n) {
  const int64_t want = (n + 255) / 256, cap = (int64_t)sm_count() * 16;
  return (int)(want < cap ? (want > 0 ? want : 1) : cap);
}

}  // namespace
}  // namespace si

using namespace si;

extern "C" int si_nn_conv3d_fwd(const void* x, const void* w, const float* bias, const void* residual, void* y,
                                int N, int D, int H, int W, int cin, int cout, int dil, int relu, int out_f32,
                                void* stream) {
  clear_error();
  if (!x || !w || !y) return set_error(SI_ERR_ARG, "si_nn_conv3d_fwd: null pointer");
  if (N < 1 || D < 1 || H < 1 || W < 1 || cin < 16 || cin % 16 || dil < 1)
    return set_error(SI_ERR_ARG, "si_nn_conv3d_fwd: bad shape (cin must be a multiple of 16)");
  const int64_t V = (int64_t)N * D * H * W;
  const Vol5 g{N, D, H, W};
  const int grid = (int)((V + 63) / 64);
  cudaStream_t st = as_stream(stream);
  const auto* xb = static_cast<const __nv_bfloat16*>(x);
  const auto* wb = static_cast<const __nv_bfloat16*>(w);
  const auto* rb = static_cast<const __nv_bfloat16*>(residual);
  const bool aligned = ((uintptr_t)x % 16 == 0) && ((uintptr_t)w % 16 == 0) && ((uintptr_t)y % 16 == 0) &&
                       ((uintptr_t)residual % 16 == 0);
  if (cin == 16 && cout == 16 && aligned) {
    const int xchunks = (W + 63) / 64;
    const int64_t rows = (int64_t)N * D * H * xchunks;
    const int64_t blocks = (rows + kC16Warps - 1) / kC16Warps;
    if (blocks > 0x7fffffffLL) return set_error(SI_ERR_ARG, "si_nn_conv3d_fwd: volume too large");
    if (out_f32)
      conv16_kernel<true><<<(unsigned)blocks, kC16Warps * 32, 0, st>>>(xb, wb, bias, rb, y, g, dil, relu, xchunks);
    else
      conv16_kernel<false><<<(unsigned)blocks, kC16Warps * 32, 0, st>>>(xb, wb, bias, rb, y, g, dil, relu, xchunks);
    return check_launch("si_nn_conv3d_fwd");
  }
#define SI_CONV(CO)                                                                                              \
  if (out_f32)                                                                                                   \
    conv3d_fwd_kernel<CO, true><<<grid, 128, 0, st>>>(xb, wb, bias, rb, y, g, cin, dil, relu);                   \
  else                                                                                                           \
    conv3d_fwd_kernel<CO, false><<<grid, 128, 0, st>>>(xb, wb, bias, rb, y, g, cin, dil, relu);
  switch (cout) {
    case 16: SI_CONV(16) break;
    case 32: SI_CONV(32) break;
    case 48: SI_CONV(48) break;
    case 64: SI_CONV(64) break;
    default:
      return set_error(SI_ERR_ARG, "si_nn_conv3d_fwd: cout must be 16, 32, 48 or 64");
  }
#undef SI_CONV
  return check_launch("si_nn_conv3d_fwd");
}

extern "C" int si_nn_conv16_tc(const void* x, const void* w, const float* bias, const void* residual, void* y, int N,
                               int D, int H, int W, int dil, int relu, int out_f32, void* stream) {
  clear_error();
  if (!x || !w || !y) return set_error(SI_ERR_ARG, "si_nn_conv16_tc: null pointer");
  if (N < 1 || D < 1 || H < 1 || W < 1) return set_error(SI_ERR_ARG, "si_nn_conv16_tc: bad shape");
  if (((uintptr_t)x | (uintptr_t)w | (uintptr_t)y | (uintptr_t)residual) % 16)
    return set_error(SI_ERR_ARG, "si_nn_conv16_tc: tensors must be 16-byte aligned");
  return conv16_umma(x, w, bias, residual, y, N, D, H, W, dil, relu, out_f32, as_stream(stream));
}

extern "C" int si_nn_wgrad_partial_bytes(int N, int D, int H, int W, int cin, int cout, uint64_t* bytes) {
  clear_error();
  if (!bytes || N < 1 || D < 1 || H < 1 || W < 1 || cin < 1 || cout < 1)
    return set_error(SI_ERR_ARG, "si_nn_wgrad_partial_bytes: bad arguments");
  const int64_t V = (int64_t)N * D * H * W;
  const int64_t wblocks = (int64_t)sm_count() * 8;
  const int64_t bblocks = egrid(V);
  *bytes = (uint64_t)(wblocks * 27 * cout * cin + bblocks * cout) * sizeof(float);
  return 0;
}

extern "C" int si_nn_conv3d_wgrad(const void* x, const void* dy, float* dw, float* db, int N, int D, int H, int W,
                                  int cin, int cout, int dil, float* partials, uint64_t partial_bytes,
                                  void* stream) {
  clear_error();
  if (!x || !dy || !dw) return set_error(SI_ERR_ARG, "si_nn_conv3d_wgrad: null pointer");
  if (N < 1 || D < 1 || H < 1 || W < 1 || dil < 1) return set_error(SI_ERR_ARG, "si_nn_conv3d_wgrad: bad shape");
  const int64_t V = (int64_t)N * D * H * W;
  const Vol5 g{N, D, H, W};
  const int grid = (int)((V + kWgradChunk - 1) / kWgradChunk);
  cudaStream_t st = as_stream(stream);
  const auto* xb = static_cast<const __nv_bfloat16*>(x);
  const auto* db16 = static_cast<const __nv_bfloat16*>(dy);
  const bool aligned = ((uintptr_t)x % 16 == 0) && ((uintptr_t)dy % 16 == 0);
  const bool fast = cout == 16 && cin == 16 && aligned;
  if (partials) {
    uint64_t need = 0;
    si_nn_wgrad_partial_bytes(N, D, H, W, cin, cout, &need);
    if (!fast) return set_error(SI_ERR_ARG, "si_nn_conv3d_wgrad: deterministic partials need cin = cout = 16");
    if (partial_bytes < need || (uintptr_t)partials % 16)
      return set_error(SI_ERR_ARG, "si_nn_conv3d_wgrad: partials buffer too small or misaligned");
  }
  if (fast) {
    const int xchunks = (W + 63) / 64;
    const int64_t rows = (int64_t)N * D * H * xchunks;
    const int64_t want = (int64_t)sm_count() * 8;
    const int64_t per = (rows + want - 1) / want;
    const int64_t blocks = (rows + per - 1) / per;
    wgrad16_kernel<<<(unsigned)blocks, 128, 0, st>>>(xb, db16, dw, partials, g, dil, xchunks, per);
    if (partials)
      reduce_partials_kernel<<<27 * 256 / 8, 256, 0, st>>>(partials, (int)blocks, 27 * 256, dw);
  } else if (cout == 16 && cin == 16) conv3d_wgrad_kernel<16, 16><<<grid, 128, 0, st>>>(xb, db16, dw, g, dil);
  else if (cout == 32 && cin == 16) conv3d_wgrad_kernel<32, 16><<<grid, 128, 0, st>>>(xb, db16, dw, g, dil);
  else if (cout == 16 && cin == 32) conv3d_wgrad_kernel<16, 32><<<grid, 128, 0, st>>>(xb, db16, dw, g, dil);
  else if (cout == 32 && cin == 32) conv3d_wgrad_kernel<32, 32><<<grid, 128, 0, st>>>(xb, db16, dw, g, dil);
  else return set_error(SI_ERR_ARG, "si_nn_conv3d_wgrad: (cout, cin) must be in {16, 32}^2");
  if (db) {
    const int bb = egrid(V);
    float* bpart = partials ? partials + (int64_t)sm_count() * 8 * 27 * cout * cin : nullptr;
    if (cout == 16) bias_grad_kernel<16><<<bb, 256, 0, st>>>(db16, V, db, bpart);
    else bias_grad_kernel<32><<<bb, 256, 0, st>>>(db16, V, db, bpart);
    if (bpart) reduce_partials_kernel<<<(cout + 7) / 8, 256, 0, st>>>(bpart, bb, cout, db);
  }
  return check_launch("si_nn_conv3d_wgrad");
}

extern "C" int si_nn_flip_weights(const void* w, void* w_flipped, int cout, int cin, void* stream) {
  clear_error();
  if (!w || !w_flipped || cout < 1 || cin < 1) return set_error(SI_ERR_ARG, "si_nn_flip_weights: bad arguments");
  flip_weights_kernel<<<egrid(27LL * cout * cin), 256, 0, as_stream(stream)>>>(
      static_cast<const __nv_bfloat16*>(w), static_cast<__nv_bfloat16*>(w_flipped), cout, cin);
  return check_launch("si_nn_flip_weights");
}

extern "C" int si_nn_relu_bwd(void* g, const void* y, const void* add, int64_t n, void* stream) {
  clear_error();
  if (!g || !y || n < 0) return set_error(SI_ERR_ARG, "si_nn_relu_bwd: bad arguments");
  relu_bwd_kernel<<<egrid(n), 256, 0, as_stream(stream)>>>(static_cast<__nv_bfloat16*>(g),
                                                            static_cast<const __nv_bfloat16*>(y),
                                                            static_cast<const __nv_bfloat16*>(add), n);
  return check_launch("si_nn_relu_bwd");
}

extern "C" int si_nn_xent(const float* logits, const float* target, const float* weight, int64_t V, int C, int nol,
                          float scale, void* dlogits, float* loss, void* stream) {
  clear_error();
  if (!logits || !target || !dlogits || !loss || nol < 1 || nol > C)
    return set_error(SI_ERR_ARG, "si_nn_xent: bad arguments");
  xent_kernel<<<egrid(V), 256, 0, as_stream(stream)>>>(logits, target, weight, V, C, nol, scale,
                                                        static_cast<__nv_bfloat16*>(dlogits), loss);
  return check_launch("si_nn_xent");
}

extern "C" int si_nn_adamw(float* p, const float* g, float* m, float* v, void* p_bf16, int64_t n, float lr,
                           float beta1, float beta2, float eps, float wd, int step, void* stream) {
  clear_error();
  if (!p || !g || !m || !v || n < 0 || step < 1) return set_error(SI_ERR_ARG, "si_nn_adamw: bad arguments");
  const float bc1 = 1.0f - powf(beta1, (float)step), bc2 = 1.0f - powf(beta2, (float)step);
  adamw_kernel<<<egrid(n), 256, 0, as_stream(stream)>>>(p, g, m, v, static_cast<__nv_bfloat16*>(p_bf16), n, lr,
                                                         beta1, beta2, eps, wd, bc1, bc2);
  return check_launch("si_nn_adamw");
}

extern "C" int si_nn_features(const uint8_t* img, const int16_t* slot_map, const float* zinfo, int D, int H, int W,
                              int z0, int y0, int x0, int Dt, int Ht, int Wt, void* out, void* stream) {
  clear_error();
  if (!img || !slot_map || !zinfo || !out || Dt < 1 || Ht < 1 || Wt < 1)
    return set_error(SI_ERR_ARG, "si_nn_features: bad args");
  if ((uintptr_t)zinfo % 16 || (uintptr_t)out % 16) return set_error(SI_ERR_ARG, "si_nn_features: misaligned");
  features_kernel<<<egrid((int64_t)Dt * Ht * Wt), 256, 0, as_stream(stream)>>>(
      img, slot_map, reinterpret_cast<const float4*>(zinfo), D, H, W, z0, y0, x0, Dt, Ht, Wt,
      static_cast<__nv_bfloat16*>(out));
  return check_launch("si_nn_features");
}

extern "C" int si_nn_probs(const float* logits, int Ds, int H, int W, int zb, int ze, int nol, float* probs,
                           int Zout, int zo, void* stream) {
  clear_error();
  if (!logits || !probs || Ds < 1 || H < 1 || W < 1 || nol < 1 || nol > 16)
    return set_error(SI_ERR_ARG, "si_nn_probs: bad arguments");
  if (zb < 0 || ze > Ds || ze <= zb || zo < 0 || zo + (ze - zb) > Zout)
    return set_error(SI_ERR_ARG, "si_nn_probs: plane range out of bounds");
  const int64_t plane = (int64_t)H * W;
  probs_kernel<<<egrid((int64_t)(ze - zb) * plane), 256, 0, as_stream(stream)>>>(logits, plane, zb, ze, nol, probs,
                                                                                 (int64_t)Zout * plane, zo);
  return check_launch("si_nn_probs");
}
