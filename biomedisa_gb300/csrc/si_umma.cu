// 16 -> 16 channel 3x3x3 convolution of the surrogate network on the
// 5th-generation tensor cores (tcgen05): the forward pass and, with flipped
// weights W'[t][ci][co] = W[26 - t][co][ci], the data gradient.
//
// Implicit GEMM per output tile of 128 consecutive voxels of one x-row
// (n, z, y, x0 .. x0 + 127):
//   D[m][co] = sum over the 27 taps t and 16 input channels ci of
//              X[n, z + dz*dil, y + dy*dil, x0 + m + dx*dil][ci] * W[t][co][ci]
// one tcgen05.mma (kind::f16, M = 128, N = 16, K = 16, bf16 in, fp32
// accumulate in tensor memory) per tap.
//
// Shared-memory operands, K-major without swizzle (core matrices of 8 rows x
// 16 bytes): an input row block holds the channels of 128 + 2*dil voxels as
// [channel half h][voxel][8 channels] (two TMA boxes of 8 channels x 128 + 2*dil
// voxels); the A operand of tap (dz, dy, dx) is that block of row
// (z + dz*dil, y + dy*dil) starting dil*(dx + 1) voxels in, i.e. the same
// layout at a start address 16*dil*(dx + 1) bytes further (any 16-byte
// aligned start is a valid descriptor without swizzle): leading-dimension
// offset = the distance between the halves, stride offset = 128 bytes per 8
// voxels. Out-of-volume rows and voxels arrive as zeros from TMA (the
// "same" padding). The weights sit once per CTA as [tap][h][co][8 ci]
// (512 bytes per tap).
//
// Schedule (persistent CTAs of 128 threads, three per SM): a CTA walks
// "columns" (n, z, x chunk, y phase) along y in steps of the dilation, so a
// tile's 9 input rows (z + {-1,0,1}*dil) x (y + {-1,0,1}*dil) share 6 with the
// previous tile's: a ring of four y-row slots, each holding its three z-rows,
// takes one new y-row (6 TMA boxes) per tile, loaded a tile ahead. While the
// tensor core runs tile j's 27 MMAs into one of two TMEM accumulators, all
// 128 threads run the epilogue of tile j - 1 from the other accumulator
// (thread m owns TMEM lane m = voxel x0 + m): bias, residual, ReLU, bf16 or
// fp32 store, 32 or 64 contiguous bytes per voxel.
// One thread issues the copies and the MMAs; mbarriers carry the copy
// completion (expect_tx) and the MMA completion (tcgen05.commit). Every wait
// is bounded: a wait that gives up records the error, lets the operations in
// flight complete (bounded), frees the tensor memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>

#include "si_common.cuh"
#include "si_internal.h"
#include "si_tma.cuh"

namespace si {
namespace {

constexpr int kTileM = 128;
constexpr int kMaxDil = 8;
constexpr int kRowVox = kTileM + 2 * kMaxDil;     // voxels per staged input row (max)
constexpr int kHalfBytes = kRowVox * 16;          // one channel half of a row: 2304 bytes (128-byte multiple)
constexpr int kRowBytes = 2 * kHalfBytes;         // both channel halves
constexpr int kYSlots = 4;                        // ring of y-rows (each with its 3 z-rows)
constexpr int kAhead = 1;                         // tiles of prefetch: rows up to j + 2 + kAhead are in flight
constexpr int kSlotBytes = 3 * kRowBytes;
constexpr int kWBytes = 27 * 512;                 // weights, [tap][h][co][8]
constexpr int kSmemBytes = kWBytes + kYSlots * kSlotBytes + 128;  // + alignment slack
constexpr int kTmemCols = 32;                               // two 16-column fp32 accumulators
constexpr uint32_t kWaitSpins = 1u << 26;

__device__ uint32_t g_umma_status;  // bit 0: a wait gave up (read by si_nn_umma_status)

// Shared-memory matrix descriptor, no swizzle, K-major core matrices.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // fixed descriptor version bits 46..48 = 0b001
  return d;                // base offset 0, absolute offsets, no swizzle
}

// kind::f16 instruction descriptor: fp32 D, bf16 A and B, both K-major.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(16 >> 3) << 17) |
                            ((uint32_t)(kTileM >> 4) << 24);

__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, int c, int x, int y, int z, int n,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
      "%6}], [%7];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c), "r"(x), "r"(y), "r"(z), "r"(n), "r"(smem_u32(bar))
      : "memory");
}

struct UmmaGeom {
  int N, D, H, W, dil, xchunks;
  long long columns;  // (n, z, x chunk, y phase) tuples; each is walked along y in steps of dil
};

// Column c -> (n, z, x0, y phase); its tiles are y = phase, phase + dil, ... < H.
__device__ __forceinline__ void column_coords(const UmmaGeom& g, long long c, int& n, int& z, int& x0, int& yph) {
  yph = (int)(c % g.dil);
  c /= g.dil;
  const int xc = (int)(c % g.xchunks);
  c /= g.xchunks;
  z = (int)(c % g.D);
  n = (int)(c / g.D);
  x0 = xc * kTileM;
}

template <bool kOutF32>
__global__ void __launch_bounds__(128, 1) conv16_umma_kernel(const __grid_constant__ CUtensorMap xmap,
                                                            const __nv_bfloat16* __restrict__ w,
                                                            const float* __restrict__ bias,
                                                            const __nv_bfloat16* __restrict__ residual,
                                                            void* __restrict__ y_out, UmmaGeom g, int relu,
                                                            uint32_t wait_lim) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127);
  uint8_t* sw = smem;              // weights [tap][h][co][8]
  uint8_t* rows = smem + kWBytes;  // [y slot][dz][h][voxel][8]
  __shared__ __align__(8) uint64_t full_bar[kYSlots];  // the 3 z-rows of a y slot landed
  __shared__ __align__(8) uint64_t mma_bar[2];         // MMAs of an accumulator complete
  __shared__ uint32_t tmem_base;
  __shared__ float s_bias[16];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int rv = kTileM + 2 * g.dil;                      // staged voxels per input row
  const uint32_t slot_tx = 3u * 2u * (uint32_t)rv * 16u;  // bytes the 6 boxes of one y slot deliver

  // weights -> [tap][h][co][8 ci]; bias
  for (int i = tid; i < 27 * 16 * 2; i += blockDim.x) {
    const int tap = i / 32, co = (i / 2) % 16, h = i % 2;
    const uint4 v = reinterpret_cast<const uint4*>(w)[(tap * 16 + co) * 2 + h];
    *reinterpret_cast<uint4*>(sw + tap * 512 + h * 256 + co * 16) = v;
  }
  if (tid < 16) s_bias[tid] = bias ? bias[tid] : 0.0f;
  if (tid == 0) {
    for (int s = 0; s < kYSlots; ++s) mbar_init(&full_bar[s], 1);
    for (int s = 0; s < 2; ++s) mbar_init(&mma_bar[s], 1);
    fence_barrier_init();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_proxy_async_shared();  // weights written by threads, read by the tensor core
  tmem_fence_before();
  __syncthreads();
  tmem_fence_after();
  const uint32_t tmem = tmem_base;

  // Barrier bookkeeping, in every thread (the counts advance identically):
  // uses of each y slot / accumulator barrier so far, which give the parity of
  // the next completion. Thread 0 alone issues copies and MMAs.
  uint32_t slot_loads[kYSlots] = {}, slot_waits[kYSlots] = {};
  uint32_t acc_commits[2] = {0u, 0u}, acc_waits[2] = {0u, 0u};
  bool failed = false;

  auto load_row = [&](int n, int z, int x0, int yy, int k) {  // thread 0: input y-row yy -> slot k % 4
    const int s = k % kYSlots;
    uint64_t* bar = &full_bar[s];
    mbar_expect_tx(bar, slot_tx);
    uint8_t* dst = rows + (size_t)s * kSlotBytes;
    for (int dz = 0; dz < 3; ++dz)
      for (int h = 0; h < 2; ++h)
        tma_load_5d(dst + dz * kRowBytes + h * kHalfBytes, &xmap, 8 * h, x0 - g.dil, yy, z + (dz - 1) * g.dil, n,
                    bar);
  };
  auto wait_slot = [&](int k) -> bool {  // all threads: row k's slot landed
    const int s = k % kYSlots;
    const bool ok = mbar_wait_bounded(&full_bar[s], slot_waits[s] & 1u, wait_lim);
    if (ok) ++slot_waits[s];
    return ok;
  };
  auto wait_acc = [&](int b) -> bool {
    const bool ok = mbar_wait_bounded(&mma_bar[b], acc_waits[b] & 1u, wait_lim);
    if (ok) ++acc_waits[b];
    return ok;
  };
  auto epilogue = [&](int n, int z, int y, int x0, int b) {  // all threads: accumulator b -> output row (n, z, y)
    uint32_t v[16];
    const uint32_t taddr = tmem + (uint32_t)(b * 16) + ((uint32_t)(warp * 32) << 16);
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    const int x = x0 + tid;
    if (x >= g.W) return;
    const long long r = (((long long)n * g.D + z) * g.H + y) * g.W + x;
    float u[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) u[c] = __uint_as_float(v[c]) + s_bias[c];
    if (residual) {
      const uint4* rp = reinterpret_cast<const uint4*>(residual + r * 16);
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const uint4 rr = rp[q];
        const uint32_t words[4] = {rr.x, rr.y, rr.z, rr.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          u[q * 8 + 2 * e] += __bfloat162float(__ushort_as_bfloat16((unsigned short)(words[e] & 0xFFFFu)));
          u[q * 8 + 2 * e + 1] += __bfloat162float(__ushort_as_bfloat16((unsigned short)(words[e] >> 16)));
        }
      }
    }
    if (relu) {
#pragma unroll
      for (int c = 0; c < 16; ++c) u[c] = fmaxf(u[c], 0.0f);
    }
    if (kOutF32) {
      float4* op = reinterpret_cast<float4*>(static_cast<float*>(y_out) + r * 16);
#pragma unroll
      for (int q = 0; q < 4; ++q) op[q] = make_float4(u[4 * q], u[4 * q + 1], u[4 * q + 2], u[4 * q + 3]);
    } else {
      uint32_t pk[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const __nv_bfloat162 b2 = __floats2bfloat162_rn(u[2 * q], u[2 * q + 1]);
        pk[q] = *reinterpret_cast<const uint32_t*>(&b2);
      }
      uint4* op = reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(y_out) + r * 16);
      op[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      op[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
    }
  };

  int tile_count = 0;  // tiles this CTA has started (its accumulator is tile_count & 1)
  for (long long col = blockIdx.x; col < g.columns && !failed; col += gridDim.x) {
    int n, z, x0, yph;
    column_coords(g, col, n, z, x0, yph);
    const int nt = (g.H - yph + g.dil - 1) / g.dil;  // tiles y = yph + j*dil, j < nt
    // row k of this column is input y-row yph + (k - 1)*dil, so tile j reads
    // rows k = j, j + 1, j + 2 (y = y_j - dil, y_j, y_j + dil)
    if (tid == 0) {
      for (int k = 0; k < 3 + kAhead && k <= nt + 1; ++k) {  // rows 0 .. 2 + kAhead
        load_row(n, z, x0, yph + (k - 1) * g.dil, k);
        ++slot_loads[k % kYSlots];
      }
    }
    for (int j = 0; j <= nt; ++j) {
      const int b = (tile_count + j) & 1;
      bool ok = true;
      if (j < nt) {
        // tile j's three rows landed (rows j, j + 1 were waited before, except at the column start)
        if (j == 0) ok = wait_slot(0) && wait_slot(1);
        ok = ok && wait_slot(j + 2);
        if (ok && tid == 0) {
          tmem_fence_after();
          const uint32_t d = tmem + (uint32_t)(b * 16), wb = smem_u32(sw);
#pragma unroll 1
          for (int tap = 0; tap < 27; ++tap) {
            const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
            const int s = (j + dy) % kYSlots;
            const uint32_t a_addr = smem_u32(rows + (size_t)s * kSlotBytes + dz * kRowBytes) +
                                    (uint32_t)(dx * g.dil) * 16u;
            umma_f16(d, smem_desc(a_addr, kHalfBytes, 128), smem_desc(wb + (uint32_t)tap * 512u, 256, 128),
                     tap ? 1u : 0u);
          }
          umma_commit(&mma_bar[b]);
        }
        if (ok) ++acc_commits[b];
      }
      if (__syncthreads_or(!ok)) {
        failed = true;
        break;
      }
      if (j >= 1) {
        // tile j - 1: MMAs done -> the slot of row j - 1 (last read by tile j - 1)
        // takes row j + 2 + kAhead, which tile j + kAhead needs; epilogue of tile j - 1
        const int pb = b ^ 1;
        ok = wait_acc(pb);
        if (__syncthreads_or(!ok)) {
          failed = true;
          break;
        }
        tmem_fence_after();
        if (tid == 0 && j + 2 + kAhead <= nt + 1) {
          load_row(n, z, x0, yph + (j + 1 + kAhead) * g.dil, j + 2 + kAhead);
          ++slot_loads[(j + 2 + kAhead) % kYSlots];
        }
        epilogue(n, z, yph + (j - 1) * g.dil, x0, pb);
        tmem_fence_before();
        __syncthreads();  // accumulator pb free before tile j + 1's MMAs write it
      }
    }
    tile_count += nt;
  }
  if (failed && tid == 0) {
    // let everything in flight complete (bounded) before the CTA's shared and
    // tensor memory go away: committed MMAs not yet seen, copies not yet seen
    for (int bb = 0; bb < 2; ++bb)
      while (acc_waits[bb] < acc_commits[bb] && mbar_wait_bounded(&mma_bar[bb], acc_waits[bb] & 1u, kWaitSpins))
        ++acc_waits[bb];
    for (int s = 0; s < kYSlots; ++s)
      while (slot_waits[s] < slot_loads[s] && mbar_wait_bounded(&full_bar[s], slot_waits[s] & 1u, kWaitSpins))
        ++slot_waits[s];
    atomicOr(&g_umma_status, 1u);
  }
  tmem_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

}  // namespace

// 16 -> 16 convolution on the tensor cores (see the file comment). x, w,
// residual, y 16-byte aligned; dil <= 8. Returns SI_OK or an error code.
int conv16_umma(const void* x, const void* w, const float* bias, const void* residual, void* y, int N, int D, int H,
                int W, int dil, int relu, int out_f32, cudaStream_t st) {
  if (dil < 1 || dil > kMaxDil) return set_error(SI_ERR_ARG, "conv16_umma: dilation must be 1..%d", kMaxDil);
  const EncodeTiledFn enc = encode_fn();
  if (!enc) return set_error(SI_ERR_CUDA, "conv16_umma: cuTensorMapEncodeTiled unavailable");
  CUtensorMap map;
  std::memset(&map, 0, sizeof(map));
  const cuuint64_t dims[5] = {16, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)D, (cuuint64_t)N};
  const cuuint64_t strides[4] = {32ull, 32ull * W, 32ull * W * H, 32ull * W * H * D};  // bytes, dims 1..4
  const cuuint32_t box[5] = {8, (cuuint32_t)(kTileM + 2 * dil), 1, 1, 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  const CUresult cr = enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(x), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) return set_error(SI_ERR_CUDA, "conv16_umma: tensor map encoding failed (%d)", (int)cr);
  UmmaGeom g{N, D, H, W, dil, (W + kTileM - 1) / kTileM, 0};
  g.columns = (long long)N * D * g.xchunks * dil;
  if (g.columns == 0) return SI_OK;
  const cudaError_t ae = out_f32 ? cudaFuncSetAttribute(conv16_umma_kernel<true>,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes)
                                 : cudaFuncSetAttribute(conv16_umma_kernel<false>,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
  if (ae != cudaSuccess) return set_error(SI_ERR_CUDA, "conv16_umma: shared memory opt-in: %s", cudaGetErrorString(ae));
  const long long want = std::min<long long>(g.columns, (long long)sm_count() * 3);
  const auto* wb = static_cast<const __nv_bfloat16*>(w);
  const auto* rb = static_cast<const __nv_bfloat16*>(residual);
  const uint32_t wl = wait_limit();
  if (out_f32)
    conv16_umma_kernel<true><<<(unsigned)want, 128, kSmemBytes, st>>>(map, wb, bias, rb, y, g, relu, wl);
  else
    conv16_umma_kernel<false><<<(unsigned)want, 128, kSmemBytes, st>>>(map, wb, bias, rb, y, g, relu, wl);
  return check_launch("conv16_umma");
}

}  // namespace si

extern "C" int si_nn_umma_status(int* status, void* stream) {
  si::clear_error();
  if (!status) return si::set_error(SI_ERR_ARG, "si_nn_umma_status: null pointer");
  cudaStream_t st = si::as_stream(stream);
  uint32_t v = 0;
  const uint32_t zero = 0;
  if (cudaMemcpyFromSymbolAsync(&v, si::g_umma_status, sizeof(v), 0, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess ||
      cudaMemcpyToSymbolAsync(si::g_umma_status, &zero, sizeof(zero), 0, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return si::set_error(SI_ERR_CUDA, "si_nn_umma_status: %s", cudaGetErrorString(cudaGetLastError()));
  *status = (int)v;
  if (v) return si::set_error(SI_ERR_CUDA, "tensor-core convolution: a wait gave up (status %u)", v);
  return SI_OK;
}
