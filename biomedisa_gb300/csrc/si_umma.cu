// 16 -> 16 channel 3x3x3 convolution of the surrogate network on the
// 5th-generation tensor cores (tcgen05): the forward pass and, with flipped
// weights W'[t][ci][co] = W[26 - t][co][ci], the data gradient.
//
// Implicit GEMM over output tiles of 128 consecutive voxels of an x-row,
// organised by INPUT rows. A CTA walks "columns" (n, z, x chunk, y phase):
// output rows y_j = phase + j*dil, j < nt, and input rows i = 0 .. nt + 1 at
// y = phase + (i - 1)*dil. Input row i meets output rows j = i - 2, i - 1, i
// through the taps dy = +1, 0, -1, so per (dz, dx) ONE tcgen05.mma
// (kind::f16, M = 128 voxels, N = 48, K = 16, bf16 in, fp32 accumulate)
// multiplies the shifted input by the three stacked 16x16 weight blocks
// [W(dz,+1,dx); W(dz,0,dx); W(dz,-1,dx)] and adds into three consecutive
// 16-column accumulators in tensor memory: 9 MMAs of N = 48 per input row
// instead of 27 of N = 16 per output row, with each staged input row read
// by the tensor core 9 times instead of 27.
//
// Accumulator ring. The CTA's input rows form one sequence k = 0, 1, ...
// over all its columns (column c starts at k = P_c, P_{c+1} = P_c + nt + 2);
// input k adds into ring positions k, k + 1, k + 2 and completes position k
// (output j = k - P_c - 2 of its column; positions P_c and P_c + 1 are
// padding). Positions live in the 32 slots of 16 columns (k mod 32) of the
// 512 tensor-memory columns; a region starting at slot 30 or 31 is issued as
// two MMAs (N = 32 + 16 or 16 + 32) that continue at slot 0, so every
// position sums its 27 products in one slot, in the same order wherever it
// falls in the ring (results do not depend on the grid). Every MMA
// accumulates; the epilogue zeroes a position's slot (tcgen05.st) after
// reading it and before releasing it, and all slots start zeroed.
//
// Shared-memory operands, K-major without swizzle (core matrices of 8 rows x
// 16 bytes): an input z-row is one TMA box of {8 channels, 128 + 2*dil
// voxels, 2 channel halves} over a 5-D tensor map {8, W, 2, H, D*N} whose
// half dimension has a 16-byte stride, which lands as [half][voxel][8
// channels]; the A operand of shift dx is that block at a start address
// 16*dil*(dx + 1) bytes further. Voxels outside the row arrive as zeros
// (TMA fill); input rows outside the volume in y or z are neither loaded
// nor multiplied (their contribution is zero). The weights sit once per CTA
// as 9 blocks [dz][dx] of [half][48][8 ci].
//
// Roles (one persistent CTA per SM, 11 warps): warp 0 loads each input row's
// z-rows into a ring of 10 row slots; warp 10 loads, for a residual layer,
// each output row's residual tile into a ring of 12 slots (so the epilogue
// never waits on a global load); warp 1 issues the 9 MMAs and two commits
// per input row (row slot free; ring position complete); two groups of four
// warps (2-5, 6-9) run the epilogue of alternate positions (thread m =
// tensor-memory lane m = voxel x0 + m): bias, residual, ReLU, bf16 or fp32
// store, zeroing, release. Warps 0, 1 and 10 run their loops as whole warps
// with warp-uniform operands and issue from one elected lane (from a single
// lane every MMA cost about 80 cycles of issue, measured). Optionally the
// CTA's columns are dealt to 2 or 4 interleaved streams with rings of their
// own (si_nn_conv16_tc_set_streams; measured slower than one). Every wait is
// bounded: a role that gives up flags the CTA, the others stop at their next
// wait, the copies and MMAs in flight are waited for (bounded), the tensor
// memory is freed and the status records the error.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <cstring>

#include "si_common.cuh"
#include "si_internal.h"
#include "si_tma.cuh"

namespace si {
namespace {

constexpr int kTileM = 128;
constexpr int kMaxDil = 8;
constexpr int kRowBytes = (kTileM + 2 * kMaxDil) * 32;  // one staged z-row, both halves: 4608 bytes
constexpr int kSlotBytes = 3 * kRowBytes;               // an input row: its three z-rows
constexpr int kRowSlots = 10;                           // ring of staged input rows
constexpr int kResBytes = kTileM * 32;                  // one residual row tile [half][128][8]: 4096 bytes
constexpr int kResSlots = 12;                           // ring of staged residual rows
constexpr int kWBlockBytes = 2 * 48 * 16;               // one (dz, dx) weight block [half][48][8]
constexpr int kWBytes = 9 * kWBlockBytes;
constexpr int kSmemBytes = kWBytes + kRowSlots * kSlotBytes + kResSlots * kResBytes + 128;  // + alignment slack
constexpr int kTmemCols = 512;                          // 32 physical slots
constexpr int kEpiGroups = 2;                           // epilogue groups of 4 warps, alternate items
constexpr int kResWarp = 2 + 4 * kEpiGroups;           // the warp loading residual rows
constexpr int kThreads = 32 * (kResWarp + 1);

__device__ uint32_t g_umma_status;  // bit 0: a wait gave up (read by si_nn_umma_status)
std::atomic<int> g_umma_streams{1};  // interleaved column streams per CTA (si_nn_conv16_tc_set_streams)

// Shared-memory matrix descriptor, no swizzle, K-major core matrices.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // fixed descriptor version bits 46..48 = 0b001
  return d;                // base offset 0, absolute offsets, no swizzle
}

// kind::f16 instruction descriptor: fp32 D, bf16 A and B, both K-major, M = 128, N = kN.
template <int kN>
__host__ __device__ constexpr uint32_t idesc_f16() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kN >> 3) << 17) | ((uint32_t)(kTileM >> 4) << 24);
}

// Executed by a whole warp with warp-uniform operands (which then stay in
// uniform registers); one elected lane issues the MMA / the commit.
template <int kN>
__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t a, uint64_t b) {
  asm volatile(
      "{\n\t.reg .pred p, e;\n\tsetp.ne.b32 p, 1, 0;\n\telect.sync _|e, 0xffffffff;\n\t"
      "@e tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc_f16<kN>())
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "{\n\t.reg .pred e;\n\telect.sync _|e, 0xffffffff;\n\t"
      "@e tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n\t}" ::"r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tmem_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// The copy, the expect_tx and the plain arrival below are executed by a
// whole warp with warp-uniform operands; one elected lane issues them.
__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, int c, int x, int h, int y, int zn,
                                            uint64_t* bar) {
  asm volatile(
      "{\n\t.reg .pred e;\n\telect.sync _|e, 0xffffffff;\n\t"
      "@e cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
      "%5, %6}], [%7];\n\t}" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c), "r"(x), "r"(h), "r"(y), "r"(zn), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void expect_tx_elect(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .pred e;\n\telect.sync _|e, 0xffffffff;\n\t"
      "@e mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n\t}" ::"r"(smem_u32(bar)),
      "r"(bytes)
      : "memory");
}
__device__ __forceinline__ void arrive_elect(uint64_t* bar) {
  asm volatile(
      "{\n\t.reg .pred e;\n\telect.sync _|e, 0xffffffff;\n\t"
      "@e mbarrier.arrive.shared::cta.b64 _, [%0];\n\t}" ::"r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_zero16(uint32_t taddr) {
  const uint32_t z = 0;
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(taddr),
      "r"(z)
      : "memory");
}

struct UmmaGeom {
  int N, D, H, W, dil, xchunks;
  long long columns;  // (n, z, x chunk, y phase) tuples; each is walked along y in steps of dil
};

// Column c -> (n, z, x0, y phase, tiles); its output rows are y = phase + j*dil, j < nt.
struct Column {
  int n, z, x0, yph, nt;
};
__device__ __forceinline__ Column column_of(const UmmaGeom& g, long long c) {
  Column o;
  o.yph = (int)(c % g.dil);
  c /= g.dil;
  o.x0 = (int)(c % g.xchunks) * kTileM;
  c /= g.xchunks;
  o.z = (int)(c % g.D);
  o.n = (int)(c / g.D);
  o.nt = (g.H - o.yph + g.dil - 1) / g.dil;
  return o;
}

// A stream: one of the CTA's interleaved column sequences and its position
// in it (column, input row i of the column, the stream's ring position p =
// k mod R of its input k with the phase (k / R) & 1).
struct Stream {
  long long col;
  Column c;
  int i;
  int p;
  uint32_t ph;
};

// Index and phase of a ring of kN barriers (mbarrier parity of the use).
template <int kN>
struct Ring {
  int idx = 0;
  uint32_t ph = 0;
  uint32_t wrapped = 0;  // at least one full turn done
  __device__ __forceinline__ void next() {
    if (++idx == kN) {
      idx = 0;
      ph ^= 1u;
      wrapped = 1u;
    }
  }
};

template <bool kOutF32, int kNS>
__global__ void __launch_bounds__(kThreads, 1) conv16_umma_kernel(const __grid_constant__ CUtensorMap xmap,
                                                                 const __grid_constant__ CUtensorMap rmap,
                                                                 const __nv_bfloat16* __restrict__ w,
                                                                 const float* __restrict__ bias, int has_res,
                                                                 void* __restrict__ y_out, UmmaGeom g, int relu,
                                                                 uint32_t wait_lim) {
  constexpr int kR = 32 / kNS;  // ring positions (16-column slots) of a stream
  static_assert(kR >= 8, "accumulator ring too short");
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127);
  uint8_t* sw = smem;                             // weight blocks [dz][dx][half][48][8]
  uint8_t* rows = smem + kWBytes;                 // [row slot][dz][half][voxel][8]
  uint8_t* rres = rows + kRowSlots * kSlotBytes;  // [residual slot][half][128][8]
  __shared__ __align__(8) uint64_t full_bar[kRowSlots];   // an item's input z-rows landed
  __shared__ __align__(8) uint64_t empty_bar[kRowSlots];  // its MMAs completed (row slot free)
  __shared__ __align__(8) uint64_t done_bar[kNS * kR];    // ring position of a stream complete
  __shared__ __align__(8) uint64_t free_bar[kNS * kR];    // ... read, zeroed, released
  __shared__ __align__(8) uint64_t rfull_bar[kResSlots];  // an item's residual row landed
  __shared__ __align__(8) uint64_t rfree_bar[kResSlots];  // ... and was read
  __shared__ uint32_t tmem_base;
  __shared__ float s_bias[16];
  __shared__ volatile int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int dil = g.dil;
  const int rv = kTileM + 2 * dil;  // staged voxels per z-row
  const uint32_t box_bytes = 32u * (uint32_t)rv;

  for (int i = tid; i < 9 * 48 * 2; i += kThreads) {
    const int blk = i / 96, nrow = (i / 2) % 48, h = i % 2;
    const int q = nrow / 16, co = nrow % 16;
    const int tap = (blk / 3) * 9 + (2 - q) * 3 + blk % 3;  // dz digit, dy digit 2 - q, dx digit
    const uint4 v = reinterpret_cast<const uint4*>(w)[(tap * 16 + co) * 2 + h];
    *reinterpret_cast<uint4*>(sw + blk * kWBlockBytes + h * 768 + nrow * 16) = v;
  }
  if (tid < 16) s_bias[tid] = bias ? bias[tid] : 0.0f;
  if (tid == 0) {
    s_fail = 0;
    for (int b = 0; b < kRowSlots; ++b) {
      mbar_init(&full_bar[b], 1);
      mbar_init(&empty_bar[b], 1);
    }
    for (int b = 0; b < kNS * kR; ++b) {
      mbar_init(&done_bar[b], 1);
      mbar_init(&free_bar[b], 4);  // one arrival per epilogue warp
    }
    for (int b = 0; b < kResSlots; ++b) {
      mbar_init(&rfull_bar[b], 1);
      mbar_init(&rfree_bar[b], 4);
    }
    fence_barrier_init();
  }
  if (warp == 1) {
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
  const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;  // this warp's tensor-memory lane quadrant
  if (warp >= 2 && warp < 6) {  // all 32 slots start at zero
    for (int b = 0; b < 32; ++b) tmem_zero16(tmem + lane_base + (uint32_t)(16 * b));
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
  }
  tmem_fence_before();
  __syncthreads();
  tmem_fence_after();

  // The CTA's columns b, b + G, b + 2G, ... (G = gridDim.x) are dealt to the
  // kNS streams in turn; items (one input row of one stream) are visited by
  // every role in the same order: groups of one input per live stream,
  // streams in order.
  const long long cstep = (long long)kNS * gridDim.x;
  Stream st[kNS];
#pragma unroll
  for (int s = 0; s < kNS; ++s) {
    st[s].col = blockIdx.x + (long long)s * gridDim.x;
    st[s].i = 0;
    st[s].p = 0;
    st[s].ph = 0;
    if (st[s].col < g.columns) st[s].c = column_of(g, st[s].col);
  }
  auto advance = [&](Stream& t) {
    if (++t.p == kR) {
      t.p = 0;
      t.ph ^= 1u;
    }
    if (++t.i == t.c.nt + 2) {
      t.i = 0;
      t.col += cstep;
      if (t.col < g.columns) t.c = column_of(g, t.col);
    }
  };
  auto row_y = [&](const Stream& t) { return t.c.yph + (t.i - 1) * dil; };

  // progress (lane 0 of warps 0 / 1): items whose rows / residual rows were
  // loaded; the done barrier and parity of the last commit
  long long q_loaded = 0, q_res = 0;
  int last_done = -1;
  uint32_t last_par = 0;
  if (warp == 0) {
    // ---- producer, the whole warp in step, one elected lane issuing: each
    // item's z-rows into the row ring
    Ring<kRowSlots> rr;
    bool stop = false, any = true;
    while (any && !stop) {
      any = false;
#pragma unroll
      for (int s = 0; s < kNS; ++s) {
        Stream& t = st[s];
        if (stop || t.col >= g.columns) continue;
        any = true;
        const bool okE = !rr.wrapped || mbar_wait_fast(&empty_bar[rr.idx], rr.ph ^ 1u, wait_lim);
        if (!__all_sync(0xffffffffu, okE && !s_fail)) {
          s_fail = 1;
          stop = true;
          continue;
        }
        const int yy = row_y(t);
        uint32_t nvalid = 0;
        if (yy >= 0 && yy < g.H)
          for (int dz = 0; dz < 3; ++dz) {
            const int zz = t.c.z + (dz - 1) * dil;
            nvalid += (zz >= 0 && zz < g.D) ? 1u : 0u;
          }
        if (nvalid == 0) {
          arrive_elect(&full_bar[rr.idx]);
        } else {
          expect_tx_elect(&full_bar[rr.idx], nvalid * box_bytes);
          uint8_t* dst = rows + (size_t)rr.idx * kSlotBytes;
          for (int dz = 0; dz < 3; ++dz) {
            const int zz = t.c.z + (dz - 1) * dil;
            if (zz >= 0 && zz < g.D)
              tma_load_5d(dst + dz * kRowBytes, &xmap, 0, t.c.x0 - dil, 0, yy, t.c.n * g.D + zz, &full_bar[rr.idx]);
          }
        }
        rr.next();
        ++q_loaded;
        advance(t);
      }
    }
  } else if (warp == kResWarp) {
    // ---- residual loader, the whole warp in step: for each item the
    // residual row of the position it completes (output j = i - 2; padding
    // positions arrive without a copy)
    Ring<kResSlots> sr;
    bool stop = !has_res, any = true;
    while (any && !stop) {
      any = false;
#pragma unroll
      for (int s = 0; s < kNS; ++s) {
        Stream& t = st[s];
        if (stop || t.col >= g.columns) continue;
        any = true;
        const bool okR = !sr.wrapped || mbar_wait_fast(&rfree_bar[sr.idx], sr.ph ^ 1u, wait_lim);
        if (!__all_sync(0xffffffffu, okR && !s_fail)) {
          s_fail = 1;
          stop = true;
          continue;
        }
        if (t.i >= 2) {
          expect_tx_elect(&rfull_bar[sr.idx], (uint32_t)kResBytes);
          tma_load_5d(rres + (size_t)sr.idx * kResBytes, &rmap, 0, t.c.x0, 0, t.c.yph + (t.i - 2) * dil,
                      t.c.n * g.D + t.c.z, &rfull_bar[sr.idx]);
        } else {
          arrive_elect(&rfull_bar[sr.idx]);
        }
        sr.next();
        ++q_res;
        advance(t);
      }
    }
  } else if (warp == 1) {
    // ---- MMA issuer, the whole warp in step (operands warp-uniform), one
    // elected lane issuing: descriptors precomputed; per item only the row
    // slot's base and the accumulator column change; a group's MMAs
    // alternate between its streams
    const uint32_t tm = __shfl_sync(0xffffffffu, tmem, 0);
    // weight block b = dz*3 + dx: descriptor bdesc0 + b * kWBlockBytes / 16
    const uint64_t bdesc0 = smem_desc(smem_u32(sw), 768, 128);
    const uint64_t adesc0 = smem_desc(smem_u32(rows), 16u * (uint32_t)rv, 128);
    const uint64_t ddx = (uint64_t)dil;  // one dx step in descriptor start-address units (16 bytes)
    Ring<kRowSlots> rr;
    // position k + 2 of each stream (first touched by input k): index, phase, wrapped
    int p2[kNS];
    uint32_t ph2[kNS], w2[kNS];
#pragma unroll
    for (int s = 0; s < kNS; ++s) {
      p2[s] = 2;
      ph2[s] = 0;
      w2[s] = 0;
    }
    bool run = true;
    while (run) {
      bool live[kNS];
      int ns = 0;
#pragma unroll
      for (int s = 0; s < kNS; ++s) {
        live[s] = st[s].col < g.columns;
        ns += live[s] ? 1 : 0;
      }
      if (ns == 0) break;
      bool ok = true;
      uint64_t ad[kNS];
      uint32_t dd[kNS], d0[kNS], zm[kNS];
      int wrap[kNS];  // 0: the region fits; 1: 2 + 1 slots split at the ring end; 2: 1 + 2
      int slot[kNS];
      Ring<kRowSlots> r2 = rr;
#pragma unroll
      for (int s = 0; s < kNS; ++s) {
        zm[s] = 0;
        slot[s] = r2.idx;
        if (!live[s]) continue;
        const Stream& t = st[s];
        ok = ok && mbar_wait_fast(&full_bar[r2.idx], r2.ph, wait_lim);
        if (w2[s]) ok = ok && mbar_wait_fast(&free_bar[s * kR + p2[s]], ph2[s] ^ 1u, wait_lim);
        ad[s] = adesc0 + (uint64_t)((r2.idx * kSlotBytes) >> 4);
        dd[s] = tm + (uint32_t)(s * kR * 16 + 16 * t.p);
        d0[s] = tm + (uint32_t)(s * kR * 16);
        wrap[s] = t.p <= kR - 3 ? 0 : (t.p == kR - 2 ? 1 : 2);
        const int yy = row_y(t);
        if (yy >= 0 && yy < g.H)
#pragma unroll
          for (int dz = 0; dz < 3; ++dz) {
            const int zz = t.c.z + (dz - 1) * dil;
            zm[s] |= (zz >= 0 && zz < g.D) ? (1u << dz) : 0u;
          }
        r2.next();
      }
      if (!__all_sync(0xffffffffu, ok && !s_fail)) {  // one decision for the whole warp
        s_fail = 1;
        break;
      }
      tmem_fence_after();
      bool any_wrap = false;
#pragma unroll
      for (int s = 0; s < kNS; ++s) any_wrap |= wrap[s] != 0;
      if (!any_wrap) {  // every region fits: 9 MMAs of N = 48 per item
#pragma unroll
        for (int dz = 0; dz < 3; ++dz)
#pragma unroll
          for (int dx = 0; dx < 3; ++dx)
#pragma unroll
            for (int s = 0; s < kNS; ++s)
              if (zm[s] & (1u << dz))
                umma_f16<48>(dd[s], ad[s] + (uint64_t)((dz * kRowBytes) >> 4) + (uint64_t)dx * ddx,
                             bdesc0 + (uint64_t)((dz * 3 + dx) * (kWBlockBytes >> 4)));
      } else {
#pragma unroll 1
        for (int dz = 0; dz < 3; ++dz)
#pragma unroll 1
          for (int dx = 0; dx < 3; ++dx)
#pragma unroll
            for (int s = 0; s < kNS; ++s) {
              if (!(zm[s] & (1u << dz))) continue;
              const uint64_t a = ad[s] + (uint64_t)((dz * kRowBytes) >> 4) + (uint64_t)dx * ddx;
              const uint64_t b = bdesc0 + (uint64_t)((dz * 3 + dx) * (kWBlockBytes >> 4));
              // a region running past the ring end continues at slot 0; the
              // second piece starts 32 or 16 weight rows (16 bytes each) in
              if (wrap[s] == 0) {
                umma_f16<48>(dd[s], a, b);
              } else if (wrap[s] == 1) {
                umma_f16<32>(dd[s], a, b);
                umma_f16<16>(d0[s], a, b + 32);
              } else {
                umma_f16<16>(dd[s], a, b);
                umma_f16<32>(d0[s], a, b + 16);
              }
            }
      }
#pragma unroll
      for (int s = 0; s < kNS; ++s) {
        if (!live[s]) continue;
        Stream& t = st[s];
        umma_commit(&empty_bar[slot[s]]);
        last_done = s * kR + t.p;
        last_par = t.ph;
        umma_commit(&done_bar[last_done]);
        if (++p2[s] == kR) {
          p2[s] = 0;
          ph2[s] ^= 1u;
          w2[s] = 1u;
        }
        advance(t);
      }
      rr = r2;
    }
  } else {
    // ---- epilogue (warps 2 .. kResWarp - 1): every item's completed position, in item order, the
    // groups taking turns
    const int m = 32 * (warp & 3) + lane;  // tensor-memory lane = voxel offset in the tile
    const int group = (warp - 2) >> 2;
    int turn = 0;
    Ring<kResSlots> sr;
    bool stop = false, any = true;
    while (any && !stop) {
      any = false;
#pragma unroll
      for (int s = 0; s < kNS; ++s) {
        Stream& t = st[s];
        if (stop || t.col >= g.columns) continue;
        any = true;
        const bool mine = turn == group;
        if (++turn == kEpiGroups) turn = 0;
        if (!mine) {
          if (has_res) sr.next();
          advance(t);
          continue;
        }
        const int p = t.p;
        bool ok = !s_fail && mbar_wait_fast(&done_bar[s * kR + p], t.ph, wait_lim);
        if (has_res) ok = ok && mbar_wait_fast(&rfull_bar[sr.idx], sr.ph, wait_lim);
        if (!__all_sync(0xffffffffu, ok)) {
          s_fail = 1;
          stop = true;
          continue;
        }
        tmem_fence_after();
        const uint32_t ta = tmem + lane_base + (uint32_t)(s * kR * 16 + 16 * p);
        if (t.i >= 2) {  // output row j = i - 2 of the column
          uint32_t v[16];
          tmem_ld16(ta, v);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          float u[16];
#pragma unroll
          for (int e = 0; e < 16; ++e) u[e] = __uint_as_float(v[e]);
          const int x = t.c.x0 + m, yo = t.c.yph + (t.i - 2) * dil;
          if (x < g.W) {
            const long long r = (((long long)t.c.n * g.D + t.c.z) * g.H + yo) * g.W + x;
#pragma unroll
            for (int e = 0; e < 16; ++e) u[e] += s_bias[e];
            if (has_res) {
              const uint8_t* rp = rres + (size_t)sr.idx * kResBytes + m * 16;
#pragma unroll
              for (int h = 0; h < 2; ++h) {
                const uint4 rq = *reinterpret_cast<const uint4*>(rp + h * (kResBytes / 2));
                const uint32_t words[4] = {rq.x, rq.y, rq.z, rq.w};
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                  u[h * 8 + 2 * e] += __bfloat162float(__ushort_as_bfloat16((unsigned short)(words[e] & 0xFFFFu)));
                  u[h * 8 + 2 * e + 1] += __bfloat162float(__ushort_as_bfloat16((unsigned short)(words[e] >> 16)));
                }
              }
            }
            if (relu) {
#pragma unroll
              for (int e = 0; e < 16; ++e) u[e] = fmaxf(u[e], 0.0f);
            }
            if (kOutF32) {
              float4* op = reinterpret_cast<float4*>(static_cast<float*>(y_out) + r * 16);
#pragma unroll
              for (int e = 0; e < 4; ++e) op[e] = make_float4(u[4 * e], u[4 * e + 1], u[4 * e + 2], u[4 * e + 3]);
            } else {
              uint32_t pk[8];
#pragma unroll
              for (int e = 0; e < 8; ++e) {
                const __nv_bfloat162 b2 = __floats2bfloat162_rn(u[2 * e], u[2 * e + 1]);
                pk[e] = *reinterpret_cast<const uint32_t*>(&b2);
              }
              uint4* op = reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(y_out) + r * 16);
              op[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
              op[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
            }
          }
        }
        tmem_zero16(ta);
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        tmem_fence_before();
        __syncwarp();
        if (lane == 0) {
          mbar_arrive(&free_bar[s * kR + p]);
          if (has_res) mbar_arrive(&rfree_bar[sr.idx]);
        }
        if (has_res) sr.next();
        advance(t);
      }
    }
  }
  __syncwarp();
  __syncthreads();
  if (s_fail) {
    // let everything in flight complete (bounded) before the CTA's shared and
    // tensor memory go away: the last commit covers every MMA issued; each
    // row and residual slot has at most one copy outstanding
    if (warp == 1 && lane == 0 && last_done >= 0)
      mbar_wait_bounded(&done_bar[last_done], last_par, kDrainWaitLimit);
    if (warp == 0 && lane == 0)
      for (long long ql = q_loaded > kRowSlots ? q_loaded - kRowSlots : 0; ql < q_loaded; ++ql)
        mbar_wait_bounded(&full_bar[ql % kRowSlots], (uint32_t)((ql / kRowSlots) & 1), kDrainWaitLimit);
    if (warp == kResWarp && lane == 0)
      for (long long ql = q_res > kResSlots ? q_res - kResSlots : 0; ql < q_res; ++ql)
        mbar_wait_bounded(&rfull_bar[ql % kResSlots], (uint32_t)((ql / kResSlots) & 1), kDrainWaitLimit);
    if (tid == 0) atomicOr(&g_umma_status, 1u);
  }
  tmem_fence_before();
  __syncthreads();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

template <bool kOutF32, int kNS>
cudaError_t launch_conv16(const CUtensorMap& map, const CUtensorMap& rmap, const __nv_bfloat16* w, const float* bias,
                          int has_res, void* y, const UmmaGeom& g, int relu, uint32_t wl, int grid, cudaStream_t st) {
  const cudaError_t ae =
      cudaFuncSetAttribute(conv16_umma_kernel<kOutF32, kNS>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
  if (ae != cudaSuccess) return ae;
  conv16_umma_kernel<kOutF32, kNS><<<grid, kThreads, kSmemBytes, st>>>(map, rmap, w, bias, has_res, y, g, relu, wl);
  return cudaSuccess;
}

}  // namespace

// 16 -> 16 convolution on the tensor cores (see the file comment). x, w,
// residual, y 16-byte aligned; dil <= 8. Returns SI_OK or an error code.
int conv16_umma(const void* x, const void* w, const float* bias, const void* residual, void* y, int N, int D, int H,
                int W, int dil, int relu, int out_f32, cudaStream_t st) {
  if (dil < 1 || dil > kMaxDil) return set_error(SI_ERR_ARG, "conv16_umma: dilation must be 1..%d", kMaxDil);
  if ((long long)N * D > 0x7FFFFFFFll) return set_error(SI_ERR_ARG, "conv16_umma: too many z-planes");
  const EncodeTiledFn enc = encode_fn();
  if (!enc) return set_error(SI_ERR_CUDA, "conv16_umma: cuTensorMapEncodeTiled unavailable");
  CUtensorMap map;
  std::memset(&map, 0, sizeof(map));
  // {8 channels, x, channel half, y, z*N}: the half dimension (16-byte stride)
  // outside x makes one box land as [half][voxel][8 channels]
  const cuuint64_t dims[5] = {8, (cuuint64_t)W, 2, (cuuint64_t)H, (cuuint64_t)D * (cuuint64_t)N};
  const cuuint64_t strides[4] = {32ull, 16ull, 32ull * W, 32ull * W * H};  // bytes, dims 1..4
  const cuuint32_t box[5] = {8, (cuuint32_t)(kTileM + 2 * dil), 2, 1, 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  const CUresult cr = enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(x), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) return set_error(SI_ERR_CUDA, "conv16_umma: tensor map encoding failed (%d)", (int)cr);
  // the residual, same layout, in boxes of one 128-voxel output tile
  CUtensorMap rmap;
  std::memset(&rmap, 0, sizeof(rmap));
  if (residual) {
    const cuuint32_t rbox[5] = {8, (cuuint32_t)kTileM, 2, 1, 1};
    const CUresult rr = enc(&rmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(residual), dims, strides,
                            rbox, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (rr != CUDA_SUCCESS)
      return set_error(SI_ERR_CUDA, "conv16_umma: residual tensor map encoding failed (%d)", (int)rr);
  }
  UmmaGeom g{N, D, H, W, dil, (W + kTileM - 1) / kTileM, 0};
  g.columns = (long long)N * D * g.xchunks * dil;
  if (g.columns == 0) return SI_OK;
  const int has_res = residual ? 1 : 0;
  const uint32_t wl = wait_limit();
  const long long want = std::min<long long>(g.columns, (long long)sm_count());
  const auto* wb = static_cast<const __nv_bfloat16*>(w);
  const int ns = g_umma_streams.load(std::memory_order_relaxed);
  const cudaError_t ae =
      out_f32 ? (ns == 4 ? launch_conv16<true, 4>(map, rmap, wb, bias, has_res, y, g, relu, wl, (int)want, st)
                 : ns == 2 ? launch_conv16<true, 2>(map, rmap, wb, bias, has_res, y, g, relu, wl, (int)want, st)
                           : launch_conv16<true, 1>(map, rmap, wb, bias, has_res, y, g, relu, wl, (int)want, st))
              : (ns == 4 ? launch_conv16<false, 4>(map, rmap, wb, bias, has_res, y, g, relu, wl, (int)want, st)
                 : ns == 2 ? launch_conv16<false, 2>(map, rmap, wb, bias, has_res, y, g, relu, wl, (int)want, st)
                           : launch_conv16<false, 1>(map, rmap, wb, bias, has_res, y, g, relu, wl, (int)want, st));
  if (ae != cudaSuccess) return set_error(SI_ERR_CUDA, "conv16_umma: shared memory opt-in: %s", cudaGetErrorString(ae));
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

extern "C" int si_nn_conv16_tc_set_streams(int streams) {
  si::clear_error();
  if (streams != 1 && streams != 2 && streams != 4)
    return si::set_error(SI_ERR_ARG, "si_nn_conv16_tc_set_streams: 1, 2 or 4");
  si::g_umma_streams.store(streams, std::memory_order_relaxed);
  return SI_OK;
}
