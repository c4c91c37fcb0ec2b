// Shared device definitions for the smart-interpolation kernels.
//
// Arithmetic in this file is written with explicit round-to-nearest intrinsics
// (__fadd_rn, __fmul_rn, __fmaf_rn) so that every result is a fixed sequence of
// IEEE-754 binary32 operations. The CPU oracle restates the same sequence and
// must reproduce the integer hit maps bit for bit.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace si {

// ---------------------------------------------------------------------------
// Philox4x32-10 counter-based generator.
// Published method: J. Salmon, M. Moraes, R. Dror, D. Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11. Ten rounds of the Philox S-box with the
// key bumped by the Weyl constants between rounds.
// ---------------------------------------------------------------------------
constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;

struct U4 {
  uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += kPhiloxW0;
      k1 += kPhiloxW1;
    }
    const uint32_t hi0 = __umulhi(kPhiloxM0, c.x);
    const uint32_t lo0 = kPhiloxM0 * c.x;
    const uint32_t hi1 = __umulhi(kPhiloxM1, c.z);
    const uint32_t lo1 = kPhiloxM1 * c.z;
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
  }
  return c;
}

// Uniform float in [0, 1) from the top 24 bits of a Philox word (exact).
__device__ __forceinline__ float u01_from_bits(uint32_t bits) {
  return __fmul_rn(__uint2float_rn(bits >> 8), 5.9604644775390625e-8f);  // 2^-24
}

// ---------------------------------------------------------------------------
// The reference walker's own random stream (pycuda_small.py:155-165 state
// set-up, :197-225 update): the recurrence of MRG32k3a written in binary32
// (its products exceed 2^24, so it is not the integer generator), every
// operation rounded on its own as the source reads without contraction:
//   p1 = a12*s11 - a13n*s10; k1 = (long)(p1/m1); p1 -= (float)k1*m1;
//   p1 < 0 -> p1 += m1; shift; the same for p2 with (a21, a23n, m2);
//   u = (p1 <= p2 ? (p1 - p2) + m1 : p1 - p2) * norm.
// All six state words start at the seed's index in the reference's slice
// stack; the stream runs on across the seed's walks.
// ---------------------------------------------------------------------------
struct RefStream {
  float s10, s11, s12, s20, s21, s22;
};

__device__ __forceinline__ float ref_stream_next(RefStream& r) {
  const float m1 = 4294967087.0f, m2 = 4294944443.0f;
  const float a12 = 1403580.0f, a13n = 810728.0f, a21 = 527612.0f, a23n = 1370589.0f;
  const float norm = 2.328306549295728e-10f;
  float p1 = __fsub_rn(__fmul_rn(a12, r.s11), __fmul_rn(a13n, r.s10));
  long long k1 = __float2ll_rz(__fdiv_rn(p1, m1));
  p1 = __fsub_rn(p1, __fmul_rn(__ll2float_rn(k1), m1));
  if (p1 < 0.0f) p1 = __fadd_rn(p1, m1);
  r.s10 = r.s11;
  r.s11 = r.s12;
  r.s12 = p1;
  float p2 = __fsub_rn(__fmul_rn(a21, r.s22), __fmul_rn(a23n, r.s20));
  k1 = __float2ll_rz(__fdiv_rn(p2, m2));
  p2 = __fsub_rn(p2, __fmul_rn(__ll2float_rn(k1), m2));
  if (p2 < 0.0f) p2 = __fadd_rn(p2, m2);
  r.s20 = r.s21;
  r.s21 = r.s22;
  r.s22 = p2;
  if (p1 <= p2) return __fmul_rn(__fadd_rn(__fsub_rn(p1, p2), m1), norm);
  return __fmul_rn(__fsub_rn(p1, p2), norm);
}

// ---------------------------------------------------------------------------
// Edge weight w = 2^(-d2 * c), with c = log2(e) / (2 var) per seed, i.e. the
// Gaussian intensity weight exp(-(B-I)^2 / (2 var)) of the reference walker
// (biomedisa/features/random_walk/pycuda_small.py:133-136), evaluated by our own
// method instead of the CUDA math library:
//   y = d2*c; k = nearest integer to y (round-to-nearest by adding 1.5*2^23);
//   f = y - k in [-0.5, 0.5]; 2^-f by a degree-5 polynomial fitted to 2^x on
//   [-0.5, 0.5] (Chebyshev-node least squares, max rel. error 3e-7 in binary32
//   Horner form); scale by 2^-k through the exponent field.
// Weights with y >= 125 (exp(-86.6) ~ 2.4e-38) are flushed to zero so the
// result is always a normal number or exactly zero.
// ---------------------------------------------------------------------------
constexpr float kLog2e = 1.44269502162933349609375f;  // binary32 nearest log2(e)
constexpr float kRoundMagic = 12582912.0f;              // 1.5 * 2^23
constexpr float kWeightYMax = 125.0f;
constexpr float kP1 = 0.6931470036506653f;   // 0x3f317215
constexpr float kP2 = 0.2402222454547882f;   // 0x3e75fcd2
constexpr float kP3 = 0.055507123470306396f; // 0x3d635b70
constexpr float kP4 = 0.009670175611972809f; // 0x3c1e6fa8
constexpr float kP5 = 0.0013260921696200967f;// 0x3aadd045

__device__ __forceinline__ float edge_weight(float d2, float c) {
  const float y = __fmul_rn(d2, c);
  if (!(y < kWeightYMax)) return 0.0f;
  const float r = __fadd_rn(y, kRoundMagic);
  const float kf = __fsub_rn(r, kRoundMagic);
  const float g = __fsub_rn(kf, y);  // = -(y - k), exact
  float p = __fmaf_rn(kP5, g, kP4);
  p = __fmaf_rn(p, g, kP3);
  p = __fmaf_rn(p, g, kP2);
  p = __fmaf_rn(p, g, kP1);
  p = __fmaf_rn(p, g, 1.0f);
  const int k = __float_as_int(r) - 0x4B400000;
  return __int_as_float(__float_as_int(p) - (k << 23));
}

// ---------------------------------------------------------------------------
// Two edge weights at once on the packed binary32 pipe of sm_100-class SMs
// (add/sub/fma.rn.f32x2: one instruction, two independent IEEE-754
// round-to-nearest results). Each lane performs exactly the operation sequence
// of edge_weight() above, so the pair equals two scalar calls bit for bit. The
// walker is issue-bound and this halves the floating-point instructions of its
// six weights. Operands travel as 64-bit registers {lo, hi}.
//
// Products: ptxas fuses a packed mul.rn.f32x2 into a following packed add or
// sub (one rounding instead of two), with or without --fmad=false, and it
// also folds fma(a, b, -0.0) with a literal -0.0 back into that product. A
// packed product is therefore written as fma(a, b, z) with z = -0.0 read at
// run time from a mutable device variable (f2_negzero): RN(a*b + -0) equals
// RN(a*b) for every input (signed zeros, infinities and NaN included), and an
// FMA result cannot be fused further. Measured on the GB300: a mul->add chain
// differed from the two-rounding sequence in 41 % of random pairs, every time
// equal to the fused result; with the run-time -0 addend in none.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t f2_pack(float lo, float hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f2_unpack(uint64_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ void u2_unpack(uint64_t v, uint32_t& lo, uint32_t& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t f2_sub(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
__device__ __forceinline__ uint64_t f2_splat(float v) { return f2_pack(v, v); }

// -0.0 that neither compiler can see (read once per thread; see above).
static __device__ float g_opaque_negzero = -0.0f;
__device__ __forceinline__ uint64_t f2_negzero() {
  return f2_splat(*static_cast<volatile float*>(&g_opaque_negzero));
}
// Packed product RN(a*b) that is never fused into a later sum; nz = f2_negzero().
__device__ __forceinline__ uint64_t f2_mul(uint64_t a, uint64_t b, uint64_t nz) { return f2_fma(a, b, nz); }

// Weights of the two neighbours whose (B - I) differences are the lanes of d;
// cc = {c, c}. Returns w_lo, w_hi equal to edge_weight(d_lo^2, c) and
// edge_weight(d_hi^2, c).
__device__ __forceinline__ void edge_weight_pair(uint64_t d, uint64_t cc, uint64_t nz, float& w_lo, float& w_hi) {
  const uint64_t magic2 = f2_splat(kRoundMagic);
  const uint64_t y = f2_mul(f2_mul(d, d, nz), cc, nz);
  const uint64_t r = f2_add(y, magic2);
  const uint64_t g = f2_sub(f2_sub(r, magic2), y);
  uint64_t p = f2_fma(f2_splat(kP5), g, f2_splat(kP4));
  p = f2_fma(p, g, f2_splat(kP3));
  p = f2_fma(p, g, f2_splat(kP2));
  p = f2_fma(p, g, f2_splat(kP1));
  p = f2_fma(p, g, f2_splat(1.0f));
  uint32_t p_lo, p_hi, r_lo, r_hi;
  u2_unpack(p, p_lo, p_hi);
  u2_unpack(r, r_lo, r_hi);
  float y_lo, y_hi;
  f2_unpack(y, y_lo, y_hi);
  // 2^-k through the exponent field: k = bits(r) - bits(1.5*2^23), and
  // (bits(1.5*2^23) << 23) vanishes modulo 2^32, so k << 23 == bits(r) << 23.
  w_lo = y_lo < kWeightYMax ? __uint_as_float(p_lo - (r_lo << 23)) : 0.0f;
  w_hi = y_hi < kWeightYMax ? __uint_as_float(p_hi - (r_hi << 23)) : 0.0f;
}

// Per-seed weight constant c = RN(RN(1 / RN(2 var)) * log2e).
__device__ __forceinline__ float weight_constant(float var) {
  const float div1 = __fdiv_rn(1.0f, __fmul_rn(2.0f, var));
  return __fmul_rn(div1, kLog2e);
}

// ---------------------------------------------------------------------------
// One walker start point. pos is the linear index in the working (cropped,
// padded) volume; c is the weight constant; b is the seed intensity.
// meta: bits 0-7 label slot, bits 8-9 seed axis, bits 16-23 label value.
// ---------------------------------------------------------------------------
struct __align__(16) SeedRec {
  uint32_t pos;
  float c;
  float b;
  uint32_t meta;
};

__host__ __device__ __forceinline__ uint32_t seed_slot(uint32_t meta) { return meta & 0xFFu; }
__host__ __device__ __forceinline__ uint32_t seed_axis(uint32_t meta) { return (meta >> 8) & 0x3u; }
__host__ __device__ __forceinline__ uint32_t seed_label(uint32_t meta) { return (meta >> 16) & 0xFFu; }

// ---------------------------------------------------------------------------
// Walker steps t in [t, t_end) from voxel pos over packed neighbourhood
// records (8-byte uint8 records or 32-byte float records, see si_walk.cu).
// Returns the final position. s_delta[d]: linear offset of move d.
// Semantics: pycuda_small.py:183-253 (weights, cumulative intervals, rnd == 0
// -> +z, refused border moves count as steps, one hit per accepted move).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float byte_plus_2p23(uint32_t w, uint32_t k) {
  return __int_as_float((int)__byte_perm(w, 0x4B000000u, 0x7540u + k));
}

// A voxel's packed neighbourhood record: 8 bytes for uint8 volumes, 32 for
// float volumes (see si_walk.cu).
template <bool kFloat>
struct WalkRec;
template <>
struct WalkRec<false> {
  uint2 r;
};
template <>
struct WalkRec<true> {
  float4 a, b;
};

template <bool kFloat>
__device__ __forceinline__ WalkRec<kFloat> load_rec(const void* __restrict__ packed_v, uint32_t pos);
template <>
__device__ __forceinline__ WalkRec<false> load_rec<false>(const void* __restrict__ packed_v, uint32_t pos) {
  return WalkRec<false>{static_cast<const uint2*>(packed_v)[pos]};
}
template <>
__device__ __forceinline__ WalkRec<true> load_rec<true>(const void* __restrict__ packed_v, uint32_t pos) {
  const float4* rec = static_cast<const float4*>(packed_v) + 2 * (size_t)pos;
  return WalkRec<true>{rec[0], rec[1]};
}

// One step from voxel pos, whose record is rec, with the uniform variate u in
// [0, 1) given.
template <bool kFloat>
__device__ __forceinline__ uint32_t step_from_rec(const WalkRec<kFloat>& rec, uint32_t pos, float u, float c,
                                                  float bf, float b23, uint32_t* __restrict__ hl,
                                                  const int32_t* s_delta, uint64_t nz) {
  float w0, w1, w2, w3, w4, w5;
  uint32_t mask;
  // The (B - I) differences are formed pairwise (+z,-z), (+y,-y), (+x,-x) and
  // weighted on the packed pipe; d = B - I is exact in both record kinds
  // (uint8: (2^23 + B) - (2^23 + I); float: one RN subtraction, as before).
  const uint64_t cc = f2_splat(c);
  if constexpr (kFloat) {
    const uint64_t bf2 = f2_splat(bf);
    edge_weight_pair(f2_sub(bf2, f2_pack(rec.a.x, rec.a.y)), cc, nz, w0, w1);
    edge_weight_pair(f2_sub(bf2, f2_pack(rec.a.z, rec.a.w)), cc, nz, w2, w3);
    edge_weight_pair(f2_sub(bf2, f2_pack(rec.b.x, rec.b.y)), cc, nz, w4, w5);
    mask = __float_as_uint(rec.b.z);
  } else {
    const uint2 r = rec.r;
    const uint64_t b2 = f2_splat(b23);
    edge_weight_pair(f2_sub(b2, f2_pack(byte_plus_2p23(r.x, 0), byte_plus_2p23(r.x, 1))), cc, nz, w0, w1);
    edge_weight_pair(f2_sub(b2, f2_pack(byte_plus_2p23(r.x, 2), byte_plus_2p23(r.x, 3))), cc, nz, w2, w3);
    edge_weight_pair(f2_sub(b2, f2_pack(byte_plus_2p23(r.y, 0), byte_plus_2p23(r.y, 1))), cc, nz, w4, w5);
    mask = r.y >> 16;
  }
  const float c1 = __fadd_rn(w0, w1);
  const float c2 = __fadd_rn(c1, w2);
  const float c3 = __fadd_rn(c2, w3);
  const float c4 = __fadd_rn(c3, w4);
  const float c5 = __fadd_rn(c4, w5);
  const float rnd = __fmul_rn(c5, u);
  int dir = (int)(w0 <= rnd) + (int)(c1 <= rnd) + (int)(c2 <= rnd) + (int)(c3 <= rnd) + (int)(c4 <= rnd);
  if (rnd == 0.0f) dir = 0;
  if (!((mask >> dir) & 1u)) {
    pos += (uint32_t)s_delta[dir];
    atomicAdd(&hl[pos], 1u);
  }
  return pos;
}

// One step with the uniform variate u in [0, 1) given.
template <bool kFloat>
__device__ __forceinline__ uint32_t walk_step_u(const void* __restrict__ packed_v, uint32_t pos, float u, float c,
                                                float bf, float b23, uint32_t* __restrict__ hl,
                                                const int32_t* s_delta, uint64_t nz) {
  return step_from_rec<kFloat>(load_rec<kFloat>(packed_v, pos), pos, u, c, bf, b23, hl, s_delta, nz);
}

// One step with u taken from the top 24 bits of a Philox word.
template <bool kFloat>
__device__ __forceinline__ uint32_t walk_step(const void* __restrict__ packed_v, uint32_t pos, uint32_t bits, float c,
                                              float bf, float b23, uint32_t* __restrict__ hl,
                                              const int32_t* s_delta, uint64_t nz) {
  return walk_step_u<kFloat>(packed_v, pos, u01_from_bits(bits), c, bf, b23, hl, s_delta, nz);
}

__device__ __forceinline__ uint32_t philox_word(const U4& r, uint32_t sub) {
  return sub == 0u ? r.x : (sub == 1u ? r.y : (sub == 2u ? r.z : r.w));
}

// Steps t in [t, t_end): step t uses word (t & 3) of the Philox block t >> 2.
// Aligned groups of four steps share one block evaluation; the unaligned head
// and tail take their words one by one (same words, same order).
template <bool kFloat>
__device__ __forceinline__ uint32_t walk_steps(const void* __restrict__ packed_v, uint32_t pos, uint32_t t,
                                               uint32_t t_end, float c, float bf, uint32_t seed_pos,
                                               uint32_t axis, uint32_t label, uint32_t k0, uint32_t k1,
                                               uint32_t* __restrict__ hl, const int32_t* s_delta, uint64_t nz) {
  const float b23 = __fadd_rn(bf, 8388608.0f);  // 2^23 + B, exact for uint8 B
  if ((t & 3u) && t < t_end) {
    const U4 rr = philox4x32_10(U4{t >> 2, seed_pos, axis, label}, k0, k1);
    for (; (t & 3u) && t < t_end; ++t)
      pos = walk_step<kFloat>(packed_v, pos, philox_word(rr, t & 3u), c, bf, b23, hl, s_delta, nz);
  }
  for (; t + 4u <= t_end; t += 4u) {
    const U4 rr = philox4x32_10(U4{t >> 2, seed_pos, axis, label}, k0, k1);
    pos = walk_step<kFloat>(packed_v, pos, rr.x, c, bf, b23, hl, s_delta, nz);
    pos = walk_step<kFloat>(packed_v, pos, rr.y, c, bf, b23, hl, s_delta, nz);
    pos = walk_step<kFloat>(packed_v, pos, rr.z, c, bf, b23, hl, s_delta, nz);
    pos = walk_step<kFloat>(packed_v, pos, rr.w, c, bf, b23, hl, s_delta, nz);
  }
  if (t < t_end) {
    const U4 rr = philox4x32_10(U4{t >> 2, seed_pos, axis, label}, k0, k1);
    for (; t < t_end; ++t)
      pos = walk_step<kFloat>(packed_v, pos, philox_word(rr, t & 3u), c, bf, b23, hl, s_delta, nz);
  }
  return pos;
}

// One walker of a group advanced together (walk_steps_multi).
struct PairWalker {
  uint32_t pos, t, t_end;
  float c, bf, b23;
  uint32_t seed_pos, axis, label;
  uint32_t* hl;
};

__device__ __forceinline__ PairWalker pair_walker(uint32_t pos, uint32_t t, uint32_t t_end, float c, float bf,
                                                  uint32_t seed_pos, uint32_t axis, uint32_t label, uint32_t* hl) {
  return PairWalker{pos, t, t_end, c, bf, __fadd_rn(bf, 8388608.0f), seed_pos, axis, label, hl};
}

// N walkers advanced together: while all are on aligned blocks of four
// steps, each step issues the N record loads before any weight evaluation,
// so one thread keeps N dependent gathers in flight. Every walker takes the
// same steps, words and hits as walk_steps alone (each walker's own step
// order is unchanged; hits are commutative counts).
template <bool kFloat, int N>
__device__ __forceinline__ void walk_steps_multi(const void* __restrict__ packed_v, PairWalker (&W)[N], uint32_t k0,
                                                 uint32_t k1, const int32_t* s_delta, uint64_t nz) {
  uint32_t any_t = 0u, n = 0xFFFFFFFFu;
#pragma unroll
  for (int w = 0; w < N; ++w) {
    any_t |= W[w].t;
    n = min(n, W[w].t_end - W[w].t);
  }
  if ((any_t & 3u) == 0u) {
    n &= ~3u;
    for (uint32_t k = 0; k < n; k += 4u) {
      U4 r[N];
#pragma unroll
      for (int w = 0; w < N; ++w) r[w] = philox4x32_10(U4{W[w].t >> 2, W[w].seed_pos, W[w].axis, W[w].label}, k0, k1);
#pragma unroll
      for (uint32_t j = 0; j < 4u; ++j) {
        WalkRec<kFloat> q[N];
#pragma unroll
        for (int w = 0; w < N; ++w) q[w] = load_rec<kFloat>(packed_v, W[w].pos);
#pragma unroll
        for (int w = 0; w < N; ++w)
          W[w].pos = step_from_rec<kFloat>(q[w], W[w].pos, u01_from_bits(philox_word(r[w], j)), W[w].c, W[w].bf,
                                           W[w].b23, W[w].hl, s_delta, nz);
      }
#pragma unroll
      for (int w = 0; w < N; ++w) W[w].t += 4u;
    }
  }
#pragma unroll
  for (int w = 0; w < N; ++w) {
    W[w].pos = walk_steps<kFloat>(packed_v, W[w].pos, W[w].t, W[w].t_end, W[w].c, W[w].bf, W[w].seed_pos, W[w].axis,
                                  W[w].label, k0, k1, W[w].hl, s_delta, nz);
    W[w].t = W[w].t_end;
  }
}

}  // namespace si
