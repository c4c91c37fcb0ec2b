// Random-walker kernel of smart interpolation.
//
// Semantics follow the reference walker Funktion
// (biomedisa/features/random_walk/pycuda_small.py:138-257):
//   * weights of the six moves (+z, -z, +y, -y, +x, -x) use the SEED intensity B
//     and the seed's variance: w = exp(-(B - I)^2 / (2 var)) (here 2^(-d2 c));
//   * cumulative sums W0..W5, rnd = W5 * u; the move is the first interval that
//     holds rnd, and rnd == 0 always picks +z (:227-233);
//   * a move whose target leaves [1, dim-2] is refused, the step still counts
//     and records nothing (:235-242);
//   * every accepted move adds one hit at the target voxel;
//   * nbrw walks of sorw steps restart at the seed (:244-253).
// Randomness is Philox4x32-10, counter (t / 4, seed pos, seed axis, label
// value) with t = walk * sorw + step, key = user key. Because every walk has
// its own counter range the nbrw walks of a seed are independent work items,
// and integer hit sums make the result independent of scheduling.
#include "si_common.cuh"
#include "si_internal.h"

namespace si {
namespace {

__device__ __forceinline__ uint32_t pick_word(const U4& r, uint32_t sub) {
  return sub == 0u ? r.x : (sub == 1u ? r.y : (sub == 2u ? r.z : r.w));
}

template <bool kFloat>
__global__ void __launch_bounds__(256) walk_kernel(const void* __restrict__ work_v, int Zc, int Yc, int Xc,
                                                   const SeedRec* __restrict__ seeds,
                                                   const uint32_t* __restrict__ n_seeds_ptr, uint32_t max_seeds,
                                                   int nbrw, int sorw, uint32_t k0, uint32_t k1,
                                                   uint32_t* __restrict__ hits, int order) {
  const uint32_t ns = min(*n_seeds_ptr, max_seeds);
  if (ns == 0) return;
  const uint64_t total = (uint64_t)ns * (uint32_t)nbrw;
  const uint32_t F = (uint32_t)Yc * (uint32_t)Xc;
  const size_t V = (size_t)F * Zc;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t item = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; item < total; item += stride) {
    uint32_t s, n;
    if (order == 0) {
      n = (uint32_t)(item / ns);
      s = (uint32_t)(item - (uint64_t)n * ns);
    } else {
      s = (uint32_t)(item / (uint32_t)nbrw);
      n = (uint32_t)(item - (uint64_t)s * (uint32_t)nbrw);
    }
    const SeedRec sd = seeds[s];
    uint32_t pos = sd.pos;
    int z = (int)(pos / F);
    const uint32_t rem = pos - (uint32_t)z * F;
    int y = (int)(rem / (uint32_t)Xc);
    int x = (int)(rem - (uint32_t)y * (uint32_t)Xc);
    const float c = sd.c;
    const float bf = sd.b;
    const int bi = (int)bf;
    uint32_t* __restrict__ hl = hits + (size_t)seed_slot(sd.meta) * V;
    const uint32_t axis = seed_axis(sd.meta), label = seed_label(sd.meta);
    uint32_t t = n * (uint32_t)sorw;
    U4 rr = philox4x32_10(U4{t >> 2, sd.pos, axis, label}, k0, k1);
    for (int st = 0; st < sorw; ++st, ++t) {
      const uint32_t sub = t & 3u;
      if (sub == 0u && st != 0) rr = philox4x32_10(U4{t >> 2, sd.pos, axis, label}, k0, k1);
      const uint32_t bits = pick_word(rr, sub);
      float w0, w1, w2, w3, w4, w5;
      if (kFloat) {
        const float* __restrict__ img = static_cast<const float*>(work_v);
        float d;
        d = __fsub_rn(bf, img[pos + F]); w0 = edge_weight(__fmul_rn(d, d), c);
        d = __fsub_rn(bf, img[pos - F]); w1 = edge_weight(__fmul_rn(d, d), c);
        d = __fsub_rn(bf, img[pos + Xc]); w2 = edge_weight(__fmul_rn(d, d), c);
        d = __fsub_rn(bf, img[pos - Xc]); w3 = edge_weight(__fmul_rn(d, d), c);
        d = __fsub_rn(bf, img[pos + 1]); w4 = edge_weight(__fmul_rn(d, d), c);
        d = __fsub_rn(bf, img[pos - 1]); w5 = edge_weight(__fmul_rn(d, d), c);
      } else {
        const uint8_t* __restrict__ img = static_cast<const uint8_t*>(work_v);
        int d;
        d = bi - (int)img[pos + F]; w0 = edge_weight(__int2float_rn(d * d), c);
        d = bi - (int)img[pos - F]; w1 = edge_weight(__int2float_rn(d * d), c);
        d = bi - (int)img[pos + Xc]; w2 = edge_weight(__int2float_rn(d * d), c);
        d = bi - (int)img[pos - Xc]; w3 = edge_weight(__int2float_rn(d * d), c);
        d = bi - (int)img[pos + 1]; w4 = edge_weight(__int2float_rn(d * d), c);
        d = bi - (int)img[pos - 1]; w5 = edge_weight(__int2float_rn(d * d), c);
      }
      const float c1 = __fadd_rn(w0, w1);
      const float c2 = __fadd_rn(c1, w2);
      const float c3 = __fadd_rn(c2, w3);
      const float c4 = __fadd_rn(c3, w4);
      const float c5 = __fadd_rn(c4, w5);
      const float rnd = __fmul_rn(c5, u01_from_bits(bits));
      int dir = (int)(w0 <= rnd) + (int)(c1 <= rnd) + (int)(c2 <= rnd) + (int)(c3 <= rnd) + (int)(c4 <= rnd);
      if (rnd == 0.0f) dir = 0;
      const bool plus = (dir & 1) == 0;
      const int axis_dir = dir >> 1;  // 0: z, 1: y, 2: x
      const int coord = axis_dir == 0 ? z : (axis_dir == 1 ? y : x);
      const int hi = (axis_dir == 0 ? Zc : (axis_dir == 1 ? Yc : Xc)) - 2;
      const bool ok = plus ? (coord < hi) : (coord > 1);
      if (ok) {
        const uint32_t step = axis_dir == 0 ? F : (axis_dir == 1 ? (uint32_t)Xc : 1u);
        const int dc = plus ? 1 : -1;
        pos = plus ? pos + step : pos - step;
        if (axis_dir == 0) z += dc;
        else if (axis_dir == 1) y += dc;
        else x += dc;
        atomicAdd(&hl[pos], 1u);
      }
    }
  }
}

}  // namespace
}  // namespace si

using namespace si;

extern "C" int si_walk(const void* work, int work_is_float, int Zc, int Yc, int Xc, const si_seed_t* seeds,
                       const uint32_t* n_seeds, uint32_t max_seeds, int nbrw, int sorw, uint64_t key,
                       uint32_t* hits, int nol, int grid, int block, int order, void* stream) {
  clear_error();
  if (!work || !seeds || !n_seeds || !hits) return set_error(SI_ERR_ARG, "si_walk: null pointer");
  if (Zc < 3 || Yc < 3 || Xc < 3) return set_error(SI_ERR_ARG, "si_walk: bad dims");
  if ((uint64_t)Zc * Yc * Xc > 0xFFFFFFFFull) return set_error(SI_ERR_LIMIT, "si_walk: volume above 2^32 voxels");
  if (nbrw < 0 || sorw < 0) return set_error(SI_ERR_ARG, "si_walk: negative nbrw/sorw");
  if ((uint64_t)nbrw * (uint64_t)sorw > 0xFFFFFFFFull)
    return set_error(SI_ERR_LIMIT, "si_walk: nbrw*sorw above 2^32 steps");
  if (nol < 1 || nol > 256) return set_error(SI_ERR_ARG, "si_walk: nol must be 1..256");
  if (order != 0 && order != 1) return set_error(SI_ERR_ARG, "si_walk: order must be 0 or 1");
  if (nbrw == 0 || sorw == 0 || max_seeds == 0) return SI_OK;
  if (block <= 0) block = 256;
  if (block > 256 || (block & 31)) return set_error(SI_ERR_ARG, "si_walk: block must be a multiple of 32, <= 256");
  if (grid <= 0) grid = sm_count() * (2048 / block);
  const uint32_t k0 = (uint32_t)(key & 0xFFFFFFFFull), k1 = (uint32_t)(key >> 32);
  const SeedRec* sd = reinterpret_cast<const SeedRec*>(seeds);
  cudaStream_t st = as_stream(stream);
  if (work_is_float)
    walk_kernel<true><<<grid, block, 0, st>>>(work, Zc, Yc, Xc, sd, n_seeds, max_seeds, nbrw, sorw, k0, k1, hits,
                                              order);
  else
    walk_kernel<false><<<grid, block, 0, st>>>(work, Zc, Yc, Xc, sd, n_seeds, max_seeds, nbrw, sorw, k0, k1, hits,
                                               order);
  return check_launch("si_walk");
}
