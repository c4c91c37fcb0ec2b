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

// ---------------------------------------------------------------------------
// Packed neighbourhood records. For every interior voxel v of the working
// volume one record holds the six neighbour intensities in move order
// (+z, -z, +y, -y, +x, -x), a refusal mask (bit d set when move d would leave
// [1, dim-2], pycuda_small.py:236) and I[v]. A walker step then reads ONE
// record instead of gathering six voxels, and needs no coordinates.
//   uint8 volume: 8 bytes  {n0..n5, mask, I[v]}
//   float volume: 32 bytes {n0..n5, mask (as bits), I[v]}
// Records of non-interior voxels are zero and never read.
// ---------------------------------------------------------------------------
template <bool kFloat>
__global__ void __launch_bounds__(256) pack_kernel(const void* __restrict__ work_v, int Zc, int Yc, int Xc,
                                                   void* __restrict__ packed_v) {
  const uint32_t F = (uint32_t)Yc * (uint32_t)Xc;
  const uint64_t V = (uint64_t)F * Zc;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < V; i += stride) {
    const int x = (int)(i % Xc);
    const uint64_t zy = i / Xc;
    const int y = (int)(zy % Yc);
    const int z = (int)(zy / Yc);
    const bool inner = z > 0 && y > 0 && x > 0 && z < Zc - 1 && y < Yc - 1 && x < Xc - 1;
    uint32_t mask = 0;
    if (inner) {
      mask |= (z + 1 >= Zc - 1) ? 1u : 0u;
      mask |= (z - 1 <= 0) ? 2u : 0u;
      mask |= (y + 1 >= Yc - 1) ? 4u : 0u;
      mask |= (y - 1 <= 0) ? 8u : 0u;
      mask |= (x + 1 >= Xc - 1) ? 16u : 0u;
      mask |= (x - 1 <= 0) ? 32u : 0u;
    }
    if (kFloat) {
      const float* img = static_cast<const float*>(work_v);
      float4* out = static_cast<float4*>(packed_v) + 2 * i;
      if (inner) {
        out[0] = make_float4(img[i + F], img[i - F], img[i + Xc], img[i - Xc]);
        out[1] = make_float4(img[i + 1], img[i - 1], __uint_as_float(mask), img[i]);
      } else {
        out[0] = make_float4(0.f, 0.f, 0.f, 0.f);
        out[1] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    } else {
      const uint8_t* img = static_cast<const uint8_t*>(work_v);
      uint2 r = make_uint2(0u, 0u);
      if (inner) {
        r.x = (uint32_t)img[i + F] | ((uint32_t)img[i - F] << 8) | ((uint32_t)img[i + Xc] << 16) |
              ((uint32_t)img[i - Xc] << 24);
        r.y = (uint32_t)img[i + 1] | ((uint32_t)img[i - 1] << 8) | (mask << 16) | ((uint32_t)img[i] << 24);
      }
      static_cast<uint2*>(packed_v)[i] = r;
    }
  }
}

template <bool kFloat>
__global__ void __launch_bounds__(256) walk_kernel(const void* __restrict__ packed_v, int Zc, int Yc, int Xc,
                                                   const SeedRec* __restrict__ seeds,
                                                   const uint32_t* __restrict__ n_seeds_ptr, uint32_t max_seeds,
                                                   int nbrw, int sorw, uint32_t k0, uint32_t k1,
                                                   uint32_t* __restrict__ hits, int order) {
  __shared__ int32_t s_delta[6];
  const uint32_t F = (uint32_t)Yc * (uint32_t)Xc;
  if (threadIdx.x < 6) {
    const int32_t d[6] = {(int32_t)F, -(int32_t)F, Xc, -Xc, 1, -1};
    s_delta[threadIdx.x] = d[threadIdx.x];
  }
  __syncthreads();
  const uint32_t ns = min(*n_seeds_ptr, max_seeds);
  if (ns == 0) return;
  const uint64_t total = (uint64_t)ns * (uint32_t)nbrw;
  const uint64_t nz = f2_negzero();
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
    uint32_t* __restrict__ hl = hits + (size_t)seed_slot(sd.meta) * V;
    const uint32_t t0 = n * (uint32_t)sorw;
    walk_steps<kFloat>(packed_v, sd.pos, t0, t0 + (uint32_t)sorw, sd.c, sd.b, sd.pos, seed_axis(sd.meta),
                       seed_label(sd.meta), k0, k1, hl, s_delta, nz);
  }
}

// ---------------------------------------------------------------------------
// Walker on the reference's own random stream (ref_stream_next): one thread
// per seed runs the seed's nbrw walks of sorw steps one after the other, the
// stream continuing across walks as in the reference kernel
// (pycuda_small.py:180-254). The stream of a seed starts at its index in the
// reference's slice stack: rank * R * C + r * C + c, where rank is the
// seed's slice among the listed slices of its axis (stack_rank) and (r, c) /
// (R, C) its in-slice position / the slice's size (pycuda_small.py:145-165;
// the all-axis kernels index their per-axis stacks the same way). Weights,
// border rule and hits are those of walk_step.
// ---------------------------------------------------------------------------
template <bool kFloat>
__global__ void __launch_bounds__(128) walk_refstream_kernel(const void* __restrict__ packed_v, int Zc, int Yc, int Xc,
                                                             const SeedRec* __restrict__ seeds,
                                                             const uint32_t* __restrict__ n_seeds_ptr,
                                                             uint32_t max_seeds, int nbrw, int sorw,
                                                             const int32_t* __restrict__ stack_rank,
                                                             uint32_t* __restrict__ hits) {
  __shared__ int32_t s_delta[6];
  const uint32_t F = (uint32_t)Yc * (uint32_t)Xc;
  if (threadIdx.x < 6) {
    const int32_t d[6] = {(int32_t)F, -(int32_t)F, Xc, -Xc, 1, -1};
    s_delta[threadIdx.x] = d[threadIdx.x];
  }
  __syncthreads();
  const uint32_t ns = min(*n_seeds_ptr, max_seeds);
  const size_t V = (size_t)F * Zc;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint64_t nz = f2_negzero();
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += stride) {
    const SeedRec sd = seeds[s];
    const uint32_t z = sd.pos / F, rem = sd.pos - z * F;
    const uint32_t y = rem / (uint32_t)Xc, x = rem - y * (uint32_t)Xc;
    const uint32_t axis = seed_axis(sd.meta);
    int32_t index;
    if (axis == 0)
      index = stack_rank[z] * (int32_t)F + (int32_t)(y * Xc + x);
    else if (axis == 1)
      index = stack_rank[Zc + y] * (Zc * Xc) + (int32_t)(z * Xc + x);
    else
      index = stack_rank[Zc + Yc + x] * (Zc * Yc) + (int32_t)(z * Yc + y);
    const float init = __int2float_rn(index);
    RefStream r{init, init, init, init, init, init};
    uint32_t* __restrict__ hl = hits + (size_t)seed_slot(sd.meta) * V;
    const float b23 = __fadd_rn(sd.b, 8388608.0f);
    for (int w = 0; w < nbrw; ++w) {
      uint32_t pos = sd.pos;
      for (int t = 0; t < sorw; ++t)
        pos = walk_step_u<kFloat>(packed_v, pos, ref_stream_next(r), sd.c, sd.b, b23, hl, s_delta, nz);
    }
  }
}

}  // namespace
}  // namespace si

using namespace si;

extern "C" int si_walk_refstream(const void* packed, int work_is_float, int Zc, int Yc, int Xc,
                                 const si_seed_t* seeds, const uint32_t* n_seeds, uint32_t max_seeds, int nbrw,
                                 int sorw, const int32_t* stack_rank, uint32_t* hits, int nol, void* stream) {
  clear_error();
  if (!packed || !seeds || !n_seeds || !hits || !stack_rank)
    return set_error(SI_ERR_ARG, "si_walk_refstream: null pointer");
  if (Zc < 3 || Yc < 3 || Xc < 3) return set_error(SI_ERR_ARG, "si_walk_refstream: bad dims");
  if ((uint64_t)Zc * Yc * Xc > 0x7FFFFFFFull)
    return set_error(SI_ERR_LIMIT, "si_walk_refstream: volume above 2^31 voxels (the reference's int indices)");
  if (nbrw < 0 || sorw < 0) return set_error(SI_ERR_ARG, "si_walk_refstream: negative nbrw/sorw");
  if (nol < 1 || nol > 256) return set_error(SI_ERR_ARG, "si_walk_refstream: nol must be 1..256");
  if (nbrw == 0 || sorw == 0 || max_seeds == 0) return SI_OK;
  const int block = 128;
  const uint64_t want = ((uint64_t)max_seeds + block - 1) / block, cap = (uint64_t)sm_count() * 16;
  const int grid = (int)(want < cap ? want : cap);
  const SeedRec* sd = reinterpret_cast<const SeedRec*>(seeds);
  cudaStream_t st = as_stream(stream);
  if (work_is_float)
    walk_refstream_kernel<true><<<grid, block, 0, st>>>(packed, Zc, Yc, Xc, sd, n_seeds, max_seeds, nbrw, sorw,
                                                        stack_rank, hits);
  else
    walk_refstream_kernel<false><<<grid, block, 0, st>>>(packed, Zc, Yc, Xc, sd, n_seeds, max_seeds, nbrw, sorw,
                                                         stack_rank, hits);
  return check_launch("si_walk_refstream");
}

extern "C" int si_pack_neighbours(const void* work, int work_is_float, int Zc, int Yc, int Xc, void* packed,
                                  void* stream) {
  clear_error();
  if (!work || !packed) return set_error(SI_ERR_ARG, "si_pack_neighbours: null pointer");
  if (Zc < 3 || Yc < 3 || Xc < 3) return set_error(SI_ERR_ARG, "si_pack_neighbours: bad dims");
  if ((uint64_t)Zc * Yc * Xc > 0xFFFFFFFFull)
    return set_error(SI_ERR_LIMIT, "si_pack_neighbours: volume above 2^32 voxels");
  const uint64_t V = (uint64_t)Zc * Yc * Xc;
  const int block = 256;
  const uint64_t want = (V + block - 1) / block, cap = (uint64_t)sm_count() * 16;
  const int grid = (int)(want < cap ? want : cap);
  cudaStream_t st = as_stream(stream);
  if (work_is_float)
    pack_kernel<true><<<grid, block, 0, st>>>(work, Zc, Yc, Xc, packed);
  else
    pack_kernel<false><<<grid, block, 0, st>>>(work, Zc, Yc, Xc, packed);
  return check_launch("si_pack_neighbours");
}

extern "C" int si_walk(const void* packed, int work_is_float, int Zc, int Yc, int Xc, const si_seed_t* seeds,
                       const uint32_t* n_seeds, uint32_t max_seeds, int nbrw, int sorw, uint64_t key,
                       uint32_t* hits, int nol, int grid, int block, int order, void* stream) {
  clear_error();
  if (!packed || !seeds || !n_seeds || !hits) return set_error(SI_ERR_ARG, "si_walk: null pointer");
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
    walk_kernel<true><<<grid, block, 0, st>>>(packed, Zc, Yc, Xc, sd, n_seeds, max_seeds, nbrw, sorw, k0, k1, hits,
                                              order);
  else
    walk_kernel<false><<<grid, block, 0, st>>>(packed, Zc, Yc, Xc, sd, n_seeds, max_seeds, nbrw, sorw, k0, k1, hits,
                                               order);
  return check_launch("si_walk");
}
