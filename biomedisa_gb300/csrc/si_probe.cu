// Measurement probes for the roofline denominators of the walker: L2 read
// bandwidth (16-byte loads that bypass L1 over an L2-resident buffer) and L2
// atomic throughput (random 4-byte atomic adds into an L2-resident buffer).
// They are not part of the interpolation path.
#include "si_common.cuh"
#include "si_internal.h"

namespace si {
namespace {

__global__ void __launch_bounds__(256) l2_read_kernel(const uint4* __restrict__ buf, uint64_t n16, int reps,
                                                      uint32_t* __restrict__ sink) {
  uint32_t acc = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (int r = 0; r < reps; ++r)
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride) {
      const uint4 v = __ldcg(&buf[i]);
      acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
  if (acc == 0x9E3779B9u) sink[0] = acc;  // keeps the loads; practically never stores
}

__global__ void __launch_bounds__(256) l2_atomic_kernel(uint32_t* __restrict__ buf, uint32_t word_mask,
                                                        uint64_t n_atomics, uint32_t seed) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_atomics; i += stride) {
    // xorshift-multiply hash of the index: scattered addresses
    uint32_t h = (uint32_t)i * 0x9E3779B1u ^ seed;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    atomicAdd(&buf[h & word_mask], 1u);
  }
}

}  // namespace
}  // namespace si

using namespace si;

extern "C" int si_probe_l2_read(const void* buf, uint64_t bytes, int reps, uint32_t* sink, void* stream) {
  clear_error();
  if (!buf || !sink || bytes < 16 || reps < 1) return set_error(SI_ERR_ARG, "si_probe_l2_read: bad arguments");
  const int grid = sm_count() * 8;
  l2_read_kernel<<<grid, 256, 0, as_stream(stream)>>>(static_cast<const uint4*>(buf), bytes / 16, reps, sink);
  return check_launch("si_probe_l2_read");
}

extern "C" int si_probe_l2_atomics(uint32_t* buf, uint64_t words, uint64_t n_atomics, void* stream) {
  clear_error();
  if (!buf || words == 0 || (words & (words - 1)) || words > (1ull << 32))
    return set_error(SI_ERR_ARG, "si_probe_l2_atomics: words must be a power of two <= 2^32");
  const int grid = sm_count() * 8;
  l2_atomic_kernel<<<grid, 256, 0, as_stream(stream)>>>(buf, (uint32_t)(words - 1), n_atomics, 0x85EBCA6Bu);
  return check_launch("si_probe_l2_atomics");
}
