// Seed extraction: turns the labelled slices of the label volume into a
// compact, deterministically ordered list of walker start voxels.
//
// A seed is every voxel of a labelled slice that lies in the interior of the
// working volume and whose pre-processed label has a slot (negative labels are
// ignored regions). Its weight constant comes from the variance of (B - I)
// over the same-label pixels of its 3x3 in-slice window, clamped to >= 1
// (biomedisa/features/random_walk/pycuda_small.py:114-131 and :168-171; the
// all-axis variant pycuda_small_allx.py:86-105 uses the slice's own rows and
// columns). Accumulation order: window rows outer, columns inner, binary32.
#include "si_common.cuh"
#include "si_internal.h"

namespace si {
namespace {

struct SeedGeom {
  int Z0, Y0, X0;
  int cz0, cy0, cx0;
  int Zc, Yc, Xc;
  int max_rows;
  // per axis, the box [r0, r1) x [c0, c1) of the slice plane (rows, columns);
  // labels outside it read as ignored (-1)
  int box[3][4];
};

__device__ __forceinline__ int rows_of(const SeedGeom& g, int axis) { return axis == 0 ? g.Yc : g.Zc; }
__device__ __forceinline__ int cols_of(const SeedGeom& g, int axis) { return axis == 2 ? g.Yc : g.Xc; }

// (slice s, row r, column c) of an axis -> crop coordinates.
__device__ __forceinline__ void to_crop(int axis, int s, int r, int c, int& z, int& y, int& x) {
  if (axis == 0) {
    z = s; y = r; x = c;
  } else if (axis == 1) {
    z = r; y = s; x = c;
  } else {
    z = r; y = c; x = s;
  }
}

template <typename T>
struct SlotView {
  const T* lab;
  const int16_t* slot_lut;  // shared copy, 256 entries
  SeedGeom g;
  // label slot at crop coordinates (z, y, x) = (row r, column c) of a slice
  // of `axis`; -1 = no slot (negative label, or outside the axis' box).
  __device__ __forceinline__ int slot(int axis, int r, int c, int z, int y, int x) const {
    const int* b = g.box[axis];
    if (r < b[0] || r >= b[1] || c < b[2] || c >= b[3]) return -1;
    const int oz = z + g.cz0 - 1, oy = y + g.cy0 - 1, ox = x + g.cx0 - 1;
    int v = 0;  // pad voxels carry label 0
    if ((unsigned)oz < (unsigned)g.Z0 && (unsigned)oy < (unsigned)g.Y0 && (unsigned)ox < (unsigned)g.X0)
      v = static_cast<int>(lab[((uint64_t)oz * g.Y0 + oy) * g.X0 + ox]);
    if (v < 0) return -1;
    if (v > 255) v = 0;  // pre-processing sets labels > 255 to 0
    return slot_lut[v];
  }
};

__device__ __forceinline__ bool interior(const SeedGeom& g, int z, int y, int x) {
  return z > 0 && y > 0 && x > 0 && z < g.Zc - 1 && y < g.Yc - 1 && x < g.Xc - 1;
}

template <typename T>
__device__ __forceinline__ bool is_seed(const SlotView<T>& sv, int axis, int s, int r, int c, int& slot) {
  int z, y, x;
  to_crop(axis, s, r, c, z, y, x);
  if (!interior(sv.g, z, y, x)) return false;
  slot = sv.slot(axis, r, c, z, y, x);
  return slot >= 0;
}

// Pass 1: seeds per (slice entry, row).
template <typename T>
__global__ void __launch_bounds__(128) seed_count_kernel(const T* __restrict__ lab, SeedGeom g,
                                                         const int16_t* __restrict__ slot_lut_g,
                                                         const int32_t* __restrict__ slice_list,
                                                         uint32_t* __restrict__ row_counts) {
  __shared__ int16_t lut[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = slot_lut_g[i];
  __syncthreads();
  const int e = blockIdx.y;
  const int r = blockIdx.x;
  const int axis = slice_list[2 * e];
  const int s = slice_list[2 * e + 1];
  uint32_t cnt = 0;
  if (r < rows_of(g, axis)) {
    SlotView<T> sv{lab, lut, g};
    const int C = cols_of(g, axis);
    for (int c = threadIdx.x; c < C; c += blockDim.x) {
      int slot;
      cnt += is_seed(sv, axis, s, r, c, slot) ? 1u : 0u;
    }
  }
  __shared__ uint32_t warp_sum[4];
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += warp_sum[w];
    row_counts[(size_t)e * g.max_rows + r] = t;
  }
}

// Exclusive scan of n counts in place (one CTA of 1024 threads); writes the
// total to counts[n] and *n_seeds.
__global__ void __launch_bounds__(1024) scan_kernel(uint32_t* __restrict__ counts, uint32_t n,
                                                    uint32_t* __restrict__ n_seeds) {
  __shared__ uint32_t part[1024];
  const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
  const uint32_t beg = threadIdx.x * per;
  const uint32_t end = min(beg + per, n);
  uint32_t sum = 0;
  for (uint32_t i = beg; i < end; ++i) sum += counts[i];
  part[threadIdx.x] = sum;
  __syncthreads();
  // Hillis-Steele inclusive scan over the 1024 partial sums
  for (int off = 1; off < 1024; off <<= 1) {
    const uint32_t v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
  for (uint32_t i = beg; i < end; ++i) {
    const uint32_t c = counts[i];
    counts[i] = run;
    run += c;
  }
  if (threadIdx.x == blockDim.x - 1) {
    counts[n] = part[blockDim.x - 1];
    *n_seeds = part[blockDim.x - 1];
  }
}

// Pass 2: write the seeds of one (slice entry, row) at its scanned offset.
template <typename T, bool kFloat>
__global__ void __launch_bounds__(128) seed_emit_kernel(const T* __restrict__ lab, SeedGeom g,
                                                        const int16_t* __restrict__ slot_lut_g,
                                                        const uint8_t* __restrict__ slot_label_g,
                                                        const void* __restrict__ work,
                                                        const int32_t* __restrict__ slice_list,
                                                        const uint32_t* __restrict__ offsets,
                                                        SeedRec* __restrict__ seeds) {
  __shared__ int16_t lut[256];
  __shared__ uint8_t lab_of[256];
  __shared__ uint32_t warp_cnt[4];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    lut[i] = slot_lut_g[i];
    lab_of[i] = slot_label_g[i];
  }
  __syncthreads();
  const int e = blockIdx.y;
  const int r = blockIdx.x;
  const int axis = slice_list[2 * e];
  const int s = slice_list[2 * e + 1];
  if (r >= rows_of(g, axis)) return;  // uniform across the block
  SlotView<T> sv{lab, lut, g};
  const int C = cols_of(g, axis);
  uint32_t base = offsets[(size_t)e * g.max_rows + r];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const size_t F = (size_t)g.Yc * g.Xc;
  for (int c0 = 0; c0 < C; c0 += blockDim.x) {
    const int c = c0 + threadIdx.x;
    int slot = -1;
    const bool pred = c < C && is_seed(sv, axis, s, r, c, slot);
    const uint32_t ballot = __ballot_sync(0xffffffffu, pred);
    if (lane == 0) warp_cnt[wid] = __popc(ballot);
    __syncthreads();
    uint32_t before = 0, chunk = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      if (w < wid) before += warp_cnt[w];
      chunk += warp_cnt[w];
    }
    before += __popc(ballot & ((1u << lane) - 1u));
    if (pred) {
      int z, y, x;
      to_crop(axis, s, r, c, z, y, x);
      const size_t pos = (size_t)z * F + (size_t)y * g.Xc + x;
      float b, dev = 0.0f, summe = 0.0f;
      if (kFloat) {
        const float* img = static_cast<const float*>(work);
        b = img[pos];
        for (int n = -1; n <= 1; ++n)
          for (int o = -1; o <= 1; ++o) {
            int zz, yy, xx;
            to_crop(axis, s, r + n, c + o, zz, yy, xx);
            if (sv.slot(axis, r + n, c + o, zz, yy, xx) == slot) {
              const float tmp = __fsub_rn(b, img[(size_t)zz * F + (size_t)yy * g.Xc + xx]);
              dev = __fadd_rn(dev, __fmul_rn(tmp, tmp));
              summe = __fadd_rn(summe, 1.0f);
            }
          }
      } else {
        const uint8_t* img = static_cast<const uint8_t*>(work);
        const int bi = img[pos];
        b = (float)bi;
        for (int n = -1; n <= 1; ++n)
          for (int o = -1; o <= 1; ++o) {
            int zz, yy, xx;
            to_crop(axis, s, r + n, c + o, zz, yy, xx);
            if (sv.slot(axis, r + n, c + o, zz, yy, xx) == slot) {
              const int d = bi - (int)img[(size_t)zz * F + (size_t)yy * g.Xc + xx];
              dev = __fadd_rn(dev, (float)(d * d));
              summe = __fadd_rn(summe, 1.0f);
            }
          }
      }
      float var = __fdiv_rn(dev, summe);
      if (var < 1.0f) var = 1.0f;
      SeedRec rec;
      rec.pos = (uint32_t)pos;
      rec.c = weight_constant(var);
      rec.b = b;
      rec.meta = (uint32_t)slot | ((uint32_t)axis << 8) | ((uint32_t)lab_of[slot] << 16);
      seeds[base + before] = rec;
    }
    base += chunk;
    __syncthreads();
  }
}

}  // namespace
}  // namespace si

using namespace si;

static int extract_seeds_impl(const void* labels, int dtype, int Z0, int Y0, int X0, int cz0, int cy0, int cx0,
                              int Zc, int Yc, int Xc, const int16_t* slot_lut, const uint8_t* slot_label,
                              const void* work, int work_is_float, const int32_t* slice_list, int n_slices,
                              uint32_t* row_counts, si_seed_t* seeds, uint32_t* n_seeds, const int32_t* boxes,
                              void* stream) {
  if (!labels || !slot_lut || !slot_label || !work || !row_counts || !seeds || !n_seeds)
    return set_error(SI_ERR_ARG, "si_extract_seeds: null pointer");
  if (n_slices < 0 || (n_slices > 0 && !slice_list)) return set_error(SI_ERR_ARG, "si_extract_seeds: bad slice list");
  if (Zc < 3 || Yc < 3 || Xc < 3) return set_error(SI_ERR_ARG, "si_extract_seeds: bad crop dims");
  if ((uint64_t)Zc * Yc * Xc > 0xFFFFFFFFull)
    return set_error(SI_ERR_LIMIT, "si_extract_seeds: working volume above 2^32 voxels");
  if (n_slices > 65535) return set_error(SI_ERR_LIMIT, "si_extract_seeds: more than 65535 slices");
  cudaStream_t st = as_stream(stream);
  if (n_slices == 0) {
    if (cudaMemsetAsync(n_seeds, 0, sizeof(uint32_t), st) != cudaSuccess)
      return set_error(SI_ERR_CUDA, "si_extract_seeds: memset failed");
    return SI_OK;
  }
  SeedGeom g{Z0, Y0, X0, cz0, cy0, cx0, Zc, Yc, Xc, Zc > Yc ? Zc : Yc, {}};
  for (int a = 0; a < 3; ++a) {
    const int R = a == 0 ? Yc : Zc, C = a == 2 ? Yc : Xc;
    for (int k = 0; k < 4; ++k) g.box[a][k] = boxes ? boxes[4 * a + k] : (k == 1 ? R : k == 3 ? C : 0);
  }
  const dim3 grid(g.max_rows, n_slices);
  const uint32_t n = (uint32_t)((size_t)n_slices * g.max_rows);
  SeedRec* out = reinterpret_cast<SeedRec*>(seeds);
#define SI_SEEDS_FOR(T)                                                                                         \
  do {                                                                                                          \
    const T* lab = static_cast<const T*>(labels);                                                               \
    seed_count_kernel<T><<<grid, 128, 0, st>>>(lab, g, slot_lut, slice_list, row_counts);                       \
    scan_kernel<<<1, 1024, 0, st>>>(row_counts, n, n_seeds);                                                    \
    if (work_is_float)                                                                                          \
      seed_emit_kernel<T, true><<<grid, 128, 0, st>>>(lab, g, slot_lut, slot_label, work, slice_list,           \
                                                      row_counts, out);                                         \
    else                                                                                                        \
      seed_emit_kernel<T, false><<<grid, 128, 0, st>>>(lab, g, slot_lut, slot_label, work, slice_list,          \
                                                       row_counts, out);                                        \
  } while (0)
  switch (dtype) {
    case SI_U8:
      SI_SEEDS_FOR(uint8_t);
      break;
    case SI_I16:
      SI_SEEDS_FOR(int16_t);
      break;
    case SI_I32:
      SI_SEEDS_FOR(int32_t);
      break;
    default:
      return set_error(SI_ERR_ARG, "si_extract_seeds: unsupported label dtype %d", dtype);
  }
#undef SI_SEEDS_FOR
  return check_launch("si_extract_seeds");
}

extern "C" int si_extract_seeds(const void* labels, int dtype, int Z0, int Y0, int X0, int cz0, int cy0, int cx0,
                                int Zc, int Yc, int Xc, const int16_t* slot_lut, const uint8_t* slot_label,
                                const void* work, int work_is_float, const int32_t* slice_list, int n_slices,
                                uint32_t* row_counts, si_seed_t* seeds, uint32_t* n_seeds, void* stream) {
  clear_error();
  return extract_seeds_impl(labels, dtype, Z0, Y0, X0, cz0, cy0, cx0, Zc, Yc, Xc, slot_lut, slot_label, work,
                            work_is_float, slice_list, n_slices, row_counts, seeds, n_seeds, nullptr, stream);
}

extern "C" int si_extract_seeds_box(const void* labels, int dtype, int Z0, int Y0, int X0, int cz0, int cy0,
                                    int cx0, int Zc, int Yc, int Xc, const int16_t* slot_lut,
                                    const uint8_t* slot_label, const void* work, int work_is_float,
                                    const int32_t* slice_list, int n_slices, int box_y0, int box_y1, int box_x0,
                                    int box_x1, uint32_t* row_counts, si_seed_t* seeds, uint32_t* n_seeds,
                                    void* stream) {
  clear_error();
  // the box applies to z-slices (rows y, columns x); other axes keep their planes
  const int32_t boxes[12] = {box_y0, box_y1, box_x0, box_x1, 0, Zc, 0, Xc, 0, Zc, 0, Yc};
  return extract_seeds_impl(labels, dtype, Z0, Y0, X0, cz0, cy0, cx0, Zc, Yc, Xc, slot_lut, slot_label, work,
                            work_is_float, slice_list, n_slices, row_counts, seeds, n_seeds, boxes, stream);
}

extern "C" int si_extract_seeds_boxes(const void* labels, int dtype, int Z0, int Y0, int X0, int cz0, int cy0,
                                      int cx0, int Zc, int Yc, int Xc, const int16_t* slot_lut,
                                      const uint8_t* slot_label, const void* work, int work_is_float,
                                      const int32_t* slice_list, int n_slices, const int32_t* boxes,
                                      uint32_t* row_counts, si_seed_t* seeds, uint32_t* n_seeds, void* stream) {
  clear_error();
  if (!boxes) return set_error(SI_ERR_ARG, "si_extract_seeds_boxes: null boxes");
  return extract_seeds_impl(labels, dtype, Z0, Y0, X0, cz0, cy0, cx0, Zc, Yc, Xc, slot_lut, slot_label, work,
                            work_is_float, slice_list, n_slices, row_counts, seeds, n_seeds, boxes, stream);
}

// ---------------------------------------------------------------------------
// Allocation-free seed extraction.
//
// Some callers cannot allocate device memory at the point where they extract
// seeds: a plug-in living inside a host application whose own allocator has
// already claimed the GPU's memory pool, or a pipeline that must not call
// cudaMalloc because it synchronises the whole device. For them this variant
// keeps the per-row counters of the count/scan/emit passes in a fixed array
// that is part of the loaded library image instead of a caller buffer; the
// caller still provides every input and output.
//
// Limit: n_slices * max(Zc, Yc) + 1 <= kStaticRowCounters (1,048,576 counters,
// 4 MiB, held by every GPU that loads the library until the process exits).
// The first call on a device looks up the array's device address with that
// device current; make that first call before any stream capture. The address
// is remembered together with the device's current CUDA context; when the
// context changes (after cudaDeviceReset, or when the primary context was
// released and created again) the module is loaded anew and the next call looks
// the address up again. All calls share the one array: calls whose work
// overlaps on the GPU (different streams or threads) race on it. The count pass
// writes every counter the scan and emit passes read, so nothing left over from
// an earlier call is ever read.
// ---------------------------------------------------------------------------
#include <cuda.h>

#include <mutex>

namespace {
constexpr unsigned long long kStaticRowCounters = 1ull << 20;
constexpr int kMaxDevices = 64;
std::mutex g_static_rows_mu;
uint32_t* g_static_rows_dev[kMaxDevices] = {};
CUcontext g_static_rows_ctx[kMaxDevices] = {};

using CtxGetCurrentFn = CUresult (*)(CUcontext*);

// The driver's cuCtxGetCurrent through the runtime's entry-point query (the
// library links only the runtime).
CtxGetCurrentFn ctx_get_current_fn() {
  static CtxGetCurrentFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<CtxGetCurrentFn>(p);
  });
  return fn;
}
}  // namespace

static __device__ __align__(256) uint32_t g_static_row_counts[kStaticRowCounters];

// Device address of g_static_row_counts for the current device and context
// (looked up once per context; the host-side name is not a device address).
static int static_row_counts(uint32_t** out) {
  int dev = -1;
  const cudaError_t ge = cudaGetDevice(&dev);
  if (ge != cudaSuccess) return set_error(SI_ERR_CUDA, "si_extract_seeds_noalloc: cudaGetDevice: %s",
                                          cudaGetErrorString(ge));
  if (dev < 0 || dev >= kMaxDevices) return set_error(SI_ERR_LIMIT, "si_extract_seeds_noalloc: device %d", dev);
  const CtxGetCurrentFn get_ctx = ctx_get_current_fn();
  if (!get_ctx) return set_error(SI_ERR_CUDA, "si_extract_seeds_noalloc: cuCtxGetCurrent unavailable");
  CUcontext ctx = nullptr;
  if (get_ctx(&ctx) != CUDA_SUCCESS)
    return set_error(SI_ERR_CUDA, "si_extract_seeds_noalloc: cannot read the current context");
  std::lock_guard<std::mutex> lock(g_static_rows_mu);
  if (!ctx || !g_static_rows_dev[dev] || g_static_rows_ctx[dev] != ctx) {
    // With no context current yet, the lookup itself makes the device's
    // primary context current; the context is read again after it.
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_static_row_counts);
    if (e != cudaSuccess || !p)
      return set_error(SI_ERR_CUDA, "si_extract_seeds_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    if (!ctx && (get_ctx(&ctx) != CUDA_SUCCESS || !ctx))
      return set_error(SI_ERR_CUDA, "si_extract_seeds_noalloc: no current context after the lookup");
    g_static_rows_dev[dev] = static_cast<uint32_t*>(p);
    g_static_rows_ctx[dev] = ctx;
  }
  *out = g_static_rows_dev[dev];
  return SI_OK;
}

extern "C" int si_extract_seeds_noalloc(const void* labels, int dtype, int Z0, int Y0, int X0, int cz0, int cy0,
                                        int cx0, int Zc, int Yc, int Xc, const int16_t* slot_lut,
                                        const uint8_t* slot_label, const void* work, int work_is_float,
                                        const int32_t* slice_list, int n_slices, si_seed_t* seeds,
                                        uint32_t* n_seeds, void* stream) {
  clear_error();
  if (n_slices < 0 || Zc < 0 || Yc < 0) return set_error(SI_ERR_ARG, "si_extract_seeds_noalloc: bad sizes");
  const unsigned long long need = (unsigned long long)n_slices * (unsigned long long)(Zc > Yc ? Zc : Yc) + 1ull;
  if (need > kStaticRowCounters)
    return set_error(SI_ERR_LIMIT,
                     "si_extract_seeds_noalloc: needs %llu row counters (n_slices * max(Zc, Yc) + 1), "
                     "the static scratch holds %llu; use si_extract_seeds with a caller buffer",
                     need, kStaticRowCounters);
  uint32_t* rows = nullptr;
  const int rc = static_row_counts(&rows);
  if (rc != SI_OK) return rc;
  return si_extract_seeds(labels, dtype, Z0, Y0, X0, cz0, cy0, cx0, Zc, Yc, Xc, slot_lut, slot_label, work,
                          work_is_float, slice_list, n_slices, rows, seeds, n_seeds, stream);
}
