// Outlier removal ("clean") and hole filling ("fill") of label volumes on
// the device, after biomedisa/features/remove_outlier.py:67-141. Both rest on
// 6-connected component labelling by union-find over voxel indices:
//   * a row pass gives every voxel of the region the first voxel of its x-run
//     (maximal run of same-class voxels along x) as parent, so x-neighbours
//     are joined without atomics;
//   * a merge pass joins each voxel with its -y and -z neighbours of the same
//     class, skipping pairs already joined through the left neighbour (v-1,
//     v-1-dy and v-dy all in the class); roots are hung under the smaller root
//     with atomicMin, so a parent index never increases and every parent
//     chain strictly decreases (find and merge loops end after at most
//     `index` iterations);
//   * a compress pass points every run start at its root, the smallest voxel
//     index of its component (= the component's first voxel in C order, which
//     is the order in which scipy.ndimage.label numbers components), then
//     every other voxel at its run start's root, counting component sizes
//     with one atomic per distinct root per warp.
// Scratch: int32 parent[V], uint32 size[V], a small info block.
#include <climits>
#include <cstdint>

#include "si_internal.h"

namespace si {
namespace {

struct CcInfo {
  int zmin, zmax, ymin, ymax, xmin, xmax;
  unsigned count;  // voxels of the label
  unsigned maxc;   // largest component of the complement
  int best;        // its first voxel (smallest root among the largest)
  int pad[7];
};

__device__ __forceinline__ int uf_find(const int* L, int p) {
  const volatile int* vl = L;
  int q = vl[p];
  while (q != p) {
    p = q;
    q = vl[p];
  }
  return p;
}

// find with path halving: each visited node is re-pointed at its grandparent
// (an ancestor, so atomicMin keeps parents monotone and links intact)
__device__ __forceinline__ int uf_find_halve(int* L, int p) {
  const volatile int* vl = L;
  while (true) {
    const int q = vl[p];
    if (q == p) return p;
    const int r = vl[q];
    if (r == q) return q;
    atomicMin(&L[p], r);
    p = r;
  }
}

// adds 1 to size[r] for every active lane, one atomic per distinct r in the warp
__device__ __forceinline__ void count_root(unsigned* size, int r, bool active) {
  const unsigned act = __ballot_sync(0xffffffffu, active);
  if (!active) return;
  const unsigned same = __match_any_sync(act, r);
  if ((threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(&size[r], (unsigned)__popc(same));
}

__device__ __forceinline__ void uf_merge(int* L, int a, int b) {
  while (true) {
    a = uf_find_halve(L, a);
    b = uf_find_halve(L, b);
    if (a == b) return;
    if (a < b) {
      const int t = a;
      a = b;
      b = t;
    }
    const int old = atomicMin(&L[a], b);  // hang root a under b
    if (old == a) return;
    a = old;  // a stopped being a root meanwhile: join its new parent with b
  }
}

inline int grid_for(int64_t n) {
  const int64_t want = (n + 255) / 256, cap = (int64_t)sm_count() * 16;
  return (int)(want < cap ? (want > 0 ? want : 1) : cap);
}

// ---- clean: components of all labels at once (same-label connectivity) ----
// one thread per x-row: parent = first voxel of the voxel's x-run
__global__ void clean_rows_kernel(const uint8_t* __restrict__ lab, int64_t rows, int X, int skip, int* __restrict__ L,
                                  unsigned* __restrict__ size) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t base = r * X;
    int start = -1, prev = -1;
    for (int x = 0; x < X; ++x) {
      const int64_t v = base + x;
      const int c = lab[v];
      if (c == skip) {
        L[v] = -1;
        start = -1;
      } else {
        if (start < 0 || c != prev) start = (int)v;
        L[v] = start;
      }
      prev = c;
      size[v] = 0u;
    }
  }
}

__global__ void clean_merge_kernel(const uint8_t* __restrict__ lab, int Z, int Y, int X, int* L) {
  const int64_t V = (int64_t)Z * Y * X, P = (int64_t)X * Y;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    if (L[v] < 0) continue;
    const uint8_t c = lab[v];
    const int x = (int)(v % X);
    const int64_t t = v / X;
    const int y = (int)(t % Y), z = (int)(t / Y);
    const bool left = x > 0 && lab[v - 1] == c;
    if (y > 0 && lab[v - X] == c && !(left && lab[v - 1 - X] == c)) uf_merge(L, (int)v, (int)(v - X));
    if (z > 0 && lab[v - P] == c && !(left && lab[v - 1 - P] == c)) uf_merge(L, (int)v, (int)(v - P));
  }
}

// run starts (x = 0 or left neighbour of another class) take their root
__global__ void clean_compress_starts_kernel(const uint8_t* __restrict__ lab, int X, int64_t V, int* L) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    if (L[v] < 0) continue;
    if (v % X != 0 && lab[v - 1] == lab[v]) continue;
    L[v] = uf_find(L, (int)v);
  }
}

// every other voxel: parent = its run start, whose parent is now the root
__global__ void clean_compress_rest_kernel(int64_t V, int* L, unsigned* __restrict__ size) {
  // whole warps iterate together so that count_root can use warp votes
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t n = (V + 31) / 32 * 32;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
    int r = -1;
    if (v < V) {
      r = L[v];
      if (r >= 0 && r != (int)v) r = L[r];
      if (v < V && r >= 0) L[v] = r;
    }
    count_root(size, r, r >= 0);
  }
}

__global__ void clean_max_kernel(const uint8_t* __restrict__ lab, const int* __restrict__ L,
                                 const unsigned* __restrict__ size, int64_t V, unsigned* __restrict__ big) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x)
    if (L[v] == (int)v) atomicMax(&big[lab[v]], size[v]);
}

// remove_outlier.py:85-97: keep components with size > threshold * largest
__global__ void clean_write_kernel(const uint8_t* __restrict__ lab, const int* __restrict__ L,
                                   const unsigned* __restrict__ size, const unsigned* __restrict__ big, int64_t V,
                                   double threshold, uint8_t* __restrict__ out) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    const uint8_t c = lab[v];
    const int r = L[v];
    out[v] = (r < 0 || (double)size[r] > threshold * (double)big[c]) ? c : (uint8_t)0;
  }
}

// ---- fill: one label at a time inside its grown bounding box ----
__global__ void fill_info_init_kernel(CcInfo* info) {
  info->zmin = info->ymin = info->xmin = INT_MAX;
  info->zmax = info->ymax = info->xmax = -1;
  info->count = 0u;
  info->maxc = 0u;
  info->best = INT_MAX;
}

__global__ void fill_bbox_kernel(const uint8_t* __restrict__ img, int Z, int Y, int X, int k, CcInfo* info) {
  const int64_t V = (int64_t)Z * Y * X;
  int zmn = INT_MAX, zmx = -1, ymn = INT_MAX, ymx = -1, xmn = INT_MAX, xmx = -1;
  unsigned cnt = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
    if (img[v] != k) continue;
    const int x = (int)(v % X);
    const int64_t t = v / X;
    const int y = (int)(t % Y), z = (int)(t / Y);
    zmn = min(zmn, z);
    zmx = max(zmx, z);
    ymn = min(ymn, y);
    ymx = max(ymx, y);
    xmn = min(xmn, x);
    xmx = max(xmx, x);
    ++cnt;
  }
  for (int o = 16; o; o >>= 1) {
    zmn = min(zmn, __shfl_xor_sync(0xffffffffu, zmn, o));
    zmx = max(zmx, __shfl_xor_sync(0xffffffffu, zmx, o));
    ymn = min(ymn, __shfl_xor_sync(0xffffffffu, ymn, o));
    ymx = max(ymx, __shfl_xor_sync(0xffffffffu, ymx, o));
    xmn = min(xmn, __shfl_xor_sync(0xffffffffu, xmn, o));
    xmx = max(xmx, __shfl_xor_sync(0xffffffffu, xmx, o));
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  }
  if ((threadIdx.x & 31) == 0 && cnt) {
    atomicMin(&info->zmin, zmn);
    atomicMax(&info->zmax, zmx);
    atomicMin(&info->ymin, ymn);
    atomicMax(&info->ymax, ymx);
    atomicMin(&info->xmin, xmn);
    atomicMax(&info->xmax, xmx);
    atomicAdd(&info->count, cnt);
  }
}

// The bounding box grown by one voxel and clamped (remove_outlier.py:57-63).
struct Box {
  int z0, y0, x0, nz, ny, nx;
  int64_t n;
};

__device__ __forceinline__ Box box_of(const CcInfo* info, int Z, int Y, int X) {
  Box b;
  if (info->count == 0u) {
    b.n = 0;
    b.z0 = b.y0 = b.x0 = b.nz = b.ny = b.nx = 0;
    return b;
  }
  b.z0 = max(info->zmin - 1, 0);
  b.y0 = max(info->ymin - 1, 0);
  b.x0 = max(info->xmin - 1, 0);
  b.nz = min(info->zmax + 1, Z - 1) + 1 - b.z0;
  b.ny = min(info->ymax + 1, Y - 1) + 1 - b.y0;
  b.nx = min(info->xmax + 1, X - 1) + 1 - b.x0;
  b.n = (int64_t)b.nz * b.ny * b.nx;
  return b;
}

// i-th voxel of the box (C order) -> volume index and box coordinates
__device__ __forceinline__ int64_t box_voxel(const Box& b, int Y, int X, int64_t i, int& bz, int& by, int& bx) {
  bx = (int)(i % b.nx);
  const int64_t t = i / b.nx;
  by = (int)(t % b.ny);
  bz = (int)(t / b.ny);
  return ((int64_t)(b.z0 + bz) * Y + (b.y0 + by)) * X + (b.x0 + bx);
}

// one thread per x-row of the box: parent = first voxel of the x-run of the
// complement of label k (runs end at the box face)
__global__ void fill_rows_kernel(const uint8_t* __restrict__ img, int Z, int Y, int X, int k,
                                 const CcInfo* __restrict__ info, int* __restrict__ L,
                                 unsigned* __restrict__ size) {
  const Box b = box_of(info, Z, Y, X);
  const int64_t rows = (int64_t)b.nz * b.ny;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
    const int by = (int)(r % b.ny), bz = (int)(r / b.ny);
    const int64_t base = ((int64_t)(b.z0 + bz) * Y + (b.y0 + by)) * X + b.x0;
    int start = -1;
    for (int x = 0; x < b.nx; ++x) {
      const int64_t v = base + x;
      if (img[v] == k) {
        L[v] = -1;
        start = -1;
      } else {
        if (start < 0) start = (int)v;
        L[v] = start;
      }
      size[v] = 0u;
    }
  }
}

// complement of label k, connectivity confined to the box
__global__ void fill_merge_kernel(const uint8_t* __restrict__ img, int Z, int Y, int X, int k,
                                  const CcInfo* __restrict__ info, int* L) {
  const Box b = box_of(info, Z, Y, X);
  const int64_t P = (int64_t)X * Y;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n; i += (int64_t)gridDim.x * blockDim.x) {
    int bz, by, bx;
    const int64_t v = box_voxel(b, Y, X, i, bz, by, bx);
    if (img[v] == k) continue;
    const bool left = bx > 0 && img[v - 1] != k;
    if (by > 0 && img[v - X] != k && !(left && img[v - 1 - X] != k)) uf_merge(L, (int)v, (int)(v - X));
    if (bz > 0 && img[v - P] != k && !(left && img[v - 1 - P] != k)) uf_merge(L, (int)v, (int)(v - P));
  }
}

__global__ void fill_compress_starts_kernel(const uint8_t* __restrict__ img, int Z, int Y, int X, int k,
                                            const CcInfo* __restrict__ info, int* L) {
  const Box b = box_of(info, Z, Y, X);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n; i += (int64_t)gridDim.x * blockDim.x) {
    int bz, by, bx;
    const int64_t v = box_voxel(b, Y, X, i, bz, by, bx);
    if (L[v] < 0) continue;
    if (bx > 0 && img[v - 1] != k) continue;
    L[v] = uf_find(L, (int)v);
  }
}

__global__ void fill_compress_rest_kernel(int Z, int Y, int X, const CcInfo* __restrict__ info, int* L,
                                          unsigned* __restrict__ size) {
  const Box b = box_of(info, Z, Y, X);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t n = (b.n + 31) / 32 * 32;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    int r = -1;
    if (i < b.n) {
      int bz, by, bx;
      const int64_t v = box_voxel(b, Y, X, i, bz, by, bx);
      r = L[v];
      if (r >= 0 && r != (int)v) r = L[r];
      if (r >= 0) L[v] = r;
    }
    count_root(size, r, r >= 0);
  }
}

__global__ void fill_max_kernel(int Z, int Y, int X, CcInfo* info, const int* __restrict__ L,
                                const unsigned* __restrict__ size) {
  const Box b = box_of(info, Z, Y, X);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n; i += (int64_t)gridDim.x * blockDim.x) {
    int bz, by, bx;
    const int64_t v = box_voxel(b, Y, X, i, bz, by, bx);
    if (L[v] == (int)v) atomicMax(&info->maxc, size[v]);
  }
}

__global__ void fill_best_kernel(int Z, int Y, int X, CcInfo* info, const int* __restrict__ L,
                                 const unsigned* __restrict__ size) {
  const Box b = box_of(info, Z, Y, X);
  const unsigned maxc = info->maxc;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n; i += (int64_t)gridDim.x * blockDim.x) {
    int bz, by, bx;
    const int64_t v = box_voxel(b, Y, X, i, bz, by, bx);
    if (L[v] == (int)v && size[v] == maxc) atomicMin(&info->best, (int)v);
  }
}

// remove_outlier.py:124-141. The largest entry of [label size, component
// sizes in first-voxel order] (first maximum) stays as it is, components
// larger than threshold * label size stay, the rest of the box becomes k; if
// the label itself is the largest entry its own voxels become 0.
__global__ void fill_write_kernel(uint8_t* img, int Z, int Y, int X, int k, const CcInfo* __restrict__ info,
                                  const int* __restrict__ L, const unsigned* __restrict__ size,
                                  double threshold) {
  const Box b = box_of(info, Z, Y, X);
  const unsigned count = info->count;
  const bool label_biggest = count >= info->maxc;
  const int best = info->best;
  const double limit = threshold * (double)count;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n; i += (int64_t)gridDim.x * blockDim.x) {
    int bz, by, bx;
    const int64_t v = box_voxel(b, Y, X, i, bz, by, bx);
    const int r = L[v];
    if (r < 0) {
      if (label_biggest) img[v] = 0;
      continue;
    }
    const bool keep = (!label_biggest && r == best) || (double)size[r] > limit;
    if (!keep) img[v] = (uint8_t)k;
  }
}

}  // namespace
}  // namespace si

using namespace si;

static uint64_t cc_scratch_need(int64_t V) { return (uint64_t)V * 8 + 256 * sizeof(unsigned) + 256; }

extern "C" int si_cc_scratch_bytes(int Z, int Y, int X, uint64_t* bytes) {
  clear_error();
  if (!bytes || Z < 1 || Y < 1 || X < 1) return set_error(SI_ERR_ARG, "si_cc_scratch_bytes: bad arguments");
  *bytes = cc_scratch_need((int64_t)Z * Y * X);
  return 0;
}

static int cc_check(const char* who, const void* a, int Z, int Y, int X, void* scratch, uint64_t scratch_bytes) {
  if (!a || !scratch) return set_error(SI_ERR_ARG, "%s: null pointer", who);
  if (Z < 1 || Y < 1 || X < 1) return set_error(SI_ERR_ARG, "%s: bad shape", who);
  const int64_t V = (int64_t)Z * Y * X;
  if (V > 0x7fffffffLL) return set_error(SI_ERR_ARG, "%s: more than 2^31 - 1 voxels", who);
  if (scratch_bytes < cc_scratch_need(V) || (uintptr_t)scratch % 16)
    return set_error(SI_ERR_ARG, "%s: scratch too small or misaligned", who);
  return 0;
}

extern "C" int si_clean(const uint8_t* labels, uint8_t* out, int Z, int Y, int X, double threshold, int skip_label,
                        void* scratch, uint64_t scratch_bytes, void* stream) {
  clear_error();
  if (int rc = cc_check("si_clean", labels, Z, Y, X, scratch, scratch_bytes)) return rc;
  if (!out) return set_error(SI_ERR_ARG, "si_clean: null output");
  const int64_t V = (int64_t)Z * Y * X;
  int* L = static_cast<int*>(scratch);
  unsigned* size = reinterpret_cast<unsigned*>(L + V);
  unsigned* big = size + V;
  cudaStream_t st = as_stream(stream);
  const int g = grid_for(V);
  if (cudaMemsetAsync(big, 0, 256 * sizeof(unsigned), st) != cudaSuccess)
    return set_error(SI_ERR_CUDA, "si_clean: memset failed");
  clean_rows_kernel<<<grid_for((int64_t)Z * Y), 128, 0, st>>>(labels, (int64_t)Z * Y, X, skip_label, L, size);
  clean_merge_kernel<<<g, 256, 0, st>>>(labels, Z, Y, X, L);
  clean_compress_starts_kernel<<<g, 256, 0, st>>>(labels, X, V, L);
  clean_compress_rest_kernel<<<g, 256, 0, st>>>(V, L, size);
  clean_max_kernel<<<g, 256, 0, st>>>(labels, L, size, V, big);
  clean_write_kernel<<<g, 256, 0, st>>>(labels, L, size, big, V, threshold, out);
  return check_launch("si_clean");
}

extern "C" int si_fill(uint8_t* img, int Z, int Y, int X, double threshold, const int* label_list, int n_labels,
                       void* scratch, uint64_t scratch_bytes, void* stream) {
  clear_error();
  if (int rc = cc_check("si_fill", img, Z, Y, X, scratch, scratch_bytes)) return rc;
  if (n_labels < 0 || (n_labels > 0 && !label_list)) return set_error(SI_ERR_ARG, "si_fill: bad label list");
  const int64_t V = (int64_t)Z * Y * X;
  int* L = static_cast<int*>(scratch);
  unsigned* size = reinterpret_cast<unsigned*>(L + V);
  CcInfo* info = reinterpret_cast<CcInfo*>(reinterpret_cast<uint8_t*>(size + V) + 256 * sizeof(unsigned));
  cudaStream_t st = as_stream(stream);
  const int g = grid_for(V);
  for (int i = 0; i < n_labels; ++i) {
    const int k = label_list[i];
    if (k < 0 || k > 255) return set_error(SI_ERR_ARG, "si_fill: label %d outside 0..255", k);
    fill_info_init_kernel<<<1, 1, 0, st>>>(info);
    fill_bbox_kernel<<<g, 256, 0, st>>>(img, Z, Y, X, k, info);
    fill_rows_kernel<<<grid_for((int64_t)Z * Y), 128, 0, st>>>(img, Z, Y, X, k, info, L, size);
    fill_merge_kernel<<<g, 256, 0, st>>>(img, Z, Y, X, k, info, L);
    fill_compress_starts_kernel<<<g, 256, 0, st>>>(img, Z, Y, X, k, info, L);
    fill_compress_rest_kernel<<<g, 256, 0, st>>>(Z, Y, X, info, L, size);
    fill_max_kernel<<<g, 256, 0, st>>>(Z, Y, X, info, L, size);
    fill_best_kernel<<<g, 256, 0, st>>>(Z, Y, X, info, L, size);
    fill_write_kernel<<<g, 256, 0, st>>>(img, Z, Y, X, k, info, L, size, threshold);
  }
  return check_launch("si_fill");
}
