/*
 * smartinterp.h — C ABI of the GB300 smart-interpolation library
 * (libsmartinterp.so, built from biomedisa_gb300/csrc).
 *
 * Every entry point takes DEVICE pointers (allocated by the caller), plain
 * sizes and a cudaStream_t passed as void*. Calls are asynchronous on that
 * stream; the return value only reports launch/argument errors:
 *   0 = success, non-zero = error code, message via si_last_error().
 * No entry point allocates memory unless stated.
 *
 * The sequence smart_interpolation() runs is:
 *   si_label_histogram -> (host: label set) -> si_slice_flags -> (host: crop,
 *   slice lists) -> si_image_minmax (non-uint8 input only) -> si_prepare_image
 *   -> si_extract_seeds -> si_pack_neighbours -> si_walk -> si_argmax
 *   -> si_remap_labels
 *   [-> si_smooth -> si_argmax -> si_remap_labels]
 */
#ifndef SMARTINTERP_H
#define SMARTINTERP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Element types of caller-supplied volumes. */
enum si_dtype {
  SI_U8 = 0,
  SI_I8 = 1,
  SI_U16 = 2,
  SI_I16 = 3,
  SI_I32 = 4,
  SI_F32 = 5
};

/* Error codes. */
enum si_status {
  SI_OK = 0,
  SI_ERR_ARG = 1,    /* invalid argument (null pointer, bad size, bad dtype) */
  SI_ERR_CUDA = 2,   /* CUDA launch error */
  SI_ERR_LIMIT = 3   /* size beyond a documented limit */
};

/* One walker start voxel (16 bytes). pos: linear index in the working
 * (cropped, padded) volume; c: per-seed weight constant log2(e)/(2 var);
 * b: seed intensity; meta: bits 0-7 label slot, 8-9 seed axis,
 * 16-23 label value. */
typedef struct {
  uint32_t pos;
  float c;
  float b;
  uint32_t meta;
} si_seed_t;

/* One volume of a batched walk (si_walk_sorted_batch). packed: its packed
 * records (si_pack_neighbours); hits: uint32 [nol][Zc][Yc][Xc], caller-zeroed;
 * seeds / n_seeds / max_seeds: as for si_walk. */
typedef struct {
  const void* packed;
  uint32_t* hits;
  const si_seed_t* seeds;
  const uint32_t* n_seeds;
  uint32_t max_seeds;
  int Zc, Yc, Xc;
  int nol;
  int work_is_float;
} si_volume_t;

/* Library version (major*10000 + minor*100 + patch). */
int si_version(void);

/* Message of the last error raised by this thread ("" if none). */
const char* si_last_error(void);

/* Histogram of label values. hist[0..255] counts values 0..255, hist[256]
 * counts negative values, hist[257] values > 255. hist must be zeroed by the
 * caller. Replaces the label-set scan of pre_processing
 * (biomedisa/features/biomedisa_helper.py:671 `unique(bm.labelData)`,
 * :82-103). dtype: SI_U8, SI_I16 or SI_I32. */
int si_label_histogram(const void* labels, int dtype, uint64_t n,
                       unsigned long long* hist, void* stream);

/* Labelled-slice flags and bounding box of nonzero labels on the zero-padded
 * frame (dims Z0+2, Y0+2, X0+2) without materialising the pad.
 * nz_lut[v] (v = 0..255) is 1 iff value v is nonzero after pre-processing;
 * negative values count as nonzero, values > 255 as zero.
 * allaxis = 0: flags_z[k] = 1 iff padded z-slice k holds a nonzero label
 *   (biomedisa_helper.py:1015-1022 read_labeled_slices).
 * allaxis = 1: flags_{z,y,x}[k] = 1 iff slice k of that axis keeps a nonzero
 *   pixel after removing one-pixel-wide lines (the gradient test of
 *   read_indices_allx / read_labeled_slices_allx, biomedisa_helper.py:1024-1066).
 * allaxis = 2: as 1 with negative values counting as zero, for flags and
 *   bbox (the large path's reader read_labeled_slices_allx_large,
 *   biomedisa_helper.py:1082-1099, tests labels > 0).
 * bbox[6] = (zmin, zmax, ymin, ymax, xmin, xmax) in padded coordinates; the
 * caller initialises it to (INT_MAX, -1, INT_MAX, -1, INT_MAX, -1)
 * (predict_blocksize before the +-100 margin, biomedisa_helper.py:1105-1116).
 * flags arrays are zeroed by the caller; flags_y/flags_x may be NULL when
 * allaxis = 0. */
int si_slice_flags(const void* labels, int dtype, int Z0, int Y0, int X0,
                   const uint8_t* nz_lut, int allaxis, uint8_t* flags_z,
                   uint8_t* flags_y, uint8_t* flags_x, int32_t* bbox,
                   void* stream);

/* mm[0] = min, mm[1] = max of an image converted to float32 (used for the
 * [0,255] normalisation of non-uint8 input, biomedisa/interpolation.py:140-144).
 * The caller initialises mm to (+inf, -inf). dtype: SI_U16, SI_I16, SI_F32. */
int si_image_minmax(const void* img, int dtype, uint64_t n, float* mm,
                    void* stream);

/* Working image: the crop [cz0,cz0+Zc) x [cy0,..) x [cx0,..) of the image
 * padded by one zero voxel on every side (biomedisa/interpolation.py:157 and
 * :203), after the reference's dtype normalisation (:136-144) and optional
 * 3x3x3 box denoise (biomedisa_helper.py:308-323).
 * dtype SI_U8 / SI_I8 -> work is uint8 (int8 shifted by +128);
 * other dtypes -> work is float32 ((x - norm_min) / norm_range * 255).
 * Crop coordinates are in the padded frame. */
int si_prepare_image(const void* img, int dtype, int Z0, int Y0, int X0,
                     int cz0, int cy0, int cx0, int Zc, int Yc, int Xc,
                     float norm_min, float norm_range, int denoise,
                     void* work, void* stream);

/* Seed extraction: every interior voxel of the listed slices whose
 * (pre-processed) label has a slot becomes one seed, with its in-slice 3x3
 * same-label variance (pycuda_small.py:114-131; pycuda_small_allx.py:86-105).
 * slice_list holds n_slices pairs (axis, index in crop coordinates).
 * slot_lut[v] = label slot of value v (0..255) or -1; values > 255 use
 * slot_lut[0]; negative values never seed. slot_label[s] = label value of slot s.
 * row_counts: scratch of n_slices * max(Zc, Yc) + 1 uint32.
 * seeds: capacity for every interior pixel of the listed slices.
 * *n_seeds (device) receives the count. Seeds are ordered by
 * (slice_list entry, row, column). Replaces the seed selection inside the
 * walker kernels (pycuda_small.py:140-171) and the slice reader
 * (biomedisa_helper.py:1015-1045). */
int si_extract_seeds(const void* labels, int dtype, int Z0, int Y0, int X0,
                     int cz0, int cy0, int cx0, int Zc, int Yc, int Xc,
                     const int16_t* slot_lut, const uint8_t* slot_label,
                     const void* work, int work_is_float,
                     const int32_t* slice_list, int n_slices,
                     uint32_t* row_counts, si_seed_t* seeds,
                     uint32_t* n_seeds, void* stream);

/* Allocation-free seed extraction. No counterpart in the reference: it serves
 * callers that cannot allocate device memory when they extract seeds (for
 * example a plug-in whose host application owns the GPU's memory pool, or a
 * pipeline that must avoid cudaMalloc's device-wide synchronisation).
 * Same arguments and results as si_extract_seeds without row_counts: the
 * counters live in a static device array of 1,048,576 uint32 (4 MiB per GPU
 * that loads the library, held until exit), so n_slices * max(Zc, Yc) + 1 must
 * not exceed 1,048,576 (SI_ERR_LIMIT otherwise). The first call on a device
 * looks up the array's address with that device current; make it before any
 * stream capture. The address is remembered per device with the context it
 * was looked up in, and looked up again when the device's current context
 * changes (e.g. after cudaDeviceReset). Calls share the array: calls that
 * overlap on the GPU race. Allocates nothing. */
int si_extract_seeds_noalloc(const void* labels, int dtype, int Z0, int Y0,
                             int X0, int cz0, int cy0, int cx0, int Zc,
                             int Yc, int Xc, const int16_t* slot_lut,
                             const uint8_t* slot_label, const void* work,
                             int work_is_float, const int32_t* slice_list,
                             int n_slices, si_seed_t* seeds,
                             uint32_t* n_seeds, void* stream);

/* Packed neighbourhood records for the walker: for every interior voxel of
 * the working volume, its six neighbour intensities in move order
 * (+z, -z, +y, -y, +x, -x), a refusal mask (bit d set when move d would leave
 * [1, dim-2], pycuda_small.py:236) and its own intensity.
 * uint8 work -> 8 bytes per voxel; float32 work -> 32 bytes per voxel.
 * packed: caller buffer of Zc*Yc*Xc records. */
int si_pack_neighbours(const void* work, int work_is_float, int Zc, int Yc,
                       int Xc, void* packed, void* stream);

/* Random walker over packed records (si_pack_neighbours). For every seed,
 * nbrw walks of sorw steps; a move into the interior adds one hit to
 * hits[slot][z][y][x] (uint32, caller-zeroed, nol * Zc*Yc*Xc). Direction
 * weights, border rule and walk reset follow pycuda_small.py:138-257;
 * randomness is Philox4x32-10 keyed by `key` with counter
 * (step/4, seed pos, seed axis, label value).
 * order 0: walk-major work order (all seeds' walk 0 first), 1: seed-major.
 * grid/block <= 0 select defaults. max_seeds bounds *n_seeds.
 * Replaces Funktion/randomWalk and the per-label launch loop
 * (pycuda_small.py:102-108, pyopencl_small.py:128-134). */
int si_walk(const void* packed, int work_is_float, int Zc, int Yc, int Xc,
            const si_seed_t* seeds, const uint32_t* n_seeds,
            uint32_t max_seeds, int nbrw, int sorw, uint64_t key,
            uint32_t* hits, int nol, int grid, int block, int order,
            void* stream);

/* Scratch bytes si_walk_bricks needs for a crop of Zc x Yc x Xc voxels, up
 * to max_walks walks (seeds * nbrw) and nol labels. */
int si_walk_bricks_scratch(int Zc, int Yc, int Xc, uint64_t max_walks, int nol,
                           unsigned long long* bytes);

/* Brick walker: the same walk and the same uint32 hit maps as si_walk, for a
 * uint8 working volume, computed with every step's neighbourhood record and
 * hit counter in shared memory. The crop is cut into 10^3 core bricks; a CTA
 * loads the 16^3 box around a core (TMA tensor copy of packed records) and
 * advances the walkers of one (label, brick) bucket until they leave the box
 * or finish; walkers are re-sorted by bucket every round (counting sort) until
 * none is left. work: uint8 working image (si_prepare_image); scratch: caller
 * buffer of si_walk_bricks_scratch bytes; rounds_out (nullable) receives the
 * number of rounds. nbrw * sorw must be below 2^24. Synchronises `stream`
 * once per round to read the number of live walkers. Replaces the same
 * reference code as si_walk. */
int si_walk_bricks(const void* work, int Zc, int Yc, int Xc,
                   const si_seed_t* seeds, const uint32_t* n_seeds,
                   uint32_t max_seeds, int nbrw, int sorw, uint64_t key,
                   uint32_t* hits, int nol, void* scratch,
                   unsigned long long scratch_bytes, int* rounds_out,
                   void* stream);

/* Scratch bytes si_walk_sorted needs (crop dims, max walks = seeds * nbrw,
 * labels, sort brick edge; sort_edge <= 0 selects the default 6). */
int si_walk_sorted_scratch(int Zc, int Yc, int Xc, uint64_t max_walks, int nol,
                           int sort_edge, unsigned long long* bytes);

/* Sorted-sweep walker: the same walk and the same uint32 hit maps as si_walk
 * over packed records (si_pack_neighbours), run as sweeps in which every live
 * walker advances min(sweep_steps, steps left) steps (default 32 when <= 0);
 * between sweeps the walkers are counting-sorted by (label slot, brick of
 * sort_edge^3 voxels; default 6 when <= 0),
 * so concurrently running walkers share a compact, cache-resident part of
 * the volume and of the hit maps. scratch: si_walk_sorted_scratch bytes;
 * rounds_out (nullable) receives the number of sweeps. nbrw * sorw must be
 * below 2^24. Synchronises `stream` once per sweep. */
int si_walk_sorted(const void* packed, int work_is_float, int Zc, int Yc,
                   int Xc, const si_seed_t* seeds, const uint32_t* n_seeds,
                   uint32_t max_seeds, int nbrw, int sorw, uint64_t key,
                   uint32_t* hits, int nol, int sweep_steps, int sort_edge,
                   void* scratch, unsigned long long scratch_bytes,
                   int* rounds_out, void* stream);

/* Size of si_walk_sorted's seed ranges. The walker takes the seeds (which
 * come in slice order, i.e. as compact slabs) in consecutive ranges of about
 * walks_per_range walks and walks each range to completion; 0 restores the
 * default of 2^25. Process-wide; the hit maps do not depend on it (integer
 * sums of independent walks), only the speed does. No counterpart in the
 * reference (its walker takes all seeds of a label in one launch,
 * pycuda_small.py:102-108); tests use it to split small volumes into many
 * ranges. */
int si_walk_sorted_set_range(unsigned long long walks_per_range);

/* Selects how the sorted walkers' sweep kernels map walkers to threads:
 * 0 = one walker per thread; 1 (default) = two consecutive walkers per
 * thread, advanced together so each thread keeps two record gathers in
 * flight; 2 = three walkers per thread; 3 = four (si_walk_sorted only; the
 * batched walker pairs walkers for every mode but 0). Process-wide; speed
 * only (the hit maps do not depend on it). */
int si_walk_sorted_set_pairs(int pairs);

/* Selects where si_walk_sorted's sweep loop runs: 1 (default) = on the
 * device, as a CUDA graph per seed range whose WHILE node repeats
 * (scatter, sweep, scan) rounds while walkers are live, with no host round
 * trip per sweep; 0 = on the host, reading the live count back after every
 * scan. Process-wide; the hit maps do not depend on it. */
int si_walk_sorted_set_loop(int device_loop);

/* Most sweeps one si_walk_sorted call may run (0 = 2^24, the default); a
 * walk that would need more stops there and the call returns SI_ERR_LIMIT.
 * The device loop checks it after every two sweeps. */
int si_walk_sorted_set_round_limit(unsigned long long sweeps);

/* Walker on the reference's own random stream: the same walk as si_walk
 * (packed records, weights, border rule, one uint32 hit per accepted move)
 * with u drawn from the reference walker's binary32 "MRG32k3a" recurrence
 * (pycuda_small.py:155-165 set-up, :197-225 update), each operation rounded
 * on its own. One thread per seed runs the seed's nbrw walks in sequence, the
 * stream continuing across walks. A seed's stream starts at its index in the
 * reference's slice stack, rank * R * C + r * C + c (pycuda_small.py:145,165):
 * stack_rank[Zc + Yc + Xc] holds, for axis 0 at [0, Zc), axis 1 at
 * [Zc, Zc + Yc) and axis 2 at [Zc + Yc, Zc + Yc + Xc), the rank of each listed
 * slice among the listed slices of its axis (-1 when not listed). Replaces
 * the reference walker kernels with their own randomness (pycuda_small.py:
 * 138-257, pycuda_small_allx.py:186-330). */
int si_walk_refstream(const void* packed, int work_is_float, int Zc, int Yc,
                      int Xc, const si_seed_t* seeds, const uint32_t* n_seeds,
                      uint32_t max_seeds, int nbrw, int sorw,
                      const int32_t* stack_rank, uint32_t* hits, int nol,
                      void* stream);

/* Scratch bytes si_walk_sorted_batch needs for these volumes (host array of
 * n_vols descriptors, at most 256). */
int si_walk_sorted_batch_scratch(const si_volume_t* vols, int n_vols,
                                 int nbrw, int sort_edge,
                                 unsigned long long* bytes);

/* Batched sorted sweeps: the walks of all n_vols volumes (uneven sizes,
 * uint8 or float records, any label counts) advance together in every sweep
 * launch, bucketed by (volume, label slot, brick). Each volume's hit maps
 * equal si_walk_sorted / si_walk on that volume alone (same key). vols is a
 * HOST array; scratch: si_walk_sorted_batch_scratch bytes. Replaces running
 * the reference once per volume. */
int si_walk_sorted_batch(const si_volume_t* vols, int n_vols, int nbrw,
                         int sorw, uint64_t key, int sweep_steps,
                         int sort_edge, void* scratch,
                         unsigned long long scratch_bytes, int* rounds_out,
                         void* stream);

/* Per-voxel argmax over nol maps ([nol][Zc][Yc][Xc], uint32 hits or float32
 * smoothed maps), first maximum wins (np.argmax, rw_small.py:200). The label
 * index is written to out (original frame Z0 x Y0 x X0, uint8, caller-zeroed)
 * at the crop region minus the one-voxel pad (rw_small.py:214-216);
 * presence[8] (caller-zeroed) receives a bit per index seen.
 * uq (nullable, same frame as out) receives the uncertainty
 * uint8(255 * (1 - (1 - m0/m2)(1 - m1/m2))) of the three largest values on the
 * crop interior and 0 on its border (gpu_kernels.py:54-116, rw_small.py:152-176). */
int si_argmax(const void* maps, int maps_are_float, int nol, int Zc, int Yc,
              int Xc, int cz0, int cy0, int cx0, int Z0, int Y0, int X0,
              uint8_t* out, uint32_t* presence, uint8_t* uq, void* stream);

/* Replace label indices in out (crop region) by label values as get_labels
 * does (biomedisa_helper.py:1209-1213): index k -> all_labels[k], except the
 * smallest index present, which maps to 0. */
int si_remap_labels(uint8_t* out, int Zc, int Yc, int Xc, int cz0, int cy0,
                    int cx0, int Z0, int Y0, int X0, const uint32_t* presence,
                    const uint8_t* all_labels, int nol, void* stream);

/* Update arithmetic of the smoothing step phi + 0.01 * kappa. */
enum si_smooth_update {
  SI_SMOOTH_F32 = 0,     /* binary32: phi + RN(0.01f * kappa) */
  SI_SMOOTH_REF_F64 = 1  /* the reference's `phi += 0.01 * curvature`
                            (gpu_kernels.py:133): binary64 product with the
                            binary64 literal 0.01, binary64 sum, rounded to
                            binary32 on the store */
};

/* Floats each of si_smooth's tmp0/tmp1 buffers must hold:
 * Zc*Yc*Xp + 64 with Xp = Xc rounded up to a multiple of 4. */
int si_smooth_tmp_floats(int Zc, int Yc, int Xc, unsigned long long* n);

/* Curvature smoothing (rw_small.py:114-137, gpu_kernels.py:118-183): for each
 * of the nol maps, iters steps of phi <- phi + 0.01 * kappa(phi) on the
 * interior, borders unchanged; kappa in binary32 in the reference's
 * expression order, the update as `update` (enum si_smooth_update). maps
 * holds uint32 hits on entry and float32 smoothed values (bit pattern) on
 * exit. tmp0/tmp1: 16-byte aligned float32 scratch of si_smooth_tmp_floats
 * each. Only kernel launches and asynchronous memsets on `stream`; waits
 * inside the kernels are bounded and record a give-up in the status that
 * si_smooth_status reads. */
int si_smooth(uint32_t* maps, float* tmp0, float* tmp1, int nol, int Zc,
              int Yc, int Xc, int iters, int update, void* stream);

/* si_smooth on float32 maps (in place); used for the hybrid's combined maps. */
int si_smooth_f32(float* maps, float* tmp0, float* tmp1, int nol, int Zc,
                  int Yc, int Xc, int iters, int update, void* stream);

/* Status of the smoothing kernels on the current device since the last call
 * (0 = fine; non-zero: a kernel's wait on its shared-memory copies gave up
 * and its output is incomplete). Synchronises `stream`, then clears the
 * status. Returns SI_ERR_CUDA when the status is non-zero. No counterpart in
 * the reference. */
int si_smooth_status(int* status, void* stream);

/* Voxels per thread of the smoothing kernel: pairs = 1 (default) gives each
 * thread two voxels of a 64-wide column, 2 four voxels of a 128-wide one
 * (faster on dense maps, slower on sparse hit maps). Process-wide; speed
 * only (results do not depend on it). */
int si_smooth_set_pairs(int pairs);

/* Spin limit of every bounded wait on an mbarrier in this library (TMA copies
 * of the smoothing and tile-walker kernels); spins < 0 restores the default
 * (2^26). Process-wide. A wait that runs out makes its kernel wait (bounded)
 * for its copies in flight, record an error status and return. No
 * counterpart in the reference; tests use it to make a wait run out. */
int si_set_wait_limit(long long spins);

/* ---- the reference large path's seed set (optional mode) ----
 * si_extract_seeds with an in-plane box [box_y0, box_y1) x [box_x0, box_x1)
 * (crop y, x) outside which labels read as ignored (-1), as the large path's
 * slice stack after reduceBlocksize (pycuda_large.py:39-58): no seeds there
 * and no contribution to the neighbours' 3x3 variance. */
int si_extract_seeds_box(const void* labels, int dtype, int Z0, int Y0, int X0,
                         int cz0, int cy0, int cx0, int Zc, int Yc, int Xc,
                         const int16_t* slot_lut, const uint8_t* slot_label,
                         const void* work, int work_is_float,
                         const int32_t* slice_list, int n_slices, int box_y0,
                         int box_y1, int box_x0, int box_x1,
                         uint32_t* row_counts, si_seed_t* seeds,
                         uint32_t* n_seeds, void* stream);

/* si_extract_seeds with a box per axis: boxes (HOST array of 12 int32) holds
 * for axis a = 0, 1, 2 the box [r0, r1) x [c0, c1) of that axis' slice plane
 * in crop coordinates (z-slices: rows y, columns x; y-slices: rows z,
 * columns x; x-slices: rows z, columns y) outside which labels read as
 * ignored (-1): the all-axis large path's slice stacks after reduceBlocksize
 * (pycuda_large_allx.py:37-57, one box per axis, :309-322). */
int si_extract_seeds_boxes(const void* labels, int dtype, int Z0, int Y0,
                           int X0, int cz0, int cy0, int cx0, int Zc, int Yc,
                           int Xc, const int16_t* slot_lut,
                           const uint8_t* slot_label, const void* work,
                           int work_is_float, const int32_t* slice_list,
                           int n_slices, const int32_t* boxes,
                           uint32_t* row_counts, si_seed_t* seeds,
                           uint32_t* n_seeds, void* stream);

/* Adaptive seeds (pycuda_large.py:513-533): copies to seeds_out (count in
 * *n_out) the z-slice seeds of seeds_in (*n_in of at most max_in) with
 * (row + column) % 4 == 0 or a label other than their own and -1 within the
 * in-slice window [-100, 100]^2 clipped to the crop interior. slice_z: crop z
 * of the n_slices taken slices (device). Output order is not the input
 * order. Scratch: si_adaptive_scratch_bytes (256-byte aligned). */
int si_adaptive_scratch_bytes(int Zc, int Yc, int Xc, int n_slices,
                              uint64_t* bytes);
int si_adaptive_seed_filter(const void* labels, int dtype, int Z0, int Y0,
                            int X0, int cz0, int cy0, int cx0, int Zc, int Yc,
                            int Xc, const int16_t* slot_lut,
                            const uint8_t* slot_label, const int32_t* slice_z,
                            int n_slices, int box_y0, int box_y1, int box_x0,
                            int box_x1, const si_seed_t* seeds_in,
                            const uint32_t* n_in, uint32_t max_in,
                            si_seed_t* seeds_out, uint32_t* n_out,
                            void* scratch, uint64_t scratch_bytes,
                            void* stream);

/* Adaptive seeds of the all-axis large path (pycuda_large_allx.py:513-533 and
 * :683-703): as si_adaptive_seed_filter for seeds of every axis, each tested
 * in the (row, column) plane of its own slice (axis from the seed's meta
 * bits 8-9) with that axis' box. slice_list: n_slices (axis, index) pairs in
 * crop coordinates (device); boxes: HOST array of 12 int32 as for
 * si_extract_seeds_boxes. Scratch: si_adaptive_scratch_bytes_allx. */
int si_adaptive_scratch_bytes_allx(int Zc, int Yc, int Xc, int n_slices,
                                   uint64_t* bytes);
int si_adaptive_seed_filter_allx(const void* labels, int dtype, int Z0, int Y0,
                                 int X0, int cz0, int cy0, int cx0, int Zc,
                                 int Yc, int Xc, const int16_t* slot_lut,
                                 const uint8_t* slot_label,
                                 const int32_t* slice_list, int n_slices,
                                 const int32_t* boxes,
                                 const si_seed_t* seeds_in,
                                 const uint32_t* n_in, uint32_t max_in,
                                 si_seed_t* seeds_out, uint32_t* n_out,
                                 void* scratch, uint64_t scratch_bytes,
                                 void* stream);

/* ---- outlier removal and hole filling (remove_outlier.py:67-141) ----
 * uint8 label volumes (Z, Y, X), at most 2^31 - 1 voxels; 6-connected
 * components by union-find. Scratch: si_cc_scratch_bytes (16-byte aligned). */
int si_cc_scratch_bytes(int Z, int Y, int X, uint64_t* bytes);

/* clean (remove_outlier.py:67-105): out = labels, except that voxels of a
 * 6-connected component of a label whose size is not > threshold x the
 * label's largest component become 0. Voxels of skip_label (the smallest
 * label present; -1 for none) are left alone. Replaces remove_outlier.clean. */
int si_clean(const uint8_t* labels, uint8_t* out, int Z, int Y, int X,
             double threshold, int skip_label, void* scratch,
             uint64_t scratch_bytes, void* stream);

/* fill (remove_outlier.py:107-141), in place, for the labels of label_list
 * in that order (host array; the reference's labels after the smallest):
 * inside each label's bounding box grown by one voxel, the complement's
 * 6-connected components (box-confined) are filled with the label unless
 * the component is the first maximum of [label size, component sizes] or
 * larger than threshold x label size; if the label itself is that maximum,
 * its voxels become 0. A label with no voxels left is skipped (the reference
 * raises there). Replaces remove_outlier.fill. */
int si_fill(uint8_t* img, int Z, int Y, int X, double threshold,
            const int* label_list, int n_labels, void* scratch,
            uint64_t scratch_bytes, void* stream);

/* ---- geodesic raster-scan interpolation (biomedisa/geodis.py) ----
 * The sequence geodesic_segment() runs is:
 *   si_geo_normalize -> si_label_histogram -> (host: label slots)
 *   -> si_geo_masks -> si_geo_scan -> si_geo_select */

/* out = normalised float32 image: x = float32(img); x -= min(x); x /= max(x)
 * (geodis.py:86-88, numpy semantics: a NaN or an infinite minimum gives NaN
 * everywhere, a constant image 0/0 = NaN). mm: 3 uint32 of device scratch
 * (min/max keys and a NaN flag), overwritten. n >= 1.
 * dtype: SI_U8, SI_I8, SI_U16, SI_I16, SI_I32 or SI_F32. */
int si_geo_normalize(const void* img, int dtype, uint64_t n, float* out,
                     uint32_t* mm, void* stream);

/* Distance seeds of every label slot at once: c[k][v] = 0 where the label
 * value of voxel v has slot k, +inf elsewhere (geodis.py:95-96).
 * slot_lut[v] = slot of label value v (0..255) or -1; values outside 0..255
 * have no slot. c: float32 [nol][n]. dtype: SI_U8, SI_I16 or SI_I32. */
int si_geo_masks(const void* labels, int dtype, uint64_t n,
                 const int16_t* slot_lut, int nol, float* c, void* stream);

/* Replaces geodesic_raster_scan (geodis.py:44-76), run on nol distance
 * volumes c[nol][Z][Y][X] (float32, updated in place) over one float32 image
 * img[Z][Y][X]: `iterations` times a forward and a backward raster pass with
 * cost c[q] + (1 - lamb)|q - p| + lamb (img[p] - img[q])^2, results identical
 * to the sequential scan. The passes run as wavefronts x + 2y + 4z (about
 * X + 2Y + 4Z per pass).
 *   mode 4: tiled: the voxels in skewed coordinates p = x + 2y + 4z,
 *           q = y + 2z, r = z cut into 32 x 32 x 8 tiles; one launch per
 *           tile-wavefront (about (X + 2Y + 4Z)/32 + (Y + 2Z)/32 + Z/8 per
 *           pass), a CTA per tile and volume working in shared memory;
 *   mode 5: mode 4 captured once into a CUDA graph, which later calls with
 *           the same arguments (pointers included) replay;
 *   mode 0: mode 4 on the first call with a set of arguments, mode 5 from the
 *           second on (the default);
 *   mode 1: one kernel launch per wavefront, all volumes in each launch;
 *   mode 3: mode 1 captured into a CUDA graph as mode 5 does;
 *   mode 2: one launch in which a cluster of 8 CTAs per volume runs every
 *           wavefront, separated by the cluster barrier.
 * Modes 0, 3 and 5 keep up to 8 instantiated graphs per process (graph
 * instantiation allocates device memory; the least recently used graph is
 * destroyed when a ninth is made). */
int si_geo_scan(float* c, const float* img, int Z, int Y, int X, int nol,
                double lamb, int iterations, int mode, void* stream);

/* No counterpart in the reference (launch-plan check).
 * Host only (no device work): the launch plan of si_geo_scan's tiled modes
 * for the forward (fwd = 1) or backward (fwd = 0) pass: per voxel the
 * tile-wavefront (launch) wave[v], a tile id tile[v] and the plane step[v] at
 * which its CTA updates it, -1 for voxels the pass leaves alone. Fails if a
 * voxel would be updated twice or a shared-memory neighbour is not the voxel
 * the sequential scan reads. Exposed for checking the order. */
int si_geo_tile_visit_order(int Z, int Y, int X, int fwd, int32_t* wave,
                            int32_t* tile, int32_t* step);

/* No counterpart in the reference (measurement).
 * Host only: *launches = the kernel launches one si_geo_scan call with these
 * arguments makes: 1 in cluster mode (which queries the current device), one
 * per tile-wavefront in the tiled modes (0, 4, 5), one per non-empty
 * wavefront in modes 1 and 3; all times `iterations` and both passes. */
int si_geo_scan_launches(int Z, int Y, int X, double lamb, int iterations,
                         int mode, long long* launches);

/* out[v] = slot_label[k] of the first slot k >= 1 whose distance is strictly
 * below the running minimum that starts at slot 0's, else 0 (the label loop of
 * geodesic_segment, geodis.py:94-103). */
int si_geo_select(const float* c, int nol, uint64_t n,
                  const uint8_t* slot_label, uint8_t* out, void* stream);

/* No counterpart in the reference (launch-plan checks and measurement).
 * Host only (no device work): t_of_voxel[v] = the wavefront at which
 * si_geo_scan's forward (fwd = 1) or backward (fwd = 0) pass updates voxel v,
 * -1 for voxels the pass leaves alone. Fails if a voxel would be updated
 * twice. The launch plan of si_geo_scan, exposed for checking its order. */
int si_geo_visit_order(int Z, int Y, int X, int fwd, int32_t* t_of_voxel);

/* ---- learned surrogate (no counterpart in the reference) ----
 * Tensors are NDHWC; activations bfloat16, weights bfloat16 [27][cout][cin]
 * (tap-major, tap = (dz+1)*9 + (dy+1)*3 + (dx+1)), biases and gradients fp32.
 * Convolutions are 3x3x3, stride 1, zero padding = dilation. */

/* y = relu?(conv(x, w) + bias + residual); bias/residual nullable; out_f32
 * selects an fp32 output. cin: multiple of 16; cout: 16, 32, 48 or 64.
 * Runs on mma.sync (m16n8k16 bf16); for 16 -> 16 see also si_nn_conv16_tc. */
int si_nn_conv3d_fwd(const void* x, const void* w, const float* bias,
                     const void* residual, void* y, int N, int D, int H,
                     int W, int cin, int cout, int dil, int relu, int out_f32,
                     void* stream);

/* The 16 -> 16 convolution of si_nn_conv3d_fwd (same arguments without
 * cin/cout; dil <= 8; 16-byte aligned tensors) on the 5th-generation tensor
 * cores, organised by input rows: per input row and (dz, dx) one tcgen05.mma
 * of M = 128 voxels of an x-row, N = 48 (the three output rows the input row
 * meets, 16 channels each), K = 16, into a ring of fp32 accumulators in
 * tensor memory; rows staged by TMA. Same results as si_nn_conv3d_fwd up to
 * fp32 accumulation order, and independent of the grid. The default of
 * SurrogateNet for its 16 -> 16 layers (2.4x the mma.sync kernel on large
 * volumes, measured). No counterpart in the reference. */
int si_nn_conv16_tc(const void* x, const void* w, const float* bias,
                    const void* residual, void* y, int N, int D, int H, int W,
                    int dil, int relu, int out_f32, void* stream);

/* Status of the tensor-core convolution kernel (si_nn_conv16_tc) on the
 * current device since the last call:
 * 0 = fine; non-zero: a kernel's bounded wait on its copies or MMAs gave up
 * and its output is incomplete. Synchronises `stream`, then clears the
 * status; returns SI_ERR_CUDA when it was non-zero. No counterpart in the
 * reference. */
int si_nn_umma_status(int* status, void* stream);

/* Interleaved column streams per CTA of si_nn_conv16_tc: 1 (default), 2 or
 * 4. Each stream accumulates into its own tensor-memory ring, and the MMAs
 * of a group alternate between streams, so consecutive MMAs accumulate into
 * different columns (measured slower than one stream on GB300).
 * Process-wide; results do not depend on it. */
int si_nn_conv16_tc_set_streams(int streams);

/* dw[27][cout][cin] += sum_v dy[v][co] x[v + off][ci]; db[cout] += sum_v dy
 * (db nullable). (cout, cin) in {16, 32}^2. With `partials` (cin = cout = 16
 * only; size from si_nn_wgrad_partial_bytes, 16-byte aligned) every block
 * writes its own sums and a second pass adds them in block order, so the
 * result is deterministic; with partials = NULL blocks add with atomics. */
int si_nn_wgrad_partial_bytes(int N, int D, int H, int W, int cin, int cout,
                              uint64_t* bytes);
int si_nn_conv3d_wgrad(const void* x, const void* dy, float* dw, float* db,
                       int N, int D, int H, int W, int cin, int cout, int dil,
                       float* partials, uint64_t partial_bytes, void* stream);

/* w_flipped[tap][ci][co] = w[26 - tap][co][ci] (data-gradient weights). */
int si_nn_flip_weights(const void* w, void* w_flipped, int cout, int cin,
                       void* stream);

/* g = g * (y > 0) (+ add, nullable); n elements (bf16). */
int si_nn_relu_bwd(void* g, const void* y, const void* add, int64_t n,
                   void* stream);

/* Soft-target cross entropy over the first nol of C fp32 logits per voxel:
 * *loss += sum_v w_v sum_l -p_l log softmax_l; dlogits (bf16) =
 * w_v (softmax - p) * scale. weight nullable (1). */
int si_nn_xent(const float* logits, const float* target, const float* weight,
               int64_t V, int C, int nol, float scale, void* dlogits,
               float* loss, void* stream);

/* AdamW step on fp32 params (bias-corrected, decoupled weight decay);
 * p_bf16 (nullable) receives the bfloat16 copy. */
int si_nn_adamw(float* p, const float* g, float* m, float* v, void* p_bf16,
                int64_t n, float lr, float beta1, float beta2, float eps,
                float wd, int step, void* stream);

/* Surrogate input features of a box [z0, z0+Dt) x [y0, ..) x [x0, ..) of a
 * uint8 working volume (D, H, W): bf16 [Dt][Ht][Wt][16] = I/255, signed
 * distance to the nearest labelled z-slice / 16 clamped to [-1, 1], 1 on seed
 * voxels (slot_map >= 0), then per label slot s = 0..12 the linear
 * interpolation along z of [slot_map == s] between the labelled z-slices
 * below and above. zinfo: float[D][4] = {distance, z_lo, z_hi, w_lo} (z_lo,
 * z_hi = -1 when absent; 16-byte aligned). Outside the volume: distance 1,
 * rest 0. */
int si_nn_features(const uint8_t* img, const int16_t* slot_map,
                   const float* zinfo, int D, int H, int W, int z0, int y0,
                   int x0, int Dt, int Ht, int Wt, void* out, void* stream);

/* Softmax of fp32 logits [Ds][H][W][16] over the first nol channels for slab
 * planes [zb, ze), written planar into probs[nol][Zout][H][W] at plane zo. */
int si_nn_probs(const float* logits, int Ds, int H, int W, int zb, int ze,
                int nol, float* probs, int Zout, int zo, void* stream);

/* ---- Active contour post-processing ('acwe' and 'refined') -------------
 * Replaces activeContour (biomedisa/features/active_contour.py:109-202, the
 * `acwe` option of smart_interpolation, rw_small.py:246-255 and
 * rw_large.py:262-271), its refinement (:204-225) and curvop_numba.py:5-149.
 * Everything works on the reference's crop: image and labels padded by one
 * zero voxel (padded frame, interior 1..Z, 1..Y, 1..X) and cut to
 * [cz0, cz0+cZ) x [cy0, ..) x [cx0, ..) (reduce_blocksize, :84-104; the host
 * computes the box from si_slice_flags' bbox). D (image) and L (labels) are
 * uint8 crops in C order.
 * Sequence, acwe: si_acwe_minmax (non-uint8 image) -> si_acwe_gather ->
 *   steps x (zero sums -> si_acwe_label_sums -> si_acwe_evolution ->
 *   si_acwe_curvop for every label) -> si_acwe_scatter.
 * Sequence, refined: si_acwe_minmax -> si_acwe_gather -> si_acwe_dist_init ->
 *   si_acwe_chamfer_band -> si_acwe_refine_hist -> si_acwe_refine_decide ->
 *   si_acwe_refine_apply. */

/* mm[0] = min, mm[1] = max (float32 values) of the voxels of an image array
 * that lie in the padded frame's interior; the array's voxel (a, b, c) is
 * padded voxel (iz0 + a, iy0 + b, ix0 + c). The caller initialises mm to
 * (+inf, -inf). img_to_uint8's amin/amax (biomedisa_helper.py:345-352).
 * dtype: SI_U8, SI_I8, SI_U16, SI_I16, SI_I32 or SI_F32. */
int si_acwe_minmax(const void* img, int dtype, int iZ, int iY, int iX, int iz0,
                   int iy0, int ix0, int Z, int Y, int X, float* mm,
                   void* stream);

/* D and L of the crop (active_contour.py:154-170). L = labels (uint8, Z x Y x
 * X) at interior voxels, 0 on the pad. D: the image value (0 outside the
 * image array and on the pad); convert = 0 copies a uint8 image, convert = 1
 * applies img_to_uint8: ((v - mn) / mx) * 255 in binary32, truncated, with
 * mn = amin and mx = amax - amin of the image as the reference sees it. */
int si_acwe_gather(const void* img, int dtype, int iZ, int iY, int iX, int iz0,
                   int iy0, int ix0, int convert, float mn, float mx,
                   const uint8_t* labels, int Z, int Y, int X, int cz0,
                   int cy0, int cx0, int cZ, int cY, int cX, uint8_t* D,
                   uint8_t* L, void* stream);

/* sums[l] += voxels of label l, sums[256 + l] += their intensity sum
 * (l = 0..255) over n voxels; sums zeroed by the caller. The label means of
 * active_contour.py:191-195. */
int si_acwe_label_sums(const uint8_t* D, const uint8_t* L, uint64_t n,
                       unsigned long long* sums, void* stream);

/* One evolution pass (curvop_numba.py:5-29) of the crop (Z, Y, X): out = L
 * with every interior voxel relabelled to the label, among its own and its
 * 27 neighbours', whose mean (float32(sum / count) from sums) is closest to
 * its intensity; label 0's distance is scaled by alpha (binary64). out must
 * not alias L. */
int si_acwe_evolution(const uint8_t* L, const uint8_t* D,
                      const unsigned long long* sums, double alpha, int Z,
                      int Y, int X, uint8_t* out, void* stream);

/* One erosion (erode = 1, curvop_numba.py:31-60) or dilation (erode = 0,
 * :62-84) pass of `label` over the crop; dst must not alias src. */
int si_acwe_morph(const uint8_t* src, int Z, int Y, int X, int label, int erode,
                  uint8_t* dst, void* stream);

/* curvop(L, steps, label) (curvop_numba.py:86-149): `steps` rounds, even
 * rounds erosion then dilation, odd rounds dilation then erosion; the result
 * is left in L (tmp: scratch of the crop's size). */
int si_acwe_curvop(uint8_t* L, uint8_t* tmp, int Z, int Y, int X, int label,
                   int steps, void* stream);

/* out (Z, Y, X) = the crop L put back in the padded frame without the pad
 * (active_contour.py:185-188); 0 outside the crop. */
int si_acwe_scatter(const uint8_t* L, int cz0, int cy0, int cx0, int cZ,
                    int cY, int cX, int Z, int Y, int X, uint8_t* out,
                    void* stream);

/* dist[i] = 100 where L[i] == 0, else 0 (active_contour.py:206-207). */
int si_acwe_dist_init(const uint8_t* L, uint64_t n, float* dist, void* stream);

/* The refinement's chamfer distance (active_contour.py:45-81, one forward and
 * one backward pass from si_acwe_dist_init's map) in the form the band test
 * `distance <= 10` needs: 10 Jacobi passes of the 27-point min-plus stencil
 * (weights 1, sqrt2, sqrt3; rows and columns 0 and n-1 keep their values;
 * values clamped to 11). For every voxel that reaches the result this gives
 * the same band as the reference's scan (the path lengths near 10 are
 * exactly 10 or at least 0.0246 away from it). dist (Z x Y x X float32) is
 * updated in place; tmp: scratch of the same size. */
int si_acwe_chamfer_band(float* dist, float* tmp, int Z, int Y, int X,
                         void* stream);

/* Band histograms of the refinement: hist[z][class_lut[L]][D] counts the
 * crop voxels of slice z with dist <= 10 (active_contour.py:209-210,
 * 213-216); hist (Z x ncls x 256 uint32) zeroed by the caller; class_lut[256]
 * maps a label value to its class (-1 = not counted). */
int si_acwe_refine_hist(const float* dist, const uint8_t* D, const uint8_t* L,
                        const int16_t* class_lut, int ncls, int Z, int Y,
                        int X, uint32_t* hist, void* stream);

/* lut[z][v] (Z x 256) from histograms of ncand + 1 classes: candidate j is
 * label cand_label[j] in class j + 1 (class 0 holds the other labels). For
 * every candidate in order (the reference's allLabels[1:]) whose band in
 * slice z holds voxels of the label and of other labels, the Gaussian
 * likelihoods of intensity v under the two band classes (mean, standard
 * deviation clamped to >= 1) give cand_label[j] where p1 > p2, else 0; a
 * later candidate overwrites the slice (active_contour.py:212-224). */
int si_acwe_refine_decide(const uint32_t* hist, const uint8_t* cand_label,
                          int ncand, int Z, uint8_t* lut, void* stream);

/* Refined labels out (Z, Y, X): lut[slice][D] at crop voxels with dist <= 10,
 * 0 elsewhere and outside the crop. */
int si_acwe_refine_apply(const float* dist, const uint8_t* D,
                         const uint8_t* lut, int cz0, int cy0, int cx0, int cZ,
                         int cY, int cX, int Z, int Y, int X, uint8_t* out,
                         void* stream);

/* Measurement probes (no counterpart in the reference; used by bench.py for
 * the walker's roofline denominators). si_probe_l2_read reads `bytes` of buf
 * `reps` times with L1-bypassing 16-byte loads (sink: one uint32, almost never
 * written). si_probe_l2_atomics performs n_atomics 4-byte atomic adds at
 * scattered positions of buf (`words` uint32, a power of two). */
int si_probe_l2_read(const void* buf, uint64_t bytes, int reps, uint32_t* sink,
                     void* stream);
int si_probe_l2_atomics(uint32_t* buf, uint64_t words, uint64_t n_atomics,
                        void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SMARTINTERP_H */
