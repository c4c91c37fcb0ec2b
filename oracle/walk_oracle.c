/*
 * walk_oracle.c — CPU oracle (test infrastructure only) for the random-walker
 * step of smart interpolation. Not part of the product: only tests/, the
 * smoke check and bench.py's CPU-baseline leg load it.
 *
 * A literal restatement of the reference walker loop
 * (biomedisa/features/random_walk/pycuda_small.py:138-257 and
 * pyopencl_small.py:192-314): per seed, nbrw walks of sorw steps; six
 * cumulative weights in the order +z,-z,+y,-y,+x,-x; an if-chain picks the
 * interval holding rnd = W5*u (rnd == 0 -> +z); a move that would leave
 * [1, dim-2] is refused but counts as a step; accepted moves add one hit at the
 * target; after sorw steps the walker returns to its seed and the random stream
 * continues.
 *
 * Two interchangeable parts make the same loop usable both as the checker of
 * the GPU kernel and for pinning against the reference's own kernels:
 *   rng    OR_RNG_PHILOX  Philox4x32-10 (Salmon et al., SC'11), counter
 *                         (t/4, seed pos, axis, label), t = walk*sorw + step,
 *                         u = (word >> 8) * 2^-24;
 *          OR_RNG_REF_MRG the reference's binary32 "MRG32k3a" recurrence
 *                         (pycuda_small.py:155-165, :197-225) with all six
 *                         state words set to the seed's rng_index.
 *   weight OR_W_EXP2      w = 2^(-d2 * c), c = RN(RN(1/RN(2 var)) * log2e),
 *                         by the exponent-split + degree-5 polynomial method
 *                         the product uses (fmaf is correctly rounded);
 *          OR_W_REF_EXPF  w = expf(RN(RN(-tmp*tmp) * div1)),
 *                         div1 = RN(1 / RN(2 var)) (pycuda_small.py:133-136).
 * Built with -ffp-contract=off: every binary32 operation rounds on its own.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

enum { OR_RNG_PHILOX = 0, OR_RNG_REF_MRG = 1 };
enum { OR_W_EXP2 = 0, OR_W_REF_EXPF = 1 };

typedef struct {
  uint32_t pos;       /* linear index in the working volume */
  uint32_t slot;      /* label slot (index into the hit maps) */
  uint32_t axis;      /* seed axis (0 = z slices) */
  uint32_t label;     /* label value */
  float b;            /* seed intensity (uint8 value or float) */
  float var;          /* clamped in-slice variance */
  uint32_t rng_index; /* reference MRG init value (OR_RNG_REF_MRG only) */
  uint32_t pad;
} or_seed_t;

/* ---------------- Philox4x32-10 ---------------- */
static void philox4x32_10(const uint32_t in[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
  uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

void or_philox(const uint32_t* ctr, uint32_t k0, uint32_t k1, uint32_t* out, int64_t n) {
  for (int64_t i = 0; i < n; ++i) philox4x32_10(ctr + 4 * i, k0, k1, out + 4 * i);
}

/* ---------------- weights ---------------- */
static inline float f_as(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}
static inline uint32_t u_as(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}

static const float kLog2e = 1.44269502162933349609375f;
static const float kMagic = 12582912.0f; /* 1.5 * 2^23 */

static float weight_exp2(float d2, float c) {
  const float y = d2 * c;
  if (!(y < 125.0f)) return 0.0f;
  const float r = y + kMagic;
  const float kf = r - kMagic;
  const float g = kf - y;
  float p = fmaf(0.0013260921696200967f, g, 0.009670175611972809f);
  p = fmaf(p, g, 0.055507123470306396f);
  p = fmaf(p, g, 0.2402222454547882f);
  p = fmaf(p, g, 0.6931470036506653f);
  p = fmaf(p, g, 1.0f);
  const int32_t k = (int32_t)u_as(r) - 0x4B400000;
  return f_as(u_as(p) - ((uint32_t)k << 23));
}

float or_weight_exp2(float d2, float c) { return weight_exp2(d2, c); }

float or_weight_constant(float var) {
  const float two_var = 2.0f * var;
  const float div1 = 1.0f / two_var;
  return div1 * kLog2e;
}

/* ---------------- the walk ---------------- */
typedef struct {
  /* reference MRG state */
  float s10, s11, s12, s20, s21, s22;
  /* Philox block cache */
  uint32_t blk[4];
  uint32_t blk_id;
  int blk_valid;
} rng_state;

static float next_u_ref(rng_state* st) {
  /* binary32 recurrence exactly as written in pycuda_small.py:197-225 */
  const float m1 = 4294967087.0f, m2 = 4294944443.0f;
  const float a12 = 1403580.0f, a13n = 810728.0f, a21 = 527612.0f, a23n = 1370589.0f;
  const float norm = 2.328306549295728e-10f;
  long k1;
  float p1, p2;
  p1 = a12 * st->s11 - a13n * st->s10;
  k1 = (long)(p1 / m1);
  p1 -= (float)k1 * m1;
  if (p1 < 0.0f) p1 += m1;
  st->s10 = st->s11;
  st->s11 = st->s12;
  st->s12 = p1;
  p2 = a21 * st->s22 - a23n * st->s20;
  k1 = (long)(p2 / m2);
  p2 -= (float)k1 * m2;
  if (p2 < 0.0f) p2 += m2;
  st->s20 = st->s21;
  st->s21 = st->s22;
  st->s22 = p2;
  if (p1 <= p2) return (p1 - p2 + m1) * norm;
  return (p1 - p2) * norm;
}

static float next_u_philox(rng_state* st, uint32_t t, const or_seed_t* sd, uint32_t k0, uint32_t k1) {
  const uint32_t q = t >> 2;
  if (!st->blk_valid || st->blk_id != q) {
    const uint32_t ctr[4] = {q, sd->pos, sd->axis, sd->label};
    philox4x32_10(ctr, k0, k1, st->blk);
    st->blk_id = q;
    st->blk_valid = 1;
  }
  const uint32_t w = st->blk[t & 3u];
  return (float)(w >> 8) * 5.9604644775390625e-8f;
}

static inline float intensity(const void* img, int is_float, int64_t p) {
  if (is_float) return ((const float*)img)[p];
  return (float)((const uint8_t*)img)[p];
}

static inline float weight_of(int wmode, float b, float v, float c, float div1) {
  const float tmp = b - v;
  if (wmode == OR_W_EXP2) return weight_exp2(tmp * tmp, c);
  return expf(-tmp * tmp * div1);
}

/*
 * hits: uint32 [nol][Z][Y][X], accumulated (caller zeroes).
 * Returns 0, or -1 on bad arguments.
 */
int or_walk(const void* img, int is_float, int Z, int Y, int X, const or_seed_t* seeds, int64_t n_seeds, int nbrw,
            int sorw, uint64_t key, int rng_mode, int weight_mode, uint32_t* hits, int nol, int nthreads) {
  if (!img || (!seeds && n_seeds) || !hits || Z < 3 || Y < 3 || X < 3 || nol < 1) return -1;
  const int64_t flat = (int64_t)X * Y;
  const int64_t V = flat * Z;
  const uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int64_t si = 0; si < n_seeds; ++si) {
    const or_seed_t* sd = &seeds[si];
    if (sd->slot >= (uint32_t)nol) continue;
    uint32_t* a = hits + (int64_t)sd->slot * V;
    const int plane = (int)(sd->pos / flat);
    const int row = (int)((sd->pos - (int64_t)plane * flat) / X);
    const int column = (int)(sd->pos - (int64_t)plane * flat - (int64_t)row * X);
    const float B = sd->b;
    const float c = or_weight_constant(sd->var);
    const float div1 = 1.0f / (2.0f * sd->var);
    rng_state st;
    const float init = (float)sd->rng_index;
    st.s10 = st.s11 = st.s12 = st.s20 = st.s21 = st.s22 = init;
    st.blk_valid = 0;
    st.blk_id = 0;
    int k = plane, l = row, m = column;
    int64_t position = sd->pos;
    int step = 0, n_rw = 0;
    int n = 0, o = 0, p = 0;
    uint32_t t = 0;
    while (n_rw < nbrw) {
      float W0 = weight_of(weight_mode, B, intensity(img, is_float, position + flat), c, div1);
      float W1 = weight_of(weight_mode, B, intensity(img, is_float, position - flat), c, div1);
      float W2 = weight_of(weight_mode, B, intensity(img, is_float, position + X), c, div1);
      float W3 = weight_of(weight_mode, B, intensity(img, is_float, position - X), c, div1);
      float W4 = weight_of(weight_mode, B, intensity(img, is_float, position + 1), c, div1);
      float W5 = weight_of(weight_mode, B, intensity(img, is_float, position - 1), c, div1);
      W1 += W0;
      W2 += W1;
      W3 += W2;
      W4 += W3;
      W5 += W4;
      const float u = rng_mode == OR_RNG_PHILOX ? next_u_philox(&st, t, sd, k0, k1) : next_u_ref(&st);
      const float rnd = W5 * u;
      if (rnd < W0 || rnd == 0) {
        n = 1; o = 0; p = 0;
      } else if (rnd >= W0 && rnd < W1) {
        n = -1; o = 0; p = 0;
      } else if (rnd >= W1 && rnd < W2) {
        n = 0; o = 1; p = 0;
      } else if (rnd >= W2 && rnd < W3) {
        n = 0; o = -1; p = 0;
      } else if (rnd >= W3 && rnd < W4) {
        n = 0; o = 0; p = 1;
      } else if (rnd >= W4 && rnd <= W5) {
        n = 0; o = 0; p = -1;
      }
      if (k + n > 0 && k + n < Z - 1 && l + o > 0 && l + o < Y - 1 && m + p > 0 && m + p < X - 1) {
        k += n;
        l += o;
        m += p;
        position = (int64_t)k * flat + (int64_t)l * X + m;
        __atomic_fetch_add(&a[position], 1u, __ATOMIC_RELAXED);
      }
      step += 1;
      t += 1;
      if (step == sorw) {
        k = plane;
        l = row;
        m = column;
        position = (int64_t)k * flat + (int64_t)l * X + m;
        n_rw += 1;
        step = 0;
      }
    }
  }
  return 0;
}
