/*
 * Geodesic raster scan — CPU oracle (TEST INFRASTRUCTURE ONLY; the product
 * never links this file).
 *
 * Literal restatement of geodesic_raster_scan (biomedisa/geodis.py:44-76):
 * `iterations` times a forward raster pass (z = 1..Z-1, y = 1..Y-2,
 * x = 1..X-2, in that loop order) over the 13 "earlier" neighbours of
 * geodis.py:12-26, then a backward pass (z = Z-2..0, y = Y-2..1, x = X-2..1)
 * over the negated offsets of :28-42, updating c in place.
 *
 * Scalar types follow numba's typing of that function (nopython mode):
 *   img[p] - img[q]        float32 - float32 -> float32
 *   (...)**2               float32 ** int64  -> float32 (a * a)
 *   c[q] + (1-lamb)*d      float32 + float64 -> float64
 *   ... + lamb*(...)**2    float64 + float64 -> float64
 *   best                   float32 and float64 assignments unify to float64
 *   c[p] = best            float64 -> float32, round to nearest even
 * Compiled with -ffp-contract=off so no multiply-add is fused.
 */
#include <math.h>
#include <stdint.h>

static const int kOff[13][3] = {
    {-1, -1, -1}, {-1, -1, 0}, {-1, -1, 1}, {-1, 0, -1}, {-1, 0, 0}, {-1, 0, 1}, {-1, 1, -1},
    {-1, 1, 0},   {-1, 1, 1},  {0, -1, -1}, {0, -1, 0},  {0, -1, 1}, {0, 0, -1},
};

/* d of each offset: sqrt(3) for three nonzero components, sqrt(2) for two, 1.0 for one. */
static double offset_length(int n) {
  int nz = (kOff[n][0] != 0) + (kOff[n][1] != 0) + (kOff[n][2] != 0);
  return nz == 3 ? sqrt(3.0) : nz == 2 ? sqrt(2.0) : 1.0;
}

static void update(const float* img, float* c, int64_t v, const int64_t* off, int sign, double lamb,
                   const double* w) {
  double best = (double)c[v];
  for (int n = 0; n < 13; ++n) {
    int64_t q = v + sign * off[n];
    float diff = img[v] - img[q];
    float sq = diff * diff;
    double cost = ((double)c[q] + w[n]) + lamb * (double)sq;
    if (cost < best) best = cost;
  }
  c[v] = (float)best;
}

/* Runs the scan in place on c (Z, Y, X), float32 C order. Returns 0. */
int or_geo_scan(const float* img, float* c, int Z, int Y, int X, double lamb, int iterations) {
  const int64_t YX = (int64_t)Y * X;
  int64_t off[13];
  double w[13];
  for (int n = 0; n < 13; ++n) {
    off[n] = kOff[n][0] * YX + (int64_t)kOff[n][1] * X + kOff[n][2];
    w[n] = (1.0 - lamb) * offset_length(n);
  }
  for (int it = 0; it < iterations; ++it) {
    for (int z = 1; z < Z; ++z)
      for (int y = 1; y < Y - 1; ++y)
        for (int x = 1; x < X - 1; ++x) update(img, c, z * YX + (int64_t)y * X + x, off, 1, lamb, w);
    for (int z = Z - 2; z >= 0; --z)
      for (int y = Y - 2; y > 0; --y)
        for (int x = X - 2; x > 0; --x) update(img, c, z * YX + (int64_t)y * X + x, off, -1, lamb, w);
  }
  return 0;
}
