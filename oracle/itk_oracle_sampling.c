/*
 * itk_oracle_sampling.c -- the registration method's metric sample points
 * (TEST INFRASTRUCTURE ONLY; see itk_oracle.h).
 *
 * Restates (paths relative to the ITK source tree, Modules/):
 *   MT19937 state, reload and tempering
 *       Core/Common/src/itkMersenneTwisterRandomVariateGenerator.cxx:175-263
 *   variates (open range, open upper range, normal)
 *       Core/Common/include/itkMersenneTwisterRandomVariateGenerator.h:188-227,350-373
 *   random voxel of ImageRandomConstIteratorWithIndex
 *       Core/Common/include/itkImageRandomConstIteratorWithIndex.hxx:47-68
 *   ImageBase::TransformIndexToPhysicalPoint into a float point
 *       Core/Common/include/itkImageBase.h:593-604
 *   ImageRegistrationMethodv4::SetMetricSamplePoints (REGULAR, RANDOM)
 *       Registration/RegistrationMethodsv4/include/itkImageRegistrationMethodv4.hxx:869-1024
 *
 * The generator is written here from Matsumoto and Nishimura's published
 * MT19937 (n = 624, m = 397, matrix 0x9908b0df, tempering 11 / 7 0x9d2c5680 /
 * 15 0xefc60000 / 18, seeding x[i] = 1812433253 (x[i-1] ^ (x[i-1] >> 30)) + i),
 * generating the whole state block at a time as the reference does.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "itk_oracle.h"

#define MT_N 624
#define MT_M 397

typedef struct {
  uint32_t x[MT_N];
  int next;
} orc_mt;

static void mt_regenerate(orc_mt *g) {
  for (int k = 0; k < MT_N; ++k) {
    const uint32_t y = (g->x[k] & 0x80000000u) | (g->x[(k + 1) % MT_N] & 0x7fffffffu);
    g->x[k] = g->x[(k + MT_M) % MT_N] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
  }
  g->next = 0;
}

static void mt_seed(orc_mt *g, uint32_t seed) {
  g->x[0] = seed;
  for (uint32_t i = 1; i < MT_N; ++i) g->x[i] = 1812433253u * (g->x[i - 1] ^ (g->x[i - 1] >> 30)) + i;
  mt_regenerate(g);
}

static uint32_t mt_u32(orc_mt *g) {
  if (g->next == MT_N) mt_regenerate(g);
  uint32_t y = g->x[g->next++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

static double mt_open(orc_mt *g) { return ((double)mt_u32(g) + 0.5) / 4294967296.0; }
static double mt_open_upper(orc_mt *g) { return (double)mt_u32(g) / 4294967296.0; }

static double mt_normal(orc_mt *g) {
  const double u1 = mt_open(g);
  const double r = sqrt((-2.0 * log(1.0 - u1)) * 1.0);
  const double u2 = mt_open_upper(g);
  const double phi = (2.0 * 3.14159265358979323846) * u2;
  return 0.0 + r * cos(phi);
}

int orc_mt_sequence(uint32_t seed, int64_t skip, uint32_t *out, int64_t n) {
  static orc_mt g;
  mt_seed(&g, seed);
  for (int64_t i = 0; i < skip; ++i) (void)mt_u32(&g);
  for (int64_t i = 0; i < n; ++i) out[i] = mt_u32(&g);
  return ORC_OK;
}

int orc_mt_normals(uint32_t seed, double *out, int64_t n) {
  static orc_mt g;
  mt_seed(&g, seed);
  for (int64_t i = 0; i < n; ++i) out[i] = mt_normal(&g);
  return ORC_OK;
}

/* index -> float point (compound float assignments), then the jitter */
static void make_point(const double i2p[9], const double origin[3], const double third[3], const int64_t idx[3],
                       orc_mt *rnd, float *out) {
  float p[3];
  for (int i = 0; i < 3; ++i) {
    p[i] = (float)origin[i];
    for (int j = 0; j < 3; ++j) p[i] = (float)((double)p[i] + i2p[3 * i + j] * (double)idx[j]);
  }
  for (int d = 0; d < 3; ++d) p[d] = (float)((double)p[d] + mt_normal(rnd) * third[d]);
  memcpy(out, p, sizeof(p));
}

/* strategy 1 REGULAR, 2 RANDOM; geometry = spacing[3], origin[3], direction[9] */
int orc_sample_points(int strategy, const int64_t size[3], const double *geometry, double percentage, int32_t seed,
                      float *xyz, int64_t capacity, int64_t *count) {
  const double *sp = geometry, *org = geometry + 3, *dir = geometry + 6;
  const int64_t nx = size[0], ny = size[1], nz = size[2];
  const int64_t V = nx * ny * nz;
  double i2p[9], third[3];
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) i2p[3 * r + c] = dir[3 * r + c] * sp[c];
    third[r] = sp[r] / 3.0;
  }
  static orc_mt rnd, it;
  mt_seed(&rnd, (uint32_t)seed);
  int64_t n = 0;
  if (strategy == 1) {
    const uint64_t step = (uint64_t)ceil(1.0 / percentage);
    n = (int64_t)((V + (int64_t)step - 1) / (int64_t)step);
    if (n > capacity) return ORC_ERR_BAD_ARG;
    int64_t k = 0;
    for (int64_t v = 0; v < V; v += (int64_t)step) {
      const int64_t idx[3] = {v % nx, (v / nx) % ny, v / (nx * ny)};
      make_point(i2p, org, third, idx, &rnd, xyz + 3 * k);
      ++k;
    }
  } else if (strategy == 2) {
    n = (int64_t)(unsigned long)((double)(float)V * percentage);
    if (n > capacity) return ORC_ERR_BAD_ARG;
    /* GoToBegin jumps once; after each sample ++ jumps again */
    mt_seed(&it, (uint32_t)seed + 1u);
    const double span = (double)V - 0.5;
    int64_t pos = (int64_t)(mt_open(&it) * span);
    for (int64_t k = 0; k < n; ++k) {
      int64_t idx[3];
      int64_t q = pos;
      idx[0] = q % nx;
      q /= nx;
      idx[1] = q % ny;
      q /= ny;
      idx[2] = q % nz;
      make_point(i2p, org, third, idx, &rnd, xyz + 3 * k);
      pos = (int64_t)(mt_open(&it) * span);
    }
  } else {
    return ORC_ERR_BAD_ARG;
  }
  *count = n;
  return ORC_OK;
}
