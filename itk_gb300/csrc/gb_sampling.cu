// gb_sampling.cu -- the registration method's metric sample points, made on the
// host exactly as the reference makes them (host code only).
//
// Reference semantics (paths relative to ITK's Modules/):
//   SetMetricSamplePoints (REGULAR, RANDOM)     Registration/RegistrationMethodsv4/include/itkImageRegistrationMethodv4.hxx:869-1024
//   seeds: m_CurrentRandomSeed++ per generator  same file, :927-934, :977-984, reset per Update at :794
//   random voxel                                Core/Common/include/itkImageRandomConstIteratorWithIndex.hxx:47-68
//   Mersenne Twister variates                   Core/Common/include/itkMersenneTwisterRandomVariateGenerator.h:188-227,350-373
//   Mersenne Twister state and tempering        Core/Common/src/itkMersenneTwisterRandomVariateGenerator.cxx:175-263
//   index -> float point                        Core/Common/include/itkImageBase.h:593-604
//
// The reference's generator is MT19937 (Matsumoto-Nishimura) with the 1812433253
// seeding recurrence: its 32-bit outputs are those of std::mt19937 constructed
// from the same seed, which this file uses.  The sample points are float points
// (PointSet's default coordinate type), accumulated in float exactly as the
// reference's compound assignments do, and the normal variates use the host's
// log / cos, as the reference does.
#include <cmath>
#include <cstdint>
#include <random>
#include <string>

#include "gb_internal.h"

namespace gb {

namespace {

class Variates {
 public:
  explicit Variates(int32_t seed) : g_((uint32_t)seed) {}
  uint32_t integer() { return (uint32_t)g_(); }
  // GetVariateWithOpenRange: (0, 1)
  double open_range() { return ((double)integer() + 0.5) / 4294967296.0; }
  // GetVariateWithOpenUpperRange: [0, 1)
  double open_upper_range() { return (double)integer() / 4294967296.0; }
  // GetNormalVariate(0, 1): the Box-Muller cosine branch, one variate per call
  double normal() {
    const double r = std::sqrt((-2.0 * std::log(1.0 - open_range())) * 1.0);
    const double phi = (2.0 * 3.141592653589793238462643383279502884) * open_upper_range();
    return 0.0 + r * std::cos(phi);
  }

 private:
  std::mt19937 g_;
};

// TransformIndexToPhysicalPoint into a float point, then the jitter
// point[d] += N(0,1) * spacing[d] / 3, each step rounded to float.
struct PointMaker {
  double i2p[9];
  double origin[3];
  double third[3];
  void make(int64_t ix, int64_t iy, int64_t iz, Variates& rnd, float* out) const {
    const int64_t idx[3] = {ix, iy, iz};
    float p[3];
    for (int i = 0; i < 3; ++i) {
      p[i] = (float)origin[i];
      for (int j = 0; j < 3; ++j) p[i] = (float)((double)p[i] + i2p[3 * i + j] * (double)idx[j]);
    }
    for (int d = 0; d < 3; ++d) p[d] = (float)((double)p[d] + rnd.normal() * third[d]);
    out[0] = p[0];
    out[1] = p[1];
    out[2] = p[2];
  }
};

}  // namespace

}  // namespace gb

using namespace gb;

extern "C" int gb_sample_count(int strategy, const int64_t size[3], double percentage, int64_t* count) {
  if (!size || !count) return fail(GB_ERR_BAD_ARG, "null argument");
  if (size[0] <= 0 || size[1] <= 0 || size[2] <= 0) return fail(GB_ERR_BAD_ARG, "empty virtual domain");
  const int64_t V = size[0] * size[1] * size[2];
  if (strategy == GB_SAMPLING_NONE) {
    *count = V;
  } else if (strategy == GB_SAMPLING_RANDOM) {
    // static_cast<unsigned long>(static_cast<float>(voxels) * percentage)
    *count = (int64_t)(unsigned long)((double)(float)V * percentage);
  } else if (strategy == GB_SAMPLING_REGULAR) {
    if (!(percentage > 0.0)) return fail(GB_ERR_BAD_ARG, "sampling percentage must be > 0");
    const uint64_t step = (uint64_t)std::ceil(1.0 / percentage);
    *count = (int64_t)((V + step - 1) / step);  // voxels 0, step, 2 step, ... in scan order
  } else {
    return fail(GB_ERR_BAD_ARG, "Invalid sampling strategy requested.");
  }
  return GB_OK;
}

extern "C" int gb_sample_points(int strategy, const int64_t size[3], const double spacing[3], const double origin[3],
                                const double direction[9], double percentage, int32_t seed, float* xyz,
                                int64_t capacity, int64_t* count, int32_t* next_seed) {
  if (!size || !spacing || !origin || !direction || !count) return fail(GB_ERR_BAD_ARG, "null argument");
  if (strategy != GB_SAMPLING_REGULAR && strategy != GB_SAMPLING_RANDOM)
    return fail(GB_ERR_BAD_ARG, "Invalid sampling strategy requested.");
  int64_t n = 0;
  int rc = gb_sample_count(strategy, size, percentage, &n);
  if (rc) return rc;
  if (n > capacity || (n > 0 && !xyz)) return fail(GB_ERR_BAD_ARG, "output holds fewer points than the sample count");
  Geom g;
  rc = geom_init(g, size, spacing, origin, direction);
  if (rc) return rc;
  PointMaker pm;
  for (int i = 0; i < 9; ++i) pm.i2p[i] = g.i2p[i];
  for (int i = 0; i < 3; ++i) {
    pm.origin[i] = origin[i];
    pm.third[i] = spacing[i] / 3.0;
  }
  // the randomizer takes m_CurrentRandomSeed++; RANDOM's iterator the next one
  int32_t s = seed;
  Variates rnd(s);
  s = (int32_t)((uint32_t)s + 1u);
  const int64_t nx = size[0], ny = size[1];
  if (strategy == GB_SAMPLING_REGULAR) {
    const uint64_t step = (uint64_t)std::ceil(1.0 / percentage);
    uint64_t c = step;  // the first voxel is a sample
    int64_t k = 0;
    const int64_t V = size[0] * size[1] * size[2];
    for (int64_t v = 0; v < V; ++v) {
      if (c == step) {
        c = 0;
        pm.make(v % nx, (v / nx) % ny, v / (nx * ny), rnd, xyz + 3 * k);
        ++k;
      }
      ++c;
    }
  } else {
    Variates it(s);
    s = (int32_t)((uint32_t)s + 1u);
    const double span = (double)(size[0] * size[1] * size[2]) - 0.5;
    // GoToBegin jumps once before the first sample; every ++ jumps again
    auto jump = [&](int64_t& ix, int64_t& iy, int64_t& iz) {
      int64_t pos = (int64_t)(it.open_range() * span);
      ix = pos % nx;
      pos = (pos - ix) / nx;
      iy = pos % ny;
      pos = (pos - iy) / ny;
      iz = pos;
    };
    int64_t ix, iy, iz;
    jump(ix, iy, iz);
    for (int64_t k = 0; k < n; ++k) {
      pm.make(ix, iy, iz, rnd, xyz + 3 * k);
      jump(ix, iy, iz);
    }
  }
  *count = n;
  if (next_seed) *next_seed = s;
  return GB_OK;
}
