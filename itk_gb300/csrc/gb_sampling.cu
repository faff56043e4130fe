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
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "gb_internal.h"

namespace gb {

namespace {

// GetVariateWithOpenRange (0, 1) and GetVariateWithOpenUpperRange [0, 1) of one 32-bit output.
inline double open_range(uint32_t u) { return ((double)u + 0.5) / 4294967296.0; }
inline double open_upper_range(uint32_t u) { return (double)u / 4294967296.0; }

// GetNormalVariate(0, 1) from two consecutive outputs: the Box-Muller cosine branch.
inline double normal(uint32_t u1, uint32_t u2) {
  const double r = std::sqrt((-2.0 * std::log(1.0 - open_range(u1))) * 1.0);
  const double phi = (2.0 * 3.141592653589793238462643383279502884) * open_upper_range(u2);
  return 0.0 + r * std::cos(phi);
}

// TransformIndexToPhysicalPoint into a float point, then the jitter
// point[d] += N(0,1) * spacing[d] / 3, each step rounded to float; `u` holds the
// sample's six jitter outputs.
struct PointMaker {
  double i2p[9];
  double origin[3];
  double third[3];
  void make(int64_t ix, int64_t iy, int64_t iz, const uint32_t* u, float* out) const {
    const int64_t idx[3] = {ix, iy, iz};
    float p[3];
    for (int i = 0; i < 3; ++i) {
      p[i] = (float)origin[i];
      for (int j = 0; j < 3; ++j) p[i] = (float)((double)p[i] + i2p[3 * i + j] * (double)idx[j]);
    }
    for (int d = 0; d < 3; ++d) p[d] = (float)((double)p[d] + normal(u[2 * d], u[2 * d + 1]) * third[d]);
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
  // the randomizer takes m_CurrentRandomSeed++; RANDOM's iterator the next one.  The
  // generators' outputs are drawn in sequence; the points (float index-to-point
  // sums, normal variates) are then formed on all host threads.
  const int32_t s_jitter = seed;
  const int32_t s_iter = (int32_t)((uint32_t)seed + 1u);
  const int32_t s = (int32_t)((uint32_t)seed + (strategy == GB_SAMPLING_RANDOM ? 2u : 1u));
  std::vector<uint32_t> jitter((size_t)(6 * n));
  auto draw_jitter = [&]() {
    std::mt19937 rnd((uint32_t)s_jitter);
    for (uint32_t& u : jitter) u = (uint32_t)rnd();
  };
  const int64_t nx = size[0], ny = size[1];
  std::vector<int64_t> vox((size_t)n);
  if (strategy == GB_SAMPLING_REGULAR) {
    // every ceil(1 / percentage)-th voxel in scan order, starting with the first
    draw_jitter();
    const int64_t step = (int64_t)std::ceil(1.0 / percentage);
    for (int64_t k = 0; k < n; ++k) vox[(size_t)k] = k * step;
  } else {
    // ImageRandomConstIteratorWithIndex: GoToBegin jumps once, every ++ jumps again.
    // The two generators are independent: the jitter stream is drawn on a second thread.
    std::thread other;
    try {
      other = std::thread(draw_jitter);
    } catch (...) {
      draw_jitter();
    }
    std::mt19937 it((uint32_t)s_iter);
    const double span = (double)(size[0] * size[1] * size[2]) - 0.5;
    for (int64_t k = 0; k < n; ++k) vox[(size_t)k] = (int64_t)(open_range((uint32_t)it()) * span);
    if (other.joinable()) other.join();
  }
  parallel_ranges(n, [&](int64_t k0, int64_t k1) {
    for (int64_t k = k0; k < k1; ++k) {
      const int64_t v = vox[(size_t)k];
      pm.make(v % nx, (v / nx) % ny, v / (nx * ny), jitter.data() + 6 * k, xyz + 3 * k);
    }
  });
  *count = n;
  if (next_seed) *next_seed = s;
  return GB_OK;
}
