// gb_init.cuh -- Initialize()-time kernels: image ranges, the device sample
// list (fixed values / fixed Parzen bins in FP64), packing of the moving image.
#pragma once

#include <cfloat>

#include "gb_device.cuh"

namespace gb {

// FP64 trilinear interpolation with the reference's clamps
// (Core/ImageFunction/include/itkLinearInterpolateImageFunction.h:227-470);
// used once per Initialize for the fixed image, so its value equals the
// reference's double interpolation rounded to float.
__device__ __forceinline__ double interp_d(const float* __restrict__ img, const int64_t n[3], const double ci[3]) {
  int64_t b0[3], b1[3];
  double d[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    int64_t f = (int64_t)floor(ci[k]);
    if (f < 0) f = 0;
    double dist = ci[k] - (double)f;
    b0[k] = f;
    b1[k] = f + 1 <= n[k] - 1 ? f + 1 : f;
    if (!(dist > 0.0)) { dist = 0.0; b1[k] = f; }
    d[k] = dist;
  }
  const int64_t nx = n[0], nxy = n[0] * n[1];
#define GBPIX(x, y, z) ((double)img[(x) + (y) * nx + (z) * nxy])
  const double v000 = GBPIX(b0[0], b0[1], b0[2]), v100 = GBPIX(b1[0], b0[1], b0[2]);
  const double v010 = GBPIX(b0[0], b1[1], b0[2]), v110 = GBPIX(b1[0], b1[1], b0[2]);
  const double v001 = GBPIX(b0[0], b0[1], b1[2]), v101 = GBPIX(b1[0], b0[1], b1[2]);
  const double v011 = GBPIX(b0[0], b1[1], b1[2]), v111 = GBPIX(b1[0], b1[1], b1[2]);
#undef GBPIX
  if (d[0] <= 0.0 && d[1] <= 0.0 && d[2] <= 0.0) return v000;
  // a + (b - a) d with separate roundings, as the reference computes it
#define GBLERP(a, b, t) dadd((a), dmul(dadd((b), -(a)), (t)))
  const double x00 = GBLERP(v000, v100, d[0]);
  const double x10 = GBLERP(v010, v110, d[0]);
  const double x01 = GBLERP(v001, v101, d[0]);
  const double x11 = GBLERP(v011, v111, d[0]);
  const double xx0 = GBLERP(x00, x10, d[1]);
  const double xx1 = GBLERP(x01, x11, d[1]);
  return GBLERP(xx0, xx1, d[2]);
#undef GBLERP
}

struct DGeom {
  int64_t n[3];
  double origin[3];
  double i2p[9];
  double p2i[9];
};

__device__ __forceinline__ void d_point_to_cindex(const DGeom& g, const double p[3], double ci[3]) {
  double v[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) v[k] = dadd(p[k], -g.origin[k]);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s = dadd(s, dmul(g.p2i[3 * i + j], v[j]));
    ci[i] = s;
  }
}

__device__ __forceinline__ bool d_inside(const DGeom& g, const double ci[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (!(ci[k] >= -0.5 && ci[k] < (double)(g.n[k] - 1) + 0.5)) return false;
  return true;
}

// TransformPhysicalPointToIndex (round half up) + inside test, itkImageBase.h:463-479
__device__ __forceinline__ bool d_nearest_index(const DGeom& g, const double p[3], int64_t idx[3]) {
  bool inside = true;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s = dadd(s, dmul(g.p2i[3 * i + j], dadd(p[j], -g.origin[j])));
    idx[i] = (int64_t)floor(dadd(s, 0.5));
    if (idx[i] < 0 || idx[i] >= g.n[i]) inside = false;
  }
  return inside;
}

struct BuildArgs {
  const float* points;  // sampled points (xyz) or nullptr for the dense virtual grid
  int64_t n;            // candidates
  int points_virtual;
  DGeom virt, fixed;
  const float* fixed_img;
  int mattes;
  int bins;
  double f_bs, f_normmin;
  // B-spline support (transform kinds 1, 2)
  int bspline;
  int64_t grid[3];
  double g_origin[3];
  double g_p2i[9];
  uint64_t* keys;
  uint32_t* vals;
  float4* recs;
  float4* sup;  // B-spline support record per candidate (null without a B-spline)
  uint32_t* voff;  // nearest virtual voxel per candidate, ~0u outside (displacement field on a point set; else null)
  unsigned long long* nvalid;
};

__device__ __forceinline__ int64_t dbl_ulp_order(double x) {
  long long i = __double_as_longlong(x);
  if (i < 0) i = (long long)0x8000000000000000LL - i;
  return i;
}

// BSplineTransform::InsideValidRegion, Core/Transform/include/itkBSplineTransform.hxx:478-507
__device__ __forceinline__ bool d_bspline_inside(const int64_t grid[3], double ci[3]) {
  const double minLimit = 1.0;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const double maxLimit = (double)grid[j] - 1.0 - 1.0;
    bool almost = fabs(ci[j] - maxLimit) <= 0.1 * DBL_EPSILON;
    if (!almost && (signbit(ci[j]) == signbit(maxLimit))) {
      long long d = dbl_ulp_order(ci[j]) - dbl_ulp_order(maxLimit);
      if (d < 0) d = -d;
      almost = d <= 4;
    }
    if (almost) ci[j] = __longlong_as_double(__double_as_longlong(maxLimit) - 6);
    else if (ci[j] >= maxLimit) return false;
    else if (ci[j] < minLimit) return false;
  }
  return true;
}

// One candidate sample: virtual point -> fixed value (FP64 interpolation,
// TransformAndEvaluateFixedPoint, itkImageToImageMetricv4.hxx:290-322) and,
// for Mattes, the fixed Parzen bin (ComputeSingleFixedImageParzenWindowIndex,
// Mattes...v4.hxx:571-597).  Invalid candidates get key ~0 and sort last.
__global__ void k_build_samples(BuildArgs b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.n) return;
  double vp[3];
  bool ok = true;
  if (b.points) {
    vp[0] = b.points[3 * i];
    vp[1] = b.points[3 * i + 1];
    vp[2] = b.points[3 * i + 2];
    if (!b.points_virtual) {
      // MapFixedSampledPointSetToVirtual keeps points whose nearest virtual index is inside, .hxx:594-607
      int64_t vi[3];
      ok = d_nearest_index(b.virt, vp, vi);
    }
  } else {
    const int64_t nx = b.virt.n[0], ny = b.virt.n[1];
    const double idx[3] = {(double)(i % nx), (double)((i / nx) % ny), (double)(i / (nx * ny))};
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      double p = b.virt.origin[r];
      for (int c = 0; c < 3; ++c) p = dadd(p, dmul(b.virt.i2p[3 * r + c], idx[c]));
      vp[r] = p;
    }
  }
  float fval = 0.f;
  if (ok) {
    double ci[3];
    d_point_to_cindex(b.fixed, vp, ci);
    ok = d_inside(b.fixed, ci);
    if (ok) fval = (float)interp_d(b.fixed_img, b.fixed.n, ci);
  }
  float aux = fval;
  if (ok && b.mattes) {
    const double term = (double)fval / b.f_bs - b.f_normmin;
    long long p = (long long)term;
    if (p < 2) p = 2;
    else if (p > b.bins - 3) p = b.bins - 3;
    aux = __int_as_float((int)p);
  }
  // B-spline support of the virtual point (BSplineTransform::TransformPoint,
  // itkBSplineTransform.hxx:510-591): in-cell positions t = ci - start - 1 in
  // [0, 1] and the start node packed as sx | sy << 10 | sz << 20 | valid << 30;
  // cell = 1 + start's linear node index (0: outside the valid region).
  float4 sup = make_float4(0.f, 0.f, 0.f, 0.f);
  uint64_t cell = 0;
  if (ok && b.bspline) {
    double ci[3], v[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) v[k] = dadd(vp[k], -b.g_origin[k]);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      double s = 0.0;
      for (int j = 0; j < 3; ++j) s = dadd(s, dmul(b.g_p2i[3 * r + j], v[j]));
      ci[r] = s;
    }
    if (d_bspline_inside(b.grid, ci)) {
      int st[3];
      float t[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        st[k] = (int)floor(dadd(dadd(ci[k], 0.5), -1.5));  // BSplineInterpolationWeightFunction start index
        t[k] = (float)dadd(dadd(ci[k], -(double)st[k]), -1.0);
      }
      const unsigned packed = (unsigned)st[0] | ((unsigned)st[1] << 10) | ((unsigned)st[2] << 20) | (1u << 30);
      sup = make_float4(t[0], t[1], t[2], __uint_as_float(packed));
      cell = 1 + (uint64_t)st[0] + (uint64_t)b.grid[0] * ((uint64_t)st[1] + (uint64_t)b.grid[1] * (uint64_t)st[2]);
    }
  }
  uint64_t key = ~0ull;
  if (ok) {
    int64_t vi[3];
    d_nearest_index(b.virt, vp, vi);
    const uint32_t x = (uint32_t)(vi[0] < 0 ? 0 : vi[0]);
    const uint32_t y = (uint32_t)(vi[1] < 0 ? 0 : vi[1]);
    const uint32_t z = (uint32_t)(vi[2] < 0 ? 0 : vi[2]);
    // 8 x 2 x 2 bricks of the virtual grid in Morton order, scan order inside a
    // brick: a warp's samples cover long x runs over few (y, z) rows, so the
    // trilinear gathers of one load instruction touch few 128-byte lines
    const uint64_t brick = morton3((x >> 3) & 0xfff, (y >> 1) & 0xfff, (z >> 1) & 0xfff) & ((1ull << 36) - 1);
    key = (brick << 5) | ((uint64_t)(z & 1) << 4) | ((uint64_t)(y & 1) << 3) | (uint64_t)(x & 7) |
          (cell << kCellShift);
    atomicAdd(b.nvalid, 1ull);
  }
  b.keys[i] = key;
  b.vals[i] = (uint32_t)i;
  // domain coordinates: the point for a point set, the exact grid index for the dense domain
  if (b.points) b.recs[i] = make_float4((float)vp[0], (float)vp[1], (float)vp[2], aux);
  else b.recs[i] = make_float4((float)(i % b.virt.n[0]), (float)((i / b.virt.n[0]) % b.virt.n[1]),
                               (float)(i / (b.virt.n[0] * b.virt.n[1])), aux);
  if (b.sup) b.sup[i] = sup;
  if (b.voff) {
    // the derivative block's voxel: TransformPhysicalPointToIndex of the point
    // (ImageToImageMetricv4GetValueAndDerivativeThreader.hxx:58), with
    // ComputeParameterOffsetFromVirtualIndex (itkObjectToObjectMetric.hxx:332-343)
    int64_t vi[3];
    const bool in = d_nearest_index(b.virt, vp, vi);
    b.voff[i] = in ? (uint32_t)(vi[0] + b.virt.n[0] * (vi[1] + b.virt.n[1] * vi[2])) : 0xffffffffu;
  }
}

__global__ void k_gather_samples(const uint32_t* __restrict__ perm, int64_t n, const float4* __restrict__ recs,
                                 float4* __restrict__ out, const float4* __restrict__ sup_in,
                                 float4* __restrict__ sup_out, const uint32_t* __restrict__ voff_in,
                                 uint32_t* __restrict__ voff_out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t j = perm[i];
  out[i] = recs[j];
  if (sup_out) sup_out[i] = sup_in[j];
  if (voff_out) voff_out[i] = voff_in[j];
}

// min / max over a float buffer (ordered-int atomics): out[0] = min, out[1] = max
__global__ void k_minmax(const float* __restrict__ img, int64_t n, int* out) {
  float lo = FLT_MAX, hi = -FLT_MAX;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float v = img[i];
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&out[0], float_to_ordered(lo));
    atomicMax(&out[1], float_to_ordered(hi));
  }
}

// Mattes fixed range over the sampled points (nearest-index pixel values),
// itkMattesMutualInformationImageToImageMetricv4.hxx:99-153
__global__ void k_minmax_points(const float* __restrict__ pts, int64_t n, DGeom fixed, const float* __restrict__ img,
                                int* out) {
  float lo = FLT_MAX, hi = -FLT_MAX;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double p[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    int64_t idx[3];
    if (d_nearest_index(fixed, p, idx)) {
      const float v = img[idx[0] + fixed.n[0] * (idx[1] + fixed.n[1] * idx[2])];
      lo = fminf(lo, v);
      hi = fmaxf(hi, v);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&out[0], float_to_ordered(lo));
    atomicMax(&out[1], float_to_ordered(hi));
  }
}

// (value, gx, gy, gz) packing of the moving image and its gradient image
// (CovariantVector<double,3> voxels, rounded to FP32).
__global__ void k_pack_moving(const float* __restrict__ mov, const double* __restrict__ grad, int64_t n,
                              float4* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 v = make_float4(mov[i], 0.f, 0.f, 0.f);
  if (grad) {
    v.y = (float)grad[3 * i];
    v.z = (float)grad[3 * i + 1];
    v.w = (float)grad[3 * i + 2];
  }
  out[i] = v;
}

}  // namespace gb
