// gb_device.cuh -- device-side building blocks of the registration-metric kernels.
//
// Per-point arithmetic is FP32.  Positions are carried as an exact integer
// voxel index plus an FP32 fraction: each warp anchors its 32 (spatially
// sorted) samples on one of them, maps the anchor to moving-image index space
// in FP64 once, and maps every other sample by its small offset from the
// anchor in FP32.  The fraction inside the voxel is then accurate to ~1e-6
// voxel instead of the ~2e-5 that a plain FP32 transform of a 256 mm
// coordinate gives.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gb {

constexpr int kWarp = 32;

// ---------------------------------------------------------------------------
// Kahan-compensated FP32 accumulator (the reference's CompensatedSummation,
// Core/Common/include/itkCompensatedSummation.hxx:38-48, at FP32).
struct KahanF {
  float s, c;
  __device__ __forceinline__ void zero() { s = 0.f; c = 0.f; }
  __device__ __forceinline__ void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = __fsub_rn(__fsub_rn(t, s), y);  // _rn intrinsics keep nvcc from contracting this away
    s = t;
  }
  __device__ __forceinline__ float value() const { return s - c; }
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ unsigned warp_sum_u(unsigned v) {
  return __reduce_add_sync(0xffffffffu, v);
}

// ---------------------------------------------------------------------------
// Cubic B-spline Parzen kernels (order 3), as polynomials of |u|:
// BSplineKernelFunction<3>, Core/Common/include/itkBSplineKernelFunction.h:152-169
// BSplineDerivativeKernelFunction<3>, Core/Common/include/itkBSplineDerivativeKernelFunction.h:156-180
__device__ __forceinline__ float bspline3(float u) {
  const float a = fabsf(u);
  if (a < 1.f) {
    const float s = a * a;
    return (4.f - 6.f * s + 3.f * s * a) * (1.f / 6.f);
  }
  if (a < 2.f) {
    const float s = a * a;
    return (8.f - 12.f * a + 6.f * s - s * a) * (1.f / 6.f);
  }
  return 0.f;
}

__device__ __forceinline__ float bspline3_deriv(float u) {
  if (u >= 0.f && u < 1.f) return -2.f * u + 1.5f * u * u;
  if (u > -1.f && u < 0.f) return -2.f * u - 1.5f * u * u;
  if (u >= 1.f && u < 2.f) return -2.f + 2.f * u - 0.5f * u * u;
  if (u > -2.f && u <= -1.f) return 2.f + 2.f * u + 0.5f * u * u;
  return 0.f;
}

// ---------------------------------------------------------------------------
// A continuous index as integer base + fraction in [0, 1).
struct CIdx {
  int b[3];
  float f[3];
};

// Buffer test of LinearInterpolateImageFunction / ImageFunction::IsInsideBuffer:
// cindex in [-0.5, n - 0.5) per axis (Core/ImageFunction/include/itkImageFunction.h:157-169).
__device__ __forceinline__ bool ci_inside(const CIdx& c, int nx, int ny, int nz) {
  const int n[3] = {nx, ny, nz};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int b = c.b[k];
    if (b >= 0 && b <= n[k] - 2) continue;
    if (b == -1) { if (!(c.f[k] >= 0.5f)) return false; continue; }
    if (b == n[k] - 1) { if (!(c.f[k] < 0.5f)) return false; continue; }
    return false;
  }
  return true;
}

// Corner indices and weights of LinearInterpolateImageFunction's 3-D path
// (Core/ImageFunction/include/itkLinearInterpolateImageFunction.h:227-470):
// base clamped to 0, distance clamped to >= 0, neighbour clamped to the end.
struct Stencil {
  int x0, x1, y0, y1, z0, z1;
  float dx, dy, dz;
};

__device__ __forceinline__ Stencil make_stencil(const CIdx& c, int nx, int ny, int nz) {
  Stencil s;
  int b;
  float d;
  b = c.b[0]; d = c.f[0];
  if (b < 0) { b = 0; d = 0.f; }
  s.x0 = b; s.x1 = (b + 1 <= nx - 1 && d > 0.f) ? b + 1 : b; s.dx = d > 0.f ? d : 0.f;
  b = c.b[1]; d = c.f[1];
  if (b < 0) { b = 0; d = 0.f; }
  s.y0 = b; s.y1 = (b + 1 <= ny - 1 && d > 0.f) ? b + 1 : b; s.dy = d > 0.f ? d : 0.f;
  b = c.b[2]; d = c.f[2];
  if (b < 0) { b = 0; d = 0.f; }
  s.z0 = b; s.z1 = (b + 1 <= nz - 1 && d > 0.f) ? b + 1 : b; s.dz = d > 0.f ? d : 0.f;
  return s;
}

__device__ __forceinline__ float lerp(float a, float b, float t) { return fmaf(b - a, t, a); }

__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float t) {
  return make_float4(lerp(a.x, b.x, t), lerp(a.y, b.y, t), lerp(a.z, b.z, t), lerp(a.w, b.w, t));
}

// Trilinear gather of the packed (value, gx, gy, gz) moving image.
__device__ __forceinline__ float4 gather4(const float4* __restrict__ img, const Stencil& s, int nx, int ny) {
  // 32-bit offsets: volumes are limited to 2^31 voxels at set-up
  const unsigned sy = (unsigned)nx, sz = (unsigned)nx * (unsigned)ny;
  const unsigned r00 = s.z0 * sz + s.y0 * sy, r10 = s.z0 * sz + s.y1 * sy;
  const unsigned r01 = s.z1 * sz + s.y0 * sy, r11 = s.z1 * sz + s.y1 * sy;
  const float4 v000 = __ldg(img + r00 + s.x0), v100 = __ldg(img + r00 + s.x1);
  const float4 v010 = __ldg(img + r10 + s.x0), v110 = __ldg(img + r10 + s.x1);
  const float4 v001 = __ldg(img + r01 + s.x0), v101 = __ldg(img + r01 + s.x1);
  const float4 v011 = __ldg(img + r11 + s.x0), v111 = __ldg(img + r11 + s.x1);
  const float4 x00 = lerp4(v000, v100, s.dx), x10 = lerp4(v010, v110, s.dx);
  const float4 x01 = lerp4(v001, v101, s.dx), x11 = lerp4(v011, v111, s.dx);
  const float4 xx0 = lerp4(x00, x10, s.dy), xx1 = lerp4(x01, x11, s.dy);
  return lerp4(xx0, xx1, s.dz);
}

// Trilinear gather of a scalar image.
__device__ __forceinline__ float gather1(const float* __restrict__ img, const Stencil& s, int nx, int ny) {
  // 32-bit offsets: volumes are limited to 2^31 voxels at set-up
  const unsigned sy = (unsigned)nx, sz = (unsigned)nx * (unsigned)ny;
  const unsigned r00 = s.z0 * sz + s.y0 * sy, r10 = s.z0 * sz + s.y1 * sy;
  const unsigned r01 = s.z1 * sz + s.y0 * sy, r11 = s.z1 * sz + s.y1 * sy;
  const float v000 = __ldg(img + r00 + s.x0), v100 = __ldg(img + r00 + s.x1);
  const float v010 = __ldg(img + r10 + s.x0), v110 = __ldg(img + r10 + s.x1);
  const float v001 = __ldg(img + r01 + s.x0), v101 = __ldg(img + r01 + s.x1);
  const float v011 = __ldg(img + r11 + s.x0), v111 = __ldg(img + r11 + s.x1);
  const float x00 = lerp(v000, v100, s.dx), x10 = lerp(v010, v110, s.dx);
  const float x01 = lerp(v001, v101, s.dx), x11 = lerp(v011, v111, s.dx);
  const float xx0 = lerp(x00, x10, s.dy), xx1 = lerp(x01, x11, s.dy);
  return lerp(xx0, xx1, s.dz);
}

// Split a small FP32 offset t (relative to an integer base) into base + fraction.
__device__ __forceinline__ void split_add(int base, float t, int& b, float& f) {
  const float fl = floorf(t);
  b = base + (int)fl;
  f = t - fl;
}

// Warp anchor: integer + fractional moving-index position of the anchor sample.
struct Anchor {
  float ax, ay, az;   // anchor position (virtual space, float)
  int ib[3];          // floor of the anchor's moving continuous index
  float fb[3];        // fraction of the anchor's moving continuous index
};

// Moving continuous index of a sample at (x, y, z) from the warp anchor:
// cidx = A (p - a) + cidx(a), A the 3x3 map virtual point -> moving index.
__device__ __forceinline__ CIdx map_from_anchor(const Anchor& an, const float* A, float x, float y, float z) {
  const float d0 = x - an.ax, d1 = y - an.ay, d2 = z - an.az;
  CIdx c;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float t = fmaf(A[3 * k + 0], d0, fmaf(A[3 * k + 1], d1, fmaf(A[3 * k + 2], d2, an.fb[k])));
    split_add(an.ib[k], t, c.b[k], c.f[k]);
  }
  return c;
}

// Anchor from a moving-index position given in FP64.
__device__ __forceinline__ void anchor_set(Anchor& an, float ax, float ay, float az, const double ci[3]) {
  an.ax = ax; an.ay = ay; an.az = az;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double fl = floor(ci[k]);
    an.ib[k] = (int)fl;
    an.fb[k] = (float)(ci[k] - fl);
  }
}

__device__ __forceinline__ Anchor anchor_bcast(const Anchor& a, int src) {
  Anchor r;
  r.ax = __shfl_sync(0xffffffffu, a.ax, src);
  r.ay = __shfl_sync(0xffffffffu, a.ay, src);
  r.az = __shfl_sync(0xffffffffu, a.az, src);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    r.ib[k] = __shfl_sync(0xffffffffu, a.ib[k], src);
    r.fb[k] = __shfl_sync(0xffffffffu, a.fb[k], src);
  }
  return r;
}

// Ordered-int encodings of floats for atomic min/max.
__device__ __forceinline__ int float_to_ordered(float f) {
  int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float ordered_to_float(int i) {
  return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff);
}

// 10-bit-per-axis Morton interleave (x fastest bit).
__device__ __forceinline__ uint64_t morton_spread(uint64_t v) {
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffULL;
  v = (v | v << 16) & 0x1f0000ff0000ffULL;
  v = (v | v << 8) & 0x100f00f00f00f00fULL;
  v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
  v = (v | v << 2) & 0x1249249249249249ULL;
  return v;
}
__device__ __forceinline__ uint64_t morton3(uint32_t x, uint32_t y, uint32_t z) {
  return morton_spread(x) | (morton_spread(y) << 1) | (morton_spread(z) << 2);
}

}  // namespace gb
