// gb_device.cuh -- device-side building blocks of the registration-metric kernels.
//
// GB300 issues FP64 at a small fraction of its FP32 rate, so nothing in the
// per-sample loops is FP64.  Positions are mapped in double-float arithmetic:
// the per-evaluation affine map (virtual point -> moving continuous index) is
// computed once in FP64 and split into FP32 hi/lo pairs; each sample's
// (exactly representable, float) coordinates are multiplied with error-free
// FMA products and summed with two-sum, giving the continuous index to ~1e-12
// voxel, i.e. the reference's double arithmetic for every practical input,
// including points that fall exactly on a buffer edge.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gb {

constexpr int kWarp = 32;

// FP64 multiply / add that are never fused into an FMA: positions computed in
// FP64 must round exactly like the reference's separate operations (a fused
// product-sum turns an exact cancellation into a 1e-20 residue, which moves
// points off exact buffer-edge ties).  Host code is built with -ffp-contract=off.
__host__ __device__ __forceinline__ double dmul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
__host__ __device__ __forceinline__ double dadd(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}

// ---------------------------------------------------------------------------
// Programmatic dependent launch.  The kernels of one evaluation run back to
// back on a stream; each one after the first is launched with programmatic
// stream serialization, so its blocks may be scheduled while its predecessor
// drains.  griddep_wait() blocks until the predecessor grids have completed
// and their memory writes are visible (a no-op for a normal launch); nothing
// before it may touch global memory that a predecessor reads or writes.
// griddep_launch_dependents() lets the next kernel's blocks be scheduled.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// ---------------------------------------------------------------------------
// Kahan-compensated FP32 accumulator (the reference's CompensatedSummation,
// Core/Common/include/itkCompensatedSummation.hxx:38-48, at FP32).
struct KahanF {
  float s, c;
  __device__ __forceinline__ void zero() { s = 0.f; c = 0.f; }
  __device__ __forceinline__ void add(float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);  // _rn intrinsics are never contracted or reassociated
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

__device__ __forceinline__ unsigned warp_sum_u(unsigned v) { return __reduce_add_sync(0xffffffffu, v); }

// ---------------------------------------------------------------------------
// Cubic B-spline Parzen window (order 3).  With the window starting at bin
// pdfm = midx - 1 and t = term - midx in [0, 1], the four arguments are
// -1-t, -t, 1-t, 2-t; BSplineKernelFunction<3> (Core/Common/include/itkBSplineKernelFunction.h:152-169)
// and BSplineDerivativeKernelFunction<3> (itkBSplineDerivativeKernelFunction.h:156-180)
// evaluated there are the uniform cubic B-spline basis polynomials below.

// 6 * beta3(arg_k), k = 0..3 (integer coefficients: no rounding of 1/6)
__device__ __forceinline__ void parzen6(float t, float w6[4]) {
  const float u = 1.f - t;
  const float t2 = t * t, t3 = t2 * t;
  w6[0] = u * u * u;
  w6[1] = fmaf(3.f, t3, fmaf(-6.f, t2, 4.f));
  w6[2] = fmaf(-3.f, t3, fmaf(3.f, t2, fmaf(3.f, t, 1.f)));
  w6[3] = t3;
}

// beta3'(arg_k), k = 0..3
__device__ __forceinline__ void parzen_deriv(float t, float d[4]) {
  const float u = 1.f - t;
  d[0] = 0.5f * u * u;
  d[1] = t * fmaf(-1.5f, t, 2.f);
  d[2] = u * fmaf(1.5f, u, -2.f);
  d[3] = -0.5f * t * t;
}

// ---------------------------------------------------------------------------
// A continuous index as its nearest integer b = floor(cidx + 0.5) and the
// centred remainder f = cidx - b in [-0.5, 0.5).  Positions close to a voxel
// centre keep full relative precision in f, and the buffer test becomes exact.
struct CIdx {
  int b[3];
  float f[3];
};

// ImageFunction::IsInsideBuffer: cidx in [-0.5, n - 0.5) per axis, NaN outside
// (Core/ImageFunction/include/itkImageFunction.h:157-169).  With b the
// round-half-up index, cidx >= -0.5 <=> b >= 0 and cidx < n - 0.5 <=> b <= n - 1.
__device__ __forceinline__ bool ci_inside(const CIdx& c, int nx, int ny, int nz) {
  const int n[3] = {nx, ny, nz};
  bool in = true;
#pragma unroll
  for (int k = 0; k < 3; ++k) in = in && (c.f[k] == c.f[k]) && c.b[k] >= 0 && c.b[k] <= n[k] - 1;
  return in;
}

// Corner indices and weights of LinearInterpolateImageFunction's 3-D path
// (Core/ImageFunction/include/itkLinearInterpolateImageFunction.h:227-470):
// trilinear interpolation with neighbours clamped to the buffer, an axis with
// distance <= 0 below the start contributing the start voxel only.  Measured
// from the nearest voxel b, the second corner is b + sign(f) with weight |f|.
struct Stencil {
  int x0, x1, y0, y1, z0, z1;
  float dx, dy, dz;
};

__device__ __forceinline__ void stencil_axis(int b, float f, int n, int& i0, int& i1, float& w) {
  i0 = b;
  int j = f > 0.f ? b + 1 : (f < 0.f ? b - 1 : b);
  j = j < 0 ? 0 : (j > n - 1 ? n - 1 : j);
  i1 = j;
  w = fabsf(f);
}

__device__ __forceinline__ Stencil make_stencil(const CIdx& c, int nx, int ny, int nz) {
  Stencil s;
  stencil_axis(c.b[0], c.f[0], nx, s.x0, s.x1, s.dx);
  stencil_axis(c.b[1], c.f[1], ny, s.y0, s.y1, s.dy);
  stencil_axis(c.b[2], c.f[2], nz, s.z0, s.z1, s.dz);
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

// ---------------------------------------------------------------------------
// double-float helpers

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// A position as unevaluated sums hi + lo per axis (|lo| <= ulp(hi) / 2).
struct DFPos {
  float hi[3], lo[3];
};

// Affine map virtual point -> moving continuous index, as FP32 hi/lo pairs:
// cidx_k = sum_j (Ahi + Alo)[k][j] x_j + (bhi + blo)[k].
struct __align__(16) AffineDF {
  float Ahi[9], Alo[9], bhi[3], blo[3];
};

// A copy of a shared-memory map in six 16-byte loads (the per-sample loops read
// the map once per sample; narrower loads cost more shared-memory wavefronts).
__device__ __forceinline__ AffineDF load_map(const AffineDF& s) {
  static_assert(sizeof(AffineDF) == 96, "six float4");
  AffineDF r;
  const float4* v = reinterpret_cast<const float4*>(&s);
  float4* o = reinterpret_cast<float4*>(&r);
#pragma unroll
  for (int k = 0; k < 6; ++k) o[k] = v[k];
  return r;
}

// Continuous index of one float point to ~1e-12 voxel: products by FMA error
// terms, sums by two-sum.
__device__ __forceinline__ DFPos map_pos(const AffineDF& K, float x, float y, float z) {
  const float xs[3] = {x, y, z};
  DFPos r;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float s = K.bhi[k], err = K.blo[k];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float a = K.Ahi[3 * k + j];
      const float p = __fmul_rn(a, xs[j]);
      const float pe = __fmaf_rn(a, xs[j], -p);  // exact product error
      float t, e;
      two_sum(s, p, t, e);
      s = t;
      err = __fadd_rn(err, __fadd_rn(e, __fmaf_rn(K.Alo[3 * k + j], xs[j], pe)));
    }
    r.hi[k] = __fadd_rn(s, err);
    r.lo[k] = __fsub_rn(err, __fsub_rn(r.hi[k], s));
  }
  return r;
}

// Nearest integer b = floor(hi + lo + 0.5) and the remainder hi + lo - b.
__device__ __forceinline__ void split_nearest(float hi, float lo, int& b, float& f) {
  float s, e;
  two_sum(hi, 0.5f, s, e);
  const float e2 = __fadd_rn(e, lo);
  float fl = floorf(s);
  if (s == fl) {
    if (e2 < 0.f) fl -= 1.f;
  } else if (e2 >= __fsub_rn(fl + 1.f, s)) {
    fl += 1.f;
  }
  b = (int)fl;  // saturates for huge values: outside any buffer
  f = __fadd_rn(__fsub_rn(hi, fl), lo);
}

__device__ __forceinline__ CIdx to_cidx(const DFPos& p) {
  CIdx c;
#pragma unroll
  for (int k = 0; k < 3; ++k) split_nearest(p.hi[k], p.lo[k], c.b[k], c.f[k]);
  return c;
}

__device__ __forceinline__ CIdx map_df(const AffineDF& K, float x, float y, float z) {
  return to_cidx(map_pos(K, x, y, z));
}

// p + (dhi + dlo) per axis, renormalized.
__device__ __forceinline__ DFPos df_offset(const DFPos& p, const float* dhi, const float* dlo, float sign) {
  DFPos r;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float s, e;
    two_sum(p.hi[k], sign * dhi[k], s, e);
    e = __fadd_rn(e, __fadd_rn(p.lo[k], sign * dlo[k]));
    r.hi[k] = __fadd_rn(s, e);
    r.lo[k] = __fsub_rn(e, __fsub_rn(r.hi[k], s));
  }
  return r;
}

// A double as an unevaluated float pair hi + lo by integer operations only (no
// FP64 instruction): hi is the double truncated to 24 significant bits, lo the
// remaining 29 bits rounded to float, so hi + lo = x within 2^-47 |x|.
// |x| < 2^-126 gives 0 (lo is 0 below 2^-74); |x| >= 2^128, inf and NaN give NaN.
__device__ __forceinline__ void split_double_bits(double x, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned w1 = (unsigned)(b >> 32), w0 = (unsigned)b;
  const unsigned sign = w1 & 0x80000000u;
  const int e = (int)((w1 >> 20) & 0x7ffu);  // biased exponent
  if (e < 897) {
    hi = 0.f;
    lo = 0.f;
    return;
  }
  if (e > 1150) {
    hi = __int_as_float(0x7fc00000);
    lo = 0.f;
    return;
  }
  hi = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | ((w1 & 0xfffffu) << 3) | (w0 >> 29));
  lo = e < 949 ? 0.f : __uint2float_rn(w0 & 0x1fffffffu) * __uint_as_float(sign | ((unsigned)(e - 948) << 23));
}

// p + A u for a double-float matrix A and a double-float vector u (products with
// FMA error terms, sums by two-sum), renormalized.
__device__ __forceinline__ DFPos df_add_matvec(const DFPos& p, const AffineDF& A, const float uhi[3],
                                               const float ulo[3]) {
  DFPos r;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float s = p.hi[k], err = p.lo[k];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float a = A.Ahi[3 * k + j];
      const float q = __fmul_rn(a, uhi[j]);
      const float qe = __fmaf_rn(a, uhi[j], -q);  // exact product error
      float t, e;
      two_sum(s, q, t, e);
      s = t;
      err = __fadd_rn(err, __fadd_rn(e, __fadd_rn(qe, __fmaf_rn(A.Alo[3 * k + j], uhi[j], __fmul_rn(a, ulo[j])))));
    }
    r.hi[k] = __fadd_rn(s, err);
    r.lo[k] = __fsub_rn(err, __fsub_rn(r.hi[k], s));
  }
  return r;
}

// ---------------------------------------------------------------------------
// Ordered-int encodings of floats for atomic min/max.
__device__ __forceinline__ int float_to_ordered(float f) {
  int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float ordered_to_float(int i) {
  return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff);
}

// 21-bit-per-axis Morton interleave (x fastest bit).
__device__ __forceinline__ uint64_t morton_spread(uint64_t v) {
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffULL;
  v = (v | v << 16) & 0x1f0000ff0000ffULL;
  v = (v | v << 8) & 0x100f00f00f00f00fULL;
  v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
  v = (v | v << 2) & 0x1249249249249249ULL;
  return v;
}
// Sample sort keys: B-spline cell above this bit, spatial order below it.
constexpr int kCellShift = 41;

__device__ __forceinline__ uint64_t morton3(uint32_t x, uint32_t y, uint32_t z) {
  return morton_spread(x) | (morton_spread(y) << 1) | (morton_spread(z) << 2);
}

}  // namespace gb
