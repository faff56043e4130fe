// gb_jhmi.cuh -- JointHistogramMutualInformationImageToImageMetricv4, affine transforms.
//
// Reference (paths under ITK's Modules/Registration/Metricsv4/include/):
//   Initialize (true min / max over the whole images, joint-PDF geometry)
//                                  itkJointHistogramMutualInformationImageToImageMetricv4.hxx:70-190
//   joint histogram, smoothing, marginals (InitializeForIteration)          .hxx:207-303
//   value (ComputeValue, MI in bits)                                        .hxx:340-378
//   joint-PDF point                                                         .hxx:389-401
//   histogram point     itkJointHistogramMutualInformationComputeJointPDFThreaderBase.hxx:57-150
//   derivative point    itkJointHistogramMutualInformationGetValueAndDerivativeThreader.hxx:41-277
//
// Three kernels per evaluation:
//   k_jhmi_pass1    per sample: moving value (and gradient, cached for pass 2), the
//                   joint bin of (f, m), an integer count in a shared-memory
//                   histogram, flushed with 64-bit atomics (order-free, so exact);
//   k_jhmi_finalize a few blocks: the normalized PDF, the discrete-Gaussian smoothing
//                   (separable, zero-flux border, moving axis first), the marginals
//                   and the value (fixed-order trees); FP32 tables for pass 2;
//   k_jhmi_pass2    per sample: bilinear PDF value and moving-axis slope, the
//                   marginal and its slope, the clamped log-slope difference times
//                   J^T g, fixed-order sums; the last block divides by the count.
// A joint bin is floor((p - origin) / spacing + 0.5) of p = (v - min) / (max - min):
// computed in FP32, and again in FP64 exactly as the reference does where the FP32
// result lies within 1e-4 of a rounding boundary, so every sample lands in the
// reference's bin.
#pragma once

#include "gb_bspline.cuh"
#include "gb_field.cuh"
#include "gb_kernels.cuh"

namespace gb {

constexpr int kJhmiMaxBins = 64;  // the finalize blocks keep two bins^2 FP64 planes in shared memory
constexpr int kJhmiFinalizeBlocks = 8;

// Joint-PDF constants (host-computed in FP64 at Initialize).
struct JhmiConsts {
  double fmin, fmax, mmin, mmax;  // true min / max of the whole fixed and moving images
  double origin, inv_spacing;     // joint-PDF geometry: origin -2 s, 1 / s, s = 1 / (bins - 5)
  double spacing;
  float fmin_f, finv_f, mmin_f, minv_f;  // FP32 twins: min, 1 / (max - min)
  float origin_f, inv_spacing_f, spacing_f;
  int radius;                            // discrete Gaussian radius (0: no smoothing)
  double kernel[65];                     // 2 radius + 1 coefficients
};

// Joint bin along one axis: TransformPhysicalPointToIndex (round half up) of the
// joint-PDF point; -1 outside [0, bins).
__device__ __forceinline__ int jhmi_bin(float v, float vmin_f, float vinv_f, double vmin, double vmax,
                                        const JhmiConsts& C, int B) {
  const float p = (v - vmin_f) * vinv_f;
  const float t = fmaf(p - C.origin_f, C.inv_spacing_f, 0.5f);
  float fl = floorf(t);
  if (fabsf(t - rintf(t)) < 1e-4f || !(t == t)) {
    // near a boundary: the reference's FP64 arithmetic
    const double pd = ((double)v - vmin) / (vmax - vmin);
    fl = (float)floor((pd - C.origin) * C.inv_spacing + 0.5);
    if (!(pd == pd)) return -1;
  }
  const int b = (int)fl;
  return (b >= 0 && b < B) ? b : -1;
}

// k_jhmi_pass1: histogram counts in shared memory (u32), the cache (m, g) for pass 2.
template <int GRAD, int TK = kMapAffine>
__device__ __forceinline__ void jhmi_pass1_body(const EvalArgs& a, const JhmiConsts* __restrict__ gC, VGrid vg) {
  extern __shared__ unsigned hist_s[];
  __shared__ EvalConsts K;
  __shared__ JhmiConsts C;
  const int B = a.bins;
  for (int k = threadIdx.x; k < B * B; k += blockDim.x) hist_s[k] = 0u;
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  load_consts(a.consts, K);
  {
    const unsigned* src = reinterpret_cast<const unsigned*>(gC);
    unsigned* dst = reinterpret_cast<unsigned*>(&C);
    for (int k = threadIdx.x; k < (int)(sizeof(JhmiConsts) / 4); k += blockDim.x) dst[k] = __ldg(src + k);
  }
  __syncthreads();
  unsigned nv = 0;
  const int64_t stride = (int64_t)vg.n * blockDim.x;
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  int64_t i = (int64_t)vg.b * blockDim.x + threadIdx.x;
  float4 s_next = i < a.n ? __ldcs(a.samples + i) : zero;
  for (; i < a.n; i += stride) {
    // the next record travels while this sample is formed
    const float4 s = s_next;
    s_next = i + stride < a.n ? __ldcs(a.samples + i + stride) : zero;
    float m = 0.f;
    float3 g = make_float3(0.f, 0.f, 0.f);
    unsigned voxel;
    const bool ok = eval_moving<GRAD>(a, sample_pos<TK>(a, K, s, i, voxel), a.with_derivative != 0, m, g);
    if (TK != kMapAffine) g = field_grad(K, g);
    if (a.with_derivative)
      __stcs(a.cache + i, ok ? make_float4(m, g.x, g.y, g.z) : make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f));
    if (!ok) continue;
    const int fb = jhmi_bin(s.w, C.fmin_f, C.finv_f, C.fmin, C.fmax, C, B);
    const int mb = jhmi_bin(m, C.mmin_f, C.minv_f, C.mmin, C.mmax, C, B);
    if (fb < 0 || mb < 0) continue;
    atomicAdd(&hist_s[fb + B * mb], 1u);
    ++nv;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < B * B; k += blockDim.x) {
    const unsigned h = hist_s[k];
    if (h) atomicAdd(&a.hist[k], (unsigned long long)h);
  }
  block_count(nv, a.acc_n);
}

template <int GRAD>
__global__ void __launch_bounds__(kBlock) k_jhmi_pass1(EvalArgs a, const JhmiConsts* C) {
  jhmi_pass1_body<GRAD>(a, C, hw_grid());
}

// One thread per output: out[x] = sum_k c[k] in[clamp(x + k - r)] along `dir`
// (0: the fixed index, contiguous; 1: the moving index), ZeroFluxNeumann border.
__device__ __forceinline__ void jhmi_gauss_pass(const double* in, double* out, int B, int dir, const JhmiConsts& C) {
  const int r = C.radius;
  for (int q = threadIdx.x; q < B * B; q += blockDim.x) {
    const int i = q % B, j = q / B;
    double s = 0.0;
    for (int k = 0; k <= 2 * r; ++k) {
      int t = (dir == 0 ? i : j) + k - r;
      t = t < 0 ? 0 : (t > B - 1 ? B - 1 : t);
      s += C.kernel[k] * (dir == 0 ? in[t + B * j] : in[i + B * t]);
    }
    out[q] = s;
  }
}

// k_jhmi_finalize (kJhmiFinalizeBlocks blocks).  Writes the smoothed PDF (FP64, pdf_out; FP32 and the
// FP32 moving marginal into the pratio table), the value, the count and the status.
__global__ void __launch_bounds__(kBlock) k_jhmi_finalize(EvalArgs a, const JhmiConsts* gC) {
  extern __shared__ double plane[];  // 2 B^2 doubles, then 2 B (marginals)
  __shared__ JhmiConsts C;
  __shared__ double red[kBlock / 32];
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  const int B = a.bins;
  {
    const unsigned* src = reinterpret_cast<const unsigned*>(gC);
    unsigned* dst = reinterpret_cast<unsigned*>(&C);
    for (int k = threadIdx.x; k < (int)(sizeof(JhmiConsts) / 4); k += blockDim.x) dst[k] = __ldg(src + k);
  }
  double* p0 = plane;
  double* p1 = plane + B * B;
  double* fm = plane + 2 * B * B;
  double* mm = fm + B;
  const unsigned long long N = __ldcg(a.acc_n);
  const double invN = N > 0 ? 1.0 / (double)N : 0.0;
  for (int k = threadIdx.x; k < B * B; k += blockDim.x) p0[k] = (double)__ldcg(&a.hist[k]) * invN;
  __syncthreads();
  double* pdf = p0;
  if (C.radius > 0) {  // DiscreteGaussianImageFilter: the moving axis, then the fixed axis
    jhmi_gauss_pass(p0, p1, B, 1, C);
    __syncthreads();
    jhmi_gauss_pass(p1, p0, B, 0, C);
    __syncthreads();
  }
  // marginals: moving = sum over the fixed index, fixed = sum over the moving index;
  // one warp per marginal bin: lane-strided loads, a fixed XOR tree (short FP64 chains)
  {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int t = warp; t < 2 * B; t += nw) {
      double s = 0.0;
      if (t < B) {
        for (int i = lane; i < B; i += 32) s += pdf[i + B * t];
      } else {
        for (int j = lane; j < B; j += 32) s += pdf[(t - B) + B * j];
      }
      s = warp_sum_d(s);
      if (lane == 0) (t < B ? mm[t] : fm[t - B]) = s;
    }
  }
  __syncthreads();
  // the value over this block's share of the bins: per-thread sums in a fixed bin
  // order, a fixed XOR tree per warp, the warps in order; the blocks' partials are
  // added in block order by the last block.  Each block repeats the (small) PDF,
  // smoothing and marginals so the FP64 logs spread over kJhmiFinalizeBlocks SMs.
  const int q0 = (int)((long long)B * B * blockIdx.x / gridDim.x);
  const int q1 = (int)((long long)B * B * (blockIdx.x + 1) / gridDim.x);
  double s = 0.0;
  for (int q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
    const int i = q % B, j = q / B;
    const double denom = fm[i] * mm[j];
    const double pxy = pdf[q];
    double local = 0.0;
    if (fabs(denom) > DBL_EPSILON && pxy / denom > DBL_EPSILON) local = pxy * log(pxy / denom);
    s += local;
    a.pdf_out[q] = pxy;
    a.pratio[q] = (float)pxy;
  }
  s = warp_sum_d(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  if (blockIdx.x == 0)
    for (int j = threadIdx.x; j < B; j += blockDim.x) a.pratio[B * B + j] = (float)mm[j];
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    a.part[blockIdx.x] = t;
  }
  if (!last_block(a.tickets + kTicketFinalize)) return;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)gridDim.x; ++k) t += __ldcg(&a.part[k]);
    a.out[1] = (double)N;
    if (N == 0) {  // GetValue: VerifyNumberOfValidPoints, a warning and the maximum value
      a.out[0] = DBL_MAX;
      *a.status = GB_ERR_NO_VALID_POINTS;
    } else {
      a.out[0] = -1.0 * t / 0.69314718055994530942;  // / log(2): bits
      *a.status = GB_OK;
    }
  }
}

// Bilinear value of the FP32 PDF table at a continuous index (LinearInterpolateImageFunction, 2-D).
__device__ __forceinline__ float jhmi_interp2(const float* t, int B, float cx, float cy) {
  int x0 = (int)floorf(cx), y0 = (int)floorf(cy);
  x0 = x0 < 0 ? 0 : x0;
  y0 = y0 < 0 ? 0 : y0;
  float dx = cx - (float)x0, dy = cy - (float)y0;
  int x1 = x0 + 1 <= B - 1 ? x0 + 1 : x0, y1 = y0 + 1 <= B - 1 ? y0 + 1 : y0;
  if (!(dx > 0.f)) { dx = 0.f; x1 = x0; }
  if (!(dy > 0.f)) { dy = 0.f; y1 = y0; }
  const float v00 = t[x0 + B * y0], v10 = t[x1 + B * y0], v01 = t[x0 + B * y1], v11 = t[x1 + B * y1];
  return lerp(lerp(v00, v10, dx), lerp(v01, v11, dx), dy);
}

__device__ __forceinline__ float jhmi_interp1(const float* t, int B, float c) {
  int x0 = (int)floorf(c);
  x0 = x0 < 0 ? 0 : x0;
  float d = c - (float)x0;
  const int x1 = x0 + 1 <= B - 1 ? x0 + 1 : x0;
  if (!(d > 0.f)) return t[x0];
  return lerp(t[x0], t[x1], d);
}

// One derivative point: false for an invalid or out-of-range sample; else sf, the
// clamped log-slope difference of the joint PDF and the moving marginal along the
// moving axis over (log 2 * moving range).
__device__ __forceinline__ bool jhmi_scaling(const JhmiConsts& C, const float* pdf, const float* mm, int B, float f,
                                             float m, float mlo, float mhi, float max_slope, float inv_scale,
                                             float& sf) {
  if (!(m == m)) return false;            // invalid sample
  if (m < mlo || m > mhi) return false;   // outside the moving range
  const float sp = C.spacing_f;
  const float pa = (f - C.fmin_f) * C.finv_f, pb = (m - C.mmin_f) * C.minv_f;
  const float ca = (pa - C.origin_f) * C.inv_spacing_f, cb = (pb - C.origin_f) * C.inv_spacing_f;
  if (!(ca >= -0.5f && ca < (float)B - 0.5f && cb >= -0.5f && cb < (float)B - 0.5f)) return false;
  const float jv = jhmi_interp2(pdf, B, ca, cb);
  float l = pb - 0.5f * sp, r = pb + 0.5f * sp;
  l = fminf(fmaxf(l, sp), 1.f);
  r = fminf(fmaxf(r, sp), 1.f);
  float dj = 0.f, dm = 0.f;
  const float delta = r - l;
  if (delta > 0.f) {
    const float cl = (l - C.origin_f) * C.inv_spacing_f, cr = (r - C.origin_f) * C.inv_spacing_f;
    // fast FP32 divisions (within 2 ulp; the divisors are spacing-sized or above 1e-16)
    dj = __fdividef(jhmi_interp2(pdf, B, ca, cr) - jhmi_interp2(pdf, B, ca, cl), delta);
    dm = __fdividef(jhmi_interp1(mm, B, cr) - jhmi_interp1(mm, B, cl), delta);
  }
  const float mv = jhmi_interp1(mm, B, cb);
  sf = 0.f;
  if (jv > 1e-16f && mv > 1e-16f) {
    const float t1 = fminf(fmaxf(__fdividef(dj, jv), -max_slope), max_slope);
    const float t2 = fminf(fmaxf(__fdividef(dm, mv), -max_slope), max_slope);
    sf = (t1 - t2) * inv_scale;
  }
  return true;
}

// The derivative passes' scalars: the slope clamp -log(1e-16) / spacing, the scale
// 1 / (log 2 (max - min)) and the moving range (exact: the true min / max are float
// values).  FP64, formed by one thread and shared (a block's worth of FP64 divisions
// would cost microseconds at GB300's FP64 rate); the caller has synchronized on C.
__device__ __forceinline__ void jhmi_pass2_scalars(const JhmiConsts& C, float& max_slope, float& inv_scale,
                                                   float& mlo, float& mhi) {
  __shared__ float sc_s[4];
  if (threadIdx.x == 0) {
    sc_s[0] = (float)(36.841361487904734 / C.spacing);
    sc_s[1] = (float)(1.0 / (0.69314718055994530942 * (C.mmax - C.mmin)));
    sc_s[2] = (float)C.mmin;
    sc_s[3] = (float)C.mmax;
  }
  __syncthreads();
  max_slope = sc_s[0];
  inv_scale = sc_s[1];
  mlo = sc_s[2];
  mhi = sc_s[3];
}

// k_jhmi_pass2: the derivative.  Dynamic shared memory: the B^2 + B FP32 tables.
template <int GRAD>
__device__ __forceinline__ void jhmi_pass2_body(const EvalArgs& a, const JhmiConsts* __restrict__ gC, VGrid vg) {
  extern __shared__ float tab[];
  __shared__ EvalConsts K;
  __shared__ JhmiConsts C;
  __shared__ float red[kBlock / 32][13];
  __shared__ double blk[13], fin[13];
  const int B = a.bins;
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  for (int k = threadIdx.x; k < B * B + B; k += blockDim.x) tab[k] = __ldcg(&a.pratio[k]);
  load_consts(a.consts, K);
  {
    const unsigned* src = reinterpret_cast<const unsigned*>(gC);
    unsigned* dst = reinterpret_cast<unsigned*>(&C);
    for (int k = threadIdx.x; k < (int)(sizeof(JhmiConsts) / 4); k += blockDim.x) dst[k] = __ldg(src + k);
  }
  __syncthreads();
  const float* pdf = tab;
  const float* mm = tab + B * B;
  float max_slope, inv_scale, mlo, mhi;
  jhmi_pass2_scalars(C, max_slope, inv_scale, mlo, mhi);
  float acc[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) acc[k] = 0.f;
  unsigned nv = 0;
  const int64_t stride = (int64_t)vg.n * blockDim.x;
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  int64_t i = (int64_t)vg.b * blockDim.x + threadIdx.x;
  float4 cc_next = i < a.n ? __ldcs(a.cache + i) : zero;
  float4 s_next = i < a.n ? __ldcs(a.samples + i) : zero;
  for (; i < a.n; i += stride) {
    // the next cache entry and record travel while this sample is formed
    const float4 cc = cc_next;
    const float4 s = s_next;
    cc_next = i + stride < a.n ? __ldcs(a.cache + i + stride) : zero;
    s_next = i + stride < a.n ? __ldcs(a.samples + i + stride) : zero;
    float sf;
    if (!jhmi_scaling(C, pdf, mm, B, s.w, cc.x, mlo, mhi, max_slope, inv_scale, sf)) continue;
    ++nv;
    const float3 v = jac_vec(K, s.x, s.y, s.z);
    const float t0 = sf * cc.y, t1 = sf * cc.z, t2 = sf * cc.w;
    acc[0] = fmaf(t0, v.x, acc[0]); acc[1] = fmaf(t0, v.y, acc[1]); acc[2] = fmaf(t0, v.z, acc[2]);
    acc[3] = fmaf(t1, v.x, acc[3]); acc[4] = fmaf(t1, v.y, acc[4]); acc[5] = fmaf(t1, v.z, acc[5]);
    acc[6] = fmaf(t2, v.x, acc[6]); acc[7] = fmaf(t2, v.y, acc[7]); acc[8] = fmaf(t2, v.z, acc[8]);
    acc[9] += t0; acc[10] += t1; acc[11] += t2;
  }
  KahanF kacc[13];
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    kacc[k].s = acc[k];
    kacc[k].c = 0.f;
  }
  // the valid count rides along as the 13th sum (exact in FP32 per thread, FP64 across blocks)
  kacc[12].s = (float)nv;
  kacc[12].c = 0.f;
  block_sums<13>(kacc, red, blk);
  if (!grid_sums<13>(blk, a.part + kPartPass2, a.grp, a.tickets + kTicketPass2, fin, vg)) return;
  if (threadIdx.x < 32) {
    // one derivative entry per lane (the FP64 divisions side by side)
    const int lane = threadIdx.x;
    const double N = fin[12];
    const int P = a.nparams;
    // VerifyNumberOfValidPoints: with no valid point a warning, value max, zero derivative
    for (int p = lane; p < P; p += 32) a.out[2 + p] = N == 0.0 ? 0.0 : fin[p] / N;
    if (lane == 0) {
      a.out[1] = N;
      if (N == 0.0) a.out[0] = DBL_MAX;
      *a.status = N == 0.0 ? GB_ERR_NO_VALID_POINTS : GB_OK;
    }
  }
}

template <int GRAD>
__global__ void __launch_bounds__(kBlock) k_jhmi_pass2(EvalArgs a, const JhmiConsts* C) {
  jhmi_pass2_body<GRAD>(a, C, hw_grid());
}

// ---------------------------------------------------------------------------
// B-spline and [affine, B-spline] composite transforms: pass 1 with the B-spline
// position (nodes staged in shared memory when they fit), caching (m, M^T g);
// the same finalize; pass 2 turns each cached sample into its derivative factor
// a_s = sf M^T g (zero for an invalid sample or one outside the B-spline's valid
// region) in place, counts the derivative points, and leaves the sparse Jacobian
// sums to the B-spline chunk and parameter kernels (MeanSquares form: sum / count).

__device__ __forceinline__ void load_jhmi(const JhmiConsts* __restrict__ gC, JhmiConsts& C) {
  const unsigned* src = reinterpret_cast<const unsigned*>(gC);
  unsigned* dst = reinterpret_cast<unsigned*>(&C);
  for (int k = threadIdx.x; k < (int)(sizeof(JhmiConsts) / 4); k += blockDim.x) dst[k] = __ldg(src + k);
}

// Dynamic shared memory: the B^2 histogram, then (16-byte aligned) the nodes.
__host__ __device__ inline size_t jhmi_bspline_node_offset(int B) { return ((size_t)4 * B * B + 15) / 16 * 16; }

template <int GRAD, bool SMEM>
__global__ void __launch_bounds__(kBlock) k_jhmi_pass1_bspline(EvalArgs a, const JhmiConsts* gC) {
  extern __shared__ __align__(16) unsigned char smem_jb[];
  unsigned* hist_s = reinterpret_cast<unsigned*>(smem_jb);
  __shared__ EvalConsts K;
  __shared__ JhmiConsts C;
  const int B = a.bins;
  for (int k = threadIdx.x; k < B * B; k += blockDim.x) hist_s[k] = 0u;
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  load_consts(a.consts, K);
  load_jhmi(gC, C);
  const float4* nodes = stage_nodes<SMEM>(a, reinterpret_cast<float4*>(smem_jb + jhmi_bspline_node_offset(B)));
  __syncthreads();
  unsigned nv = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    const float4 s = __ldcs(a.samples + i);
    const float4 su = __ldcs(a.sup + i);
    bool has_jac;
    const DFPos p = bspline_position(K, nodes, a, s, su, has_jac);
    float m = 0.f;
    float3 g = make_float3(0.f, 0.f, 0.f);
    const bool ok = eval_moving<GRAD>(a, p, a.with_derivative != 0 && has_jac, m, g);
    if (a.with_derivative) {
      const float3 gm = has_jac ? grad_map(K, g) : make_float3(0.f, 0.f, 0.f);
      __stcs(a.cache + i, ok ? make_float4(m, gm.x, gm.y, gm.z) : make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f));
    }
    if (!ok) continue;
    const int fb = jhmi_bin(s.w, C.fmin_f, C.finv_f, C.fmin, C.fmax, C, B);
    const int mb = jhmi_bin(m, C.mmin_f, C.minv_f, C.mmin, C.mmax, C, B);
    if (fb < 0 || mb < 0) continue;
    atomicAdd(&hist_s[fb + B * mb], 1u);
    ++nv;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < B * B; k += blockDim.x) {
    const unsigned h = hist_s[k];
    if (h) atomicAdd(&a.hist[k], (unsigned long long)h);
  }
  block_count(nv, a.acc_n);
}

// Pass 2 for the B-spline: a_s into the cache, the count into fmarg[0] (a spare
// accumulator here); the last block makes the count the one the parameter kernel
// divides by, and sets the status (no derivative point: a warning, value max).
__global__ void __launch_bounds__(kBlock) k_jhmi_pass2_bspline(EvalArgs a, const JhmiConsts* gC) {
  extern __shared__ float tab[];
  __shared__ JhmiConsts C;
  const int B = a.bins;
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  for (int k = threadIdx.x; k < B * B + B; k += blockDim.x) tab[k] = __ldcg(&a.pratio[k]);
  load_jhmi(gC, C);
  __syncthreads();
  float max_slope, inv_scale, mlo, mhi;
  jhmi_pass2_scalars(C, max_slope, inv_scale, mlo, mhi);
  unsigned nv = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    const float4 cc = __ldcg(a.cache + i);
    const float f = __ldcs(&a.samples[i].w);
    float sf;
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if (jhmi_scaling(C, tab, tab + B * B, B, f, cc.x, mlo, mhi, max_slope, inv_scale, sf)) {
      ++nv;
      out = make_float4(sf * cc.y, sf * cc.z, sf * cc.w, 1.f);
    }
    __stcg(a.cache + i, out);
  }
  block_count(nv, a.fmarg);
  if (!last_block(a.tickets + kTicketPass2)) return;
  if (threadIdx.x == 0) {
    const unsigned long long N = __ldcg(a.fmarg);
    *a.acc_n = N;
    a.out[1] = (double)N;
    if (N == 0) {
      a.out[0] = DBL_MAX;
      *a.status = GB_ERR_NO_VALID_POINTS;
    } else {
      *a.status = GB_OK;
    }
  }
}

// ---------------------------------------------------------------------------
// Displacement fields (local support): pass 1 with the field's positions, caching
// (m, M^T g); the same finalize; pass 2 stores each derivative point's block
// sf M^T g at its voxel, not averaged (the base threader's local branch), and the
// last block sets the count and status.

template <int GRAD, int TK>
__global__ void __launch_bounds__(kBlock) k_jhmi_pass1_field(EvalArgs a, const JhmiConsts* C) {
  jhmi_pass1_body<GRAD, TK>(a, C, hw_grid());
}

template <int TK>
__global__ void __launch_bounds__(kBlock) k_jhmi_pass2_field(EvalArgs a, const JhmiConsts* gC) {
  extern __shared__ float tab[];
  __shared__ JhmiConsts C;
  const int B = a.bins;
  griddep_wait();
  if (halted(a)) return;
  griddep_launch_dependents();
  for (int k = threadIdx.x; k < B * B + B; k += blockDim.x) tab[k] = __ldcg(&a.pratio[k]);
  load_jhmi(gC, C);
  __syncthreads();
  float max_slope, inv_scale, mlo, mhi;
  jhmi_pass2_scalars(C, max_slope, inv_scale, mlo, mhi);
  unsigned nv = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    const float4 cc = __ldcs(a.cache + i);
    const float4 s = __ldcs(a.samples + i);
    const unsigned voxel = TK == kMapFieldDense
                               ? (unsigned)s.x + (unsigned)a.vnx * ((unsigned)s.y + (unsigned)a.vny * (unsigned)s.z)
                               : __ldg(a.voff + i);
    float sf = 0.f;
    const bool ok = jhmi_scaling(C, tab, tab + B * B, B, s.w, cc.x, mlo, mhi, max_slope, inv_scale, sf);
    nv += ok ? 1u : 0u;
    field_store<TK>(a, voxel, ok, sf, make_float3(cc.y, cc.z, cc.w));
  }
  block_count(nv, a.fmarg);
  if (!last_block(a.tickets + kTicketPass2)) return;
  if (threadIdx.x == 0) {
    const unsigned long long N = __ldcg(a.fmarg);
    a.out[1] = (double)N;
    if (N == 0) {  // a warning, value max; no block was stored
      a.out[0] = DBL_MAX;
      *a.status = GB_ERR_NO_VALID_POINTS;
    } else {
      *a.status = GB_OK;
    }
  }
}

}  // namespace gb
