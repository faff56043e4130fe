// gb_filters.cu -- device forms of the per-level image filters of the
// registration method and of the metric's default moving-gradient filter:
// recursive-Gaussian smoothing, recursive-Gaussian gradient, shrink geometry.
//
// Reference semantics (paths relative to ITK's Modules/):
//   RecursiveGaussianImageFilter coefficients   Filtering/Smoothing/include/itkRecursiveGaussianImageFilter.hxx:56-300
//   RecursiveSeparableImageFilter line filter   Filtering/ImageFilterBase/include/itkRecursiveSeparableImageFilter.hxx:60-150
//   SmoothingRecursiveGaussianImageFilter       Filtering/Smoothing/include/itkSmoothingRecursiveGaussianImageFilter.hxx
//   GradientRecursiveGaussianImageFilter        Filtering/ImageGradient/include/itkGradientRecursiveGaussianImageFilter.hxx:160-270
//   ShrinkImageFilter geometry                  Filtering/ImageGrid/include/itkShrinkImageFilter.hxx:230-290
//   metric's default gradient filter settings   Registration/Metricsv4/include/itkImageToImageMetricv4.hxx:488-503
//
// Each 1-D pass is one thread per image line: the causal recursion runs
// forward and is stored, the anticausal recursion runs backward and is added,
// both with the reference's edge-extension start-up.  Lines along y and z are
// adjacent in x across the threads of a warp, so their loads coalesce; lines
// along x read one element per thread per step and lean on L1.  The
// coefficients come from FP64 on the host; the recursions run in FP32 (the
// reference filters in double and, for float images, stores float between the
// smoothing passes).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "gb_device.cuh"
#include "gb_internal.h"

namespace gb {

// IIR coefficients of one pass: N0..N3, D1..D4, M1..M4, BN1..BN4, BM1..BM4.
struct RGCoef {
  double n[4], d[4], m[4], bn[4], bm[4];
};
struct RGCoefF {
  float n[4], d[4], m[4], bn[4], bm[4];
};

// Deriche-style recursive Gaussian with the parameters of Farneback and
// Westin ("Improving Deriche-style recursive Gaussian filters", Table 3) and
// the reference's normalizations: order 0 (smoothing) or 1 (first derivative).
static int rg_setup(double sigma, double spacing, int order, bool normalize_across_scale, RGCoef& c) {
  double direction = 1.0;
  if (spacing < 0.0) {
    direction = -1.0;
    spacing = -spacing;
  }
  if (spacing < 1e-8 || !(sigma > 0.0) || (order != 0 && order != 1)) return GB_ERR_BAD_ARG;
  const double sd = sigma / spacing;  // sigma in voxels
  // exponential-series parameters: A, B per order, W, L per pair
  const double A1 = order == 0 ? 1.3530 : -0.6724, B1 = order == 0 ? 1.8151 : -3.4327;
  const double A2 = order == 0 ? -0.3531 : 0.6724, B2 = order == 0 ? 0.0902 : 0.6100;
  const double W1 = 0.6681, L1 = -1.3932, W2 = 2.0787, L2 = -1.3732;
  const double cos1 = std::cos(W1 / sd), cos2 = std::cos(W2 / sd);
  const double sin1 = std::sin(W1 / sd), sin2 = std::sin(W2 / sd);
  const double e1 = std::exp(L1 / sd), e2 = std::exp(L2 / sd);
  // denominator: poles of the two second-order sections
  c.d[3] = e1 * e1 * e2 * e2;
  c.d[2] = -2 * cos1 * e1 * e2 * e2;
  c.d[2] += -2 * cos2 * e2 * e1 * e1;
  c.d[1] = 4 * cos2 * cos1 * e1 * e2;
  c.d[1] += e1 * e1 + e2 * e2;
  c.d[0] = -2 * (e2 * cos2 + e1 * cos1);
  const double SD = 1.0 + c.d[0] + c.d[1] + c.d[2] + c.d[3];
  const double DD = c.d[0] + 2 * c.d[1] + 3 * c.d[2] + 4 * c.d[3];
  // numerator of the causal part
  c.n[0] = A1 + A2;
  c.n[1] = e2 * (B2 * sin2 - (A2 + 2 * A1) * cos2);
  c.n[1] += e1 * (B1 * sin1 - (A1 + 2 * A2) * cos1);
  c.n[2] = (A1 + A2) * cos2 * cos1;
  c.n[2] -= B1 * cos2 * sin1 + B2 * cos1 * sin2;
  c.n[2] *= 2 * e1 * e2;
  c.n[2] += A2 * e1 * e1 + A1 * e2 * e2;
  c.n[3] = e2 * e1 * e1 * (B2 * sin2 - A2 * cos2);
  c.n[3] += e1 * e2 * e2 * (B1 * sin1 - A1 * cos1);
  const double SN = c.n[0] + c.n[1] + c.n[2] + c.n[3];
  const double DN = c.n[1] + 2 * c.n[2] + 3 * c.n[3];
  // normalization: unit gain (order 0) / unit slope response (order 1, times sigma across scales)
  double alpha;
  double scale = 1.0;
  if (order == 0) {
    alpha = 2 * SN / SD - c.n[0];
  } else {
    if (normalize_across_scale) scale = sigma;
    alpha = 2 * (SN * DD - DN * SD) / (SD * SD) * direction;
  }
  for (int k = 0; k < 4; ++k) c.n[k] *= scale / alpha;
  // anticausal numerator: symmetric for order 0, antisymmetric for order 1
  const double sgn = order == 0 ? 1.0 : -1.0;
  c.m[0] = sgn * (c.n[1] - c.d[0] * c.n[0]);
  c.m[1] = sgn * (c.n[2] - c.d[1] * c.n[0]);
  c.m[2] = sgn * (c.n[3] - c.d[2] * c.n[0]);
  c.m[3] = sgn * (-c.d[3] * c.n[0]);
  // edge-extension start-up terms
  const double sn = c.n[0] + c.n[1] + c.n[2] + c.n[3];
  const double sm = c.m[0] + c.m[1] + c.m[2] + c.m[3];
  const double sdd = 1.0 + c.d[0] + c.d[1] + c.d[2] + c.d[3];
  for (int k = 0; k < 4; ++k) {
    c.bn[k] = c.d[k] * sn / sdd;
    c.bm[k] = c.d[k] * sm / sdd;
  }
  return GB_OK;
}

static RGCoefF to_float(const RGCoef& c) {
  RGCoefF f;
  for (int k = 0; k < 4; ++k) {
    f.n[k] = (float)c.n[k];
    f.d[k] = (float)c.d[k];
    f.m[k] = (float)c.m[k];
    f.bn[k] = (float)c.bn[k];
    f.bm[k] = (float)c.bm[k];
  }
  return f;
}

// One pass along an axis.  Line l = (j1, j2) starts at j1 * s1 + j2 * s2 and has
// ln elements `step` apart.  out = (causal + anticausal) * scale; in != out.
__global__ void __launch_bounds__(128) k_rg_lines(const float* __restrict__ in, float* __restrict__ out, RGCoefF c,
                                                  int64_t ln, int64_t step, int64_t n1, int64_t s1, int64_t n2,
                                                  int64_t s2, float scale) {
  const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= n1 * n2) return;
  const float* x = in + (id % n1) * s1 + (id / n1) * s2;
  float* y = out + (id % n1) * s1 + (id / n1) * s2;
  // causal: y_i = sum_k n_k x_{i-k} - sum_k d_k y_{i-k}; before the line x = x_0 and
  // the feedback of the missing outputs is x_0 bn_k
  const float v1 = __ldg(x);
  const float x1 = __ldg(x + step), x2 = __ldg(x + 2 * step), x3 = __ldg(x + 3 * step);
  float o0 = v1 * c.n[0] + v1 * c.n[1] + v1 * c.n[2] + v1 * c.n[3];
  o0 -= v1 * c.bn[0] + v1 * c.bn[1] + v1 * c.bn[2] + v1 * c.bn[3];
  float o1 = x1 * c.n[0] + v1 * c.n[1] + v1 * c.n[2] + v1 * c.n[3];
  o1 -= o0 * c.d[0] + v1 * c.bn[1] + v1 * c.bn[2] + v1 * c.bn[3];
  float o2 = x2 * c.n[0] + x1 * c.n[1] + v1 * c.n[2] + v1 * c.n[3];
  o2 -= o1 * c.d[0] + o0 * c.d[1] + v1 * c.bn[2] + v1 * c.bn[3];
  float o3 = x3 * c.n[0] + x2 * c.n[1] + x1 * c.n[2] + v1 * c.n[3];
  o3 -= o2 * c.d[0] + o1 * c.d[1] + o0 * c.d[2] + v1 * c.bn[3];
  y[0] = o0;
  y[step] = o1;
  y[2 * step] = o2;
  y[3 * step] = o3;
  float xm1 = x3, xm2 = x2, xm3 = x1;        // x_{i-1}, x_{i-2}, x_{i-3}
  float ym1 = o3, ym2 = o2, ym3 = o1, ym4 = o0;  // y_{i-1} .. y_{i-4}
  for (int64_t i = 4; i < ln; ++i) {
    const float xi = __ldg(x + i * step);
    float o = xi * c.n[0] + xm1 * c.n[1] + xm2 * c.n[2] + xm3 * c.n[3];
    o -= ym1 * c.d[0] + ym2 * c.d[1] + ym3 * c.d[2] + ym4 * c.d[3];
    y[i * step] = o;
    xm3 = xm2;
    xm2 = xm1;
    xm1 = xi;
    ym4 = ym3;
    ym3 = ym2;
    ym2 = ym1;
    ym1 = o;
  }
  // anticausal: z_{i-1} = sum_k m_k x_{i-1+k} - sum_k d_k z_{i-1+k}, x = x_{ln-1} beyond the end
  const int64_t L = ln - 1;
  const float v2 = __ldg(x + L * step);
  const float a1 = __ldg(x + (L - 1) * step), a2 = __ldg(x + (L - 2) * step);
  float z0 = v2 * c.m[0] + v2 * c.m[1] + v2 * c.m[2] + v2 * c.m[3];  // z_{L}
  z0 -= v2 * c.bm[0] + v2 * c.bm[1] + v2 * c.bm[2] + v2 * c.bm[3];
  float z1 = v2 * c.m[0] + v2 * c.m[1] + v2 * c.m[2] + v2 * c.m[3];  // z_{L-1}
  z1 -= z0 * c.d[0] + v2 * c.bm[1] + v2 * c.bm[2] + v2 * c.bm[3];
  float z2 = a1 * c.m[0] + v2 * c.m[1] + v2 * c.m[2] + v2 * c.m[3];  // z_{L-2}
  z2 -= z1 * c.d[0] + z0 * c.d[1] + v2 * c.bm[2] + v2 * c.bm[3];
  float z3 = a2 * c.m[0] + a1 * c.m[1] + v2 * c.m[2] + v2 * c.m[3];  // z_{L-3}
  z3 -= z2 * c.d[0] + z1 * c.d[1] + z0 * c.d[2] + v2 * c.bm[3];
  y[L * step] = (y[L * step] + z0) * scale;
  y[(L - 1) * step] = (y[(L - 1) * step] + z1) * scale;
  y[(L - 2) * step] = (y[(L - 2) * step] + z2) * scale;
  y[(L - 3) * step] = (y[(L - 3) * step] + z3) * scale;
  // z_{i-1} for i = L-3 .. 1 from x_i, x_{i+1}, x_{i+2}, x_{i+3} and z_i .. z_{i+3}
  float r1 = a2, r2 = a1, r3 = v2;               // x_{i+1}, x_{i+2}, x_{i+3} at i = L - 3
  float zp1 = z3, zp2 = z2, zp3 = z1, zp4 = z0;  // z_i, z_{i+1}, z_{i+2}, z_{i+3}
  for (int64_t i = L - 3; i > 0; --i) {
    const float xi = __ldg(x + i * step);
    float z = xi * c.m[0] + r1 * c.m[1] + r2 * c.m[2] + r3 * c.m[3];
    z -= zp1 * c.d[0] + zp2 * c.d[1] + zp3 * c.d[2] + zp4 * c.d[3];
    y[(i - 1) * step] = (y[(i - 1) * step] + z) * scale;
    r3 = r2;
    r2 = r1;
    r1 = xi;
    zp4 = zp3;
    zp3 = zp2;
    zp2 = zp1;
    zp1 = z;
  }
}

static cudaError_t rg_pass(cudaStream_t st, const float* in, float* out, const int64_t size[3], int axis,
                           const RGCoef& c, float scale) {
  const int64_t ln = size[axis];
  const int64_t step = axis == 0 ? 1 : (axis == 1 ? size[0] : size[0] * size[1]);
  // the two other axes, the faster-varying one first (x whenever it is not the filtered axis)
  const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
  const int64_t s1 = a1 == 0 ? 1 : size[0], s2 = a2 == 1 ? size[0] : size[0] * size[1];
  const int64_t lines = size[a1] * size[a2];
  const unsigned blocks = (unsigned)((lines + 127) / 128);
  k_rg_lines<<<blocks, 128, 0, st>>>(in, out, to_float(c), ln, step, size[a1], s1, size[a2], s2, scale);
  return cudaGetLastError();
}

// SmoothingRecursiveGaussianImageFilter: zero order along z, then x, then y.
// t1, t2: scratch images of the same size (in may equal out).
int smooth_rg_device(cudaStream_t st, const float* in, float* out, float* t1, float* t2, const int64_t size[3],
                     const double spacing[3], const double sigma[3]) {
  for (int d = 0; d < 3; ++d)
    if (size[d] < 4)
      return fail(GB_ERR_BAD_ARG, "The number of pixels along dimension " + std::to_string(d) +
                                      " is less than 4. This filter requires a minimum of four pixels along the "
                                      "dimension to be processed.");
  RGCoef c;
  const int order[3] = {2, 0, 1};
  const float* src = in;
  float* dst[3] = {t1, t2, out};
  for (int p = 0; p < 3; ++p) {
    const int ax = order[p];
    if (rg_setup(sigma[ax], spacing[ax], 0, false, c) != GB_OK) return fail(GB_ERR_BAD_ARG, "sigma must be > 0");
    cudaError_t e = rg_pass(st, src, dst[p], size, ax, c, 1.f);
    if (e != cudaSuccess) return fail(GB_ERR_CUDA, std::string("smoothing pass: ") + cudaGetErrorString(e));
    src = dst[p];
  }
  return GB_OK;
}

// (value, D (gx, gy, gz)) per voxel, the gradient in physical units.
__global__ void k_pack_gradient(const float* __restrict__ v, const float* __restrict__ gx,
                                const float* __restrict__ gy, const float* __restrict__ gz, int64_t n, float d00,
                                float d01, float d02, float d10, float d11, float d12, float d20, float d21,
                                float d22, float4* __restrict__ out4, float* __restrict__ out3) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float a = gx[i], b = gy[i], c = gz[i];
  const float px = fmaf(d00, a, fmaf(d01, b, d02 * c));
  const float py = fmaf(d10, a, fmaf(d11, b, d12 * c));
  const float pz = fmaf(d20, a, fmaf(d21, b, d22 * c));
  if (out4) out4[i] = make_float4(v[i], px, py, pz);
  if (out3) {
    out3[3 * i] = px;
    out3[3 * i + 1] = py;
    out3[3 * i + 2] = pz;
  }
}

// GradientRecursiveGaussianImageFilter: component d = first order along d and
// zero order along the other axes, / spacing[d], then the direction matrix.
// The zero-order x pass and the y passes are shared between components.
// Writes float4 (value, gradient) and/or xyz float triplets.
int gradient_rg_device(cudaStream_t st, const float* in, const int64_t size[3], const double spacing[3],
                       const double direction[9], double sigma, bool normalize_across_scale, bool use_direction,
                       float4* out4, float* out3) {
  for (int d = 0; d < 3; ++d)
    if (size[d] < 4)
      return fail(GB_ERR_BAD_ARG, "The number of pixels along dimension " + std::to_string(d) +
                                      " is less than 4. This filter requires a minimum of four pixels along the "
                                      "dimension to be processed.");
  const int64_t n = size[0] * size[1] * size[2];
  float* buf = nullptr;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&buf), sizeof(float) * 5 * (size_t)n, st);
  if (e != cudaSuccess) return fail(GB_ERR_OUT_OF_MEMORY, "gradient filter scratch: out of device memory");
  float *A = buf, *B = buf + n, *C = buf + 2 * n, *D = buf + 3 * n, *E = buf + 4 * n;
  RGCoef s[3], dv[3];
  int rc = GB_OK;
  for (int k = 0; k < 3 && rc == GB_OK; ++k) {
    rc = rg_setup(sigma, spacing[k], 0, normalize_across_scale, s[k]);
    if (rc == GB_OK) rc = rg_setup(sigma, spacing[k], 1, normalize_across_scale, dv[k]);
  }
  if (rc != GB_OK) {
    cudaFreeAsync(buf, st);
    return fail(GB_ERR_BAD_ARG, "sigma must be > 0");
  }
  const float inv[3] = {(float)(1.0 / spacing[0]), (float)(1.0 / spacing[1]), (float)(1.0 / spacing[2])};
  // x: A = Dx I, B = Sx I; y: C = Sy A, D = Dy B, E = Sy B;
  // z: gx = Sz C / sx -> A, gy = Sz D / sy -> B, gz = Dz E / sz -> C
  if (e == cudaSuccess) e = rg_pass(st, in, A, size, 0, dv[0], 1.f);
  if (e == cudaSuccess) e = rg_pass(st, in, B, size, 0, s[0], 1.f);
  if (e == cudaSuccess) e = rg_pass(st, A, C, size, 1, s[1], 1.f);
  if (e == cudaSuccess) e = rg_pass(st, B, D, size, 1, dv[1], 1.f);
  if (e == cudaSuccess) e = rg_pass(st, B, E, size, 1, s[1], 1.f);
  if (e == cudaSuccess) e = rg_pass(st, C, A, size, 2, s[2], inv[0]);
  if (e == cudaSuccess) e = rg_pass(st, D, B, size, 2, s[2], inv[1]);
  if (e == cudaSuccess) e = rg_pass(st, E, C, size, 2, dv[2], inv[2]);
  if (e == cudaSuccess) {
    double m[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (use_direction) std::copy(direction, direction + 9, m);
    k_pack_gradient<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, A, B, C, n, (float)m[0], (float)m[1],
                                                                   (float)m[2], (float)m[3], (float)m[4],
                                                                   (float)m[5], (float)m[6], (float)m[7],
                                                                   (float)m[8], out4, out3);
    e = cudaGetLastError();
  }
  cudaFreeAsync(buf, st);
  if (e != cudaSuccess) return fail(GB_ERR_CUDA, std::string("gradient filter: ") + cudaGetErrorString(e));
  return GB_OK;
}

// ShrinkImageFilter::GenerateOutputInformation (start index 0): output spacing
// spacing * f, size floor(size / f) (at least 1), origin moved so that the
// image centre stays put.
void shrink_geometry(const int64_t size[3], const double spacing[3], const double origin[3], const double dir[9],
                     const int64_t factors[3], int64_t out_size[3], double out_spacing[3], double out_origin[3]) {
  double in_c[3], out_c[3];
  for (int i = 0; i < 3; ++i) {
    const int64_t f = factors[i] < 1 ? 1 : factors[i];
    out_spacing[i] = spacing[i] * (double)f;
    out_size[i] = std::max<int64_t>(1, (int64_t)std::floor((double)size[i] / (double)f));
    in_c[i] = (double)(size[i] - 1) / 2.0;
    out_c[i] = (double)(out_size[i] - 1) / 2.0;
  }
  for (int r = 0; r < 3; ++r) {
    double s_in = 0.0, s_out = 0.0;  // continuous index -> point: the sum, then the origin
    for (int c = 0; c < 3; ++c) {
      s_in += dir[r * 3 + c] * spacing[c] * in_c[c];
      s_out += dir[r * 3 + c] * out_spacing[c] * out_c[c];
    }
    out_origin[r] = origin[r] + ((s_in + origin[r]) - (s_out + origin[r]));
  }
}

}  // namespace gb

using namespace gb;

extern "C" int gb_smooth_recursive_gaussian(gb_ctx* ctx, uint64_t stream, const float* d_in, float* d_out,
                                            const int64_t size[3], const double spacing[3], const double sigma[3]) {
  if (!ctx || !d_in || !d_out || !size || !spacing || !sigma) return fail(GB_ERR_BAD_ARG, "null argument");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(GB_ERR_CUDA, "cudaSetDevice failed");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(static_cast<uintptr_t>(stream));
  const int64_t n = size[0] * size[1] * size[2];
  float* tmp = nullptr;
  if (cudaMallocAsync(reinterpret_cast<void**>(&tmp), sizeof(float) * 2 * (size_t)n, st) != cudaSuccess)
    return fail(GB_ERR_OUT_OF_MEMORY, "smoothing scratch: out of device memory");
  const int rc = smooth_rg_device(st, d_in, d_out, tmp, tmp + n, size, spacing, sigma);
  cudaFreeAsync(tmp, st);
  return rc;
}

extern "C" int gb_gradient_recursive_gaussian(gb_ctx* ctx, uint64_t stream, const float* d_in, float* d_out_xyz,
                                              const int64_t size[3], const double spacing[3],
                                              const double direction[9], double sigma, int normalize_across_scale,
                                              int use_image_direction) {
  if (!ctx || !d_in || !d_out_xyz || !size || !spacing || !direction) return fail(GB_ERR_BAD_ARG, "null argument");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(GB_ERR_CUDA, "cudaSetDevice failed");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(static_cast<uintptr_t>(stream));
  return gradient_rg_device(st, d_in, size, spacing, direction, sigma, normalize_across_scale != 0,
                            use_image_direction != 0, nullptr, d_out_xyz);
}

// Host-buffer forms: copy in, run the device filter, copy out (synchronous).
extern "C" int gb_smooth_recursive_gaussian_host(gb_ctx* ctx, const float* in, float* out, const int64_t size[3],
                                                 const double spacing[3], const double sigma[3]) {
  if (!ctx || !in || !out || !size || !spacing || !sigma) return fail(GB_ERR_BAD_ARG, "null argument");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(GB_ERR_CUDA, "cudaSetDevice failed");
  const int64_t n = size[0] * size[1] * size[2];
  DevBuf<float> d;
  if (d.alloc(3 * (size_t)n) != cudaSuccess) return fail(GB_ERR_OUT_OF_MEMORY, "smoothing: out of device memory");
  if (cudaMemcpy(d.p, in, sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(GB_ERR_CUDA, "smoothing: copy in failed");
  int rc = smooth_rg_device(0, d.p, d.p, d.p + n, d.p + 2 * n, size, spacing, sigma);
  if (rc == GB_OK && cudaMemcpy(out, d.p, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = fail(GB_ERR_CUDA, "smoothing: copy out failed");
  return rc;
}

extern "C" int gb_gradient_recursive_gaussian_host(gb_ctx* ctx, const float* in, float* out_xyz,
                                                   const int64_t size[3], const double spacing[3],
                                                   const double direction[9], double sigma,
                                                   int normalize_across_scale, int use_image_direction) {
  if (!ctx || !in || !out_xyz || !size || !spacing || !direction) return fail(GB_ERR_BAD_ARG, "null argument");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(GB_ERR_CUDA, "cudaSetDevice failed");
  const int64_t n = size[0] * size[1] * size[2];
  DevBuf<float> d;
  if (d.alloc(4 * (size_t)n) != cudaSuccess) return fail(GB_ERR_OUT_OF_MEMORY, "gradient: out of device memory");
  if (cudaMemcpy(d.p, in, sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(GB_ERR_CUDA, "gradient: copy in failed");
  int rc = gradient_rg_device(0, d.p, size, spacing, direction, sigma, normalize_across_scale != 0,
                              use_image_direction != 0, nullptr, d.p + n);
  if (rc == GB_OK && cudaMemcpy(out_xyz, d.p + n, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = fail(GB_ERR_CUDA, "gradient: copy out failed");
  return rc;
}

extern "C" int gb_shrink_geometry(const int64_t size[3], const double spacing[3], const double origin[3],
                                  const double direction[9], const int64_t factors[3], int64_t out_size[3],
                                  double out_spacing[3], double out_origin[3]) {
  if (!size || !spacing || !origin || !direction || !factors || !out_size || !out_spacing || !out_origin)
    return fail(GB_ERR_BAD_ARG, "null argument");
  shrink_geometry(size, spacing, origin, direction, factors, out_size, out_spacing, out_origin);
  return GB_OK;
}
