// gb_metric.cu -- C ABI of the registration-metric library (include/itk_gb300.h):
// context and metric handles, Initialize, and one evaluation as a short
// sequence of kernels on the handle's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gb_bspline.cuh"
#include "gb_corr_bspline.cuh"
#include "gb_field.cuh"
#include "gb_jhmi.cuh"
#include "gb_init.cuh"
#include "gb_internal.h"
#include "gb_kernels.cuh"

namespace gb {

static thread_local std::string g_last_error;
static thread_local gb_metric* g_error_scope = nullptr;

gb_metric* error_scope() { return g_error_scope; }
void set_error_scope(gb_metric* m) { g_error_scope = m; }

void set_error(const std::string& msg) {
  g_last_error = msg;
  if (g_error_scope) g_error_scope->last_error = msg;
}

int fail(int code, const std::string& msg) {
  set_error(msg);
  return code;
}

static int cuda_fail(cudaError_t e, const char* where) {
  return fail(GB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define GB_CUDA(call)                                  \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

static int inv3(const double a[9], double out[9]) {
  const double c00 = a[4] * a[8] - a[5] * a[7];
  const double c01 = a[5] * a[6] - a[3] * a[8];
  const double c02 = a[3] * a[7] - a[4] * a[6];
  const double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
  if (det == 0.0 || !std::isfinite(det)) return GB_ERR_BAD_ARG;
  const double id = 1.0 / det;
  out[0] = c00 * id;
  out[1] = (a[2] * a[7] - a[1] * a[8]) * id;
  out[2] = (a[1] * a[5] - a[2] * a[4]) * id;
  out[3] = c01 * id;
  out[4] = (a[0] * a[8] - a[2] * a[6]) * id;
  out[5] = (a[2] * a[3] - a[0] * a[5]) * id;
  out[6] = c02 * id;
  out[7] = (a[1] * a[6] - a[0] * a[7]) * id;
  out[8] = (a[0] * a[4] - a[1] * a[3]) * id;
  return GB_OK;
}

int geom_init(Geom& g, const int64_t size[3], const double spacing[3], const double origin[3], const double dir[9]) {
  for (int i = 0; i < 3; ++i) {
    if (size[i] <= 0 || size[i] > (1 << 20)) return fail(GB_ERR_BAD_ARG, "image size must be in [1, 2^20] per axis");
    if (!(spacing[i] > 0.0) || !std::isfinite(spacing[i])) return fail(GB_ERR_BAD_ARG, "image spacing must be > 0");
    g.size[i] = size[i];
    g.spacing[i] = spacing[i];
    g.origin[i] = origin[i];
  }
  for (int i = 0; i < 9; ++i) g.dir[i] = dir[i];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) g.i2p[r * 3 + c] = dir[r * 3 + c] * spacing[c];
  if (inv3(g.i2p, g.p2i) != GB_OK) return fail(GB_ERR_BAD_ARG, "image direction matrix is singular");
  g.set = true;
  return GB_OK;
}

// host twins of float_to_ordered / ordered_to_float (gb_device.cuh)
static int float_to_ordered_host(float f) {
  int i;
  memcpy(&i, &f, 4);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
static float ordered_to_float_host(int i) {
  const int j = i >= 0 ? i : i ^ 0x7fffffff;
  float f;
  memcpy(&f, &j, 4);
  return f;
}

static DGeom to_dgeom(const Geom& g) {
  DGeom d;
  for (int i = 0; i < 3; ++i) {
    d.n[i] = g.size[i];
    d.origin[i] = g.origin[i];
  }
  for (int i = 0; i < 9; ++i) {
    d.i2p[i] = g.i2p[i];
    d.p2i[i] = g.p2i[i];
  }
  return d;
}

static int grid_for(const gb_metric* m, int64_t n, int per_sm) {
  const int64_t want = (n + kBlock - 1) / kBlock;
  const int64_t cap = std::min<int64_t>((int64_t)m->ctx->sm_count * per_sm, kMaxBlocks);
  return (int)std::max<int64_t>(1, std::min(want, cap));
}

// One full wave of resident blocks (grid-stride kernels), from the occupancy calculator.
template <typename K>
static int full_wave(const gb_metric* m, K kernel, size_t smem, int64_t n) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, smem) != cudaSuccess || per_sm < 1)
    per_sm = 2;
  return grid_for(m, n, per_sm);
}

static bool is_bspline(const gb_metric* m) {
  return m->tkind == GB_TRANSFORM_BSPLINE || m->tkind == GB_TRANSFORM_COMPOSITE;
}

static bool is_field(const gb_metric* m) { return m->tkind == GB_TRANSFORM_DISPLACEMENT_FIELD; }

// Modified Bessel functions of the first kind: Abramowitz & Stegun 9.8.1-9.8.4 for
// orders 0 and 1, Miller's downward recurrence normalized by I0 for n >= 2 (the
// published algorithm GaussianOperator uses, Core/Common/include/itkGaussianOperator.hxx:60-180).
static double bessel_i0(double y) {
  const double d = std::fabs(y);
  if (d < 3.75) {
    double t = y / 3.75;
    t *= t;
    return 1.0 + t * (3.5156229 + t * (3.0899424 + t * (1.2067492 + t * (0.2659732 + t * (0.0360768 + t * 0.0045813)))));
  }
  const double t = 3.75 / d;
  return (std::exp(d) / std::sqrt(d)) *
         (0.39894228 + t * (0.01328592 + t * (0.00225319 + t * (-0.00157565 + t * (0.00916281 +
          t * (-0.02057706 + t * (0.02635537 + t * (-0.01647633 + t * 0.00392377))))))));
}

static double bessel_i1(double y) {
  const double d = std::fabs(y);
  double r;
  if (d < 3.75) {
    double t = y / 3.75;
    t *= t;
    r = d * (0.5 + t * (0.87890594 + t * (0.51498869 + t * (0.15084934 + t * (0.02658733 +
                                                                               t * (0.00301532 + t * 0.00032411))))));
  } else {
    const double t = 3.75 / d;
    double q = 0.02282967 + t * (-0.02895312 + t * (0.01787654 - t * 0.00420059));
    q = 0.39894228 + t * (-0.03988024 + t * (-0.00362018 + t * (0.00163801 + t * (-0.01031555 + t * q))));
    r = q * (std::exp(d) / std::sqrt(d));
  }
  return y < 0.0 ? -r : r;
}

static double bessel_in(int n, double y) {
  if (y == 0.0) return 0.0;
  const double tox = 2.0 / std::fabs(y);
  double bip = 0.0, bi = 1.0, ans = 0.0;
  for (int j = 2 * (n + (int)std::sqrt(40.0 * n)); j > 0; j--) {
    const double bim = bip + j * tox * bi;
    bip = bi;
    bi = bim;
    if (std::fabs(bi) > 1.0e10) {
      ans *= 1.0e-10;
      bi *= 1.0e-10;
      bip *= 1.0e-10;
    }
    if (j == n) ans = bip;
  }
  ans *= bessel_i0(y) / bi;
  return (y < 0.0 && (n & 1)) ? -ans : ans;
}

// GaussianOperator::GenerateCoefficients (itkGaussianOperator.hxx:27-57): e^-v I_k(v)
// until the two-sided sum reaches 1 - max_error or the width limit, normalized,
// mirrored into c[0, 2r]; returns r (at most 32).
static int discrete_gaussian_kernel(double variance, double max_error, int max_width, double c[65]) {
  double half[34];
  const double et = std::exp(-variance);
  int n = 0;
  half[n++] = et * bessel_i0(variance);
  double sum = half[0];
  half[n++] = et * bessel_i1(variance);
  sum += half[1] * 2.0;
  for (int i = 2; sum < 1.0 - max_error && n < 34; ++i) {
    half[n++] = et * bessel_in(i, variance);
    sum += half[i] * 2.0;
    if (half[i] <= 0.0 || n > max_width) break;
  }
  for (int i = 0; i < n; ++i) half[i] /= sum;
  const int r = n - 1;
  for (int i = 0; i <= r; ++i) c[r + i] = c[r - i] = half[i];
  return r;
}

// Initial affine of a B-spline path: the composite's first transform ([affine,
// B-spline] queue, B-spline applied first), the identity for a plain B-spline.
static void bspline_init_affine(const gb_metric* m, double p[12], double c[3]) {
  const double I[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
  const bool comp = m->tkind == GB_TRANSFORM_COMPOSITE;
  for (int i = 0; i < 12; ++i) p[i] = comp ? m->tfixed[18 + i] : I[i];
  for (int i = 0; i < 3; ++i) c[i] = comp ? m->tfixed[30 + i] : 0.0;
}

// Dynamic shared memory of the evaluation kernels' B-spline nodes: staged when
// they leave room for at least two resident blocks per SM, else read from HBM/L2.
static size_t bspline_node_bytes(const gb_metric* m) { return (size_t)m->nper * sizeof(float4); }
static bool nodes_in_smem(const gb_metric* m) {
  const size_t base = m->kind == GB_METRIC_MATTES                ? mattes_bspline_node_offset((int)m->bins)
                      : m->kind == GB_METRIC_JOINT_HISTOGRAM_MI ? jhmi_bspline_node_offset((int)m->bins)
                                                                : 0;
  return base + bspline_node_bytes(m) <= 96 * 1024;
}

}  // namespace gb

using namespace gb;

// ===========================================================================
// context

extern "C" const char* gb_last_error(void) { return g_last_error.c_str(); }

extern "C" const char* gb_metric_last_error(gb_metric* m) { return m ? m->last_error.c_str() : ""; }

extern "C" const char* gb_version(void) { return "itk_gb300 0.1 (sm_103a)"; }

extern "C" int gb_ctx_create(int device, gb_ctx** out) {
  if (!out) return fail(GB_ERR_BAD_ARG, "null output pointer");
  int count = 0;
  GB_CUDA(cudaGetDeviceCount(&count));
  if (device < 0 || device >= count) return fail(GB_ERR_BAD_ARG, "device index out of range");
  GB_CUDA(cudaSetDevice(device));
  int sms = 0;
  GB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  // this process's stream-ordered pool keeps freed blocks for the next level's
  // buffers instead of returning them to the driver at every synchronization
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  gb_ctx* c = new gb_ctx;
  c->device = device;
  c->sm_count = sms;
  *out = c;
  return GB_OK;
}

extern "C" int gb_ctx_destroy(gb_ctx* ctx) {
  delete ctx;
  return GB_OK;
}

extern "C" int gb_ctx_info(gb_ctx* ctx, int* sm_count, uint64_t* total_bytes, uint64_t* free_bytes) {
  if (!ctx) return fail(GB_ERR_BAD_ARG, "null context");
  GB_CUDA(cudaSetDevice(ctx->device));
  size_t fr = 0, tot = 0;
  GB_CUDA(cudaMemGetInfo(&fr, &tot));
  if (sm_count) *sm_count = ctx->sm_count;
  if (total_bytes) *total_bytes = tot;
  if (free_bytes) *free_bytes = fr;
  return GB_OK;
}

// ===========================================================================
// metric handle

extern "C" int gb_metric_create(gb_ctx* ctx, int kind, gb_metric** out) {
  if (!ctx || !out) return fail(GB_ERR_BAD_ARG, "null argument");
  if (kind != GB_METRIC_MEAN_SQUARES && kind != GB_METRIC_MATTES && kind != GB_METRIC_CORRELATION &&
      kind != GB_METRIC_JOINT_HISTOGRAM_MI)
    return fail(GB_ERR_BAD_ARG, "unknown metric kind");
  GB_CUDA(cudaSetDevice(ctx->device));
  gb_metric* m = new gb_metric;
  m->ctx = ctx;
  m->kind = kind;
  if (kind == GB_METRIC_JOINT_HISTOGRAM_MI) m->bins = 20;  // the joint-histogram metric's default
  cudaError_t e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocHost(&m->h_status, sizeof(int) * 4);
  if (e != cudaSuccess) {
    delete m;
    return cuda_fail(e, "gb_metric_create");
  }
  *out = m;
  return GB_OK;
}

void gb_metric::release_buffers() {
  d_fixed.reset(); d_moving.reset(); d_fixed_s.reset(); d_moving_s.reset(); d_grad_in.reset();
  d_mov4.reset(); d_samples.reset(); d_cache.reset(); d_sup.reset(); d_chunks.reset();
  d_node_first.reset(); d_node_entries.reset(); d_chunk_part.reset(); d_nodes.reset(); d_voff.reset();
  d_jhmi.reset(); d_params.reset(); d_acc.reset(); d_scratch.reset(); d_out.reset(); d_status.reset(); d_pratio.reset(); d_pdf.reset();
  d_consts.reset(); d_opt.reset(); d_opt_vec.reset();
}

extern "C" int gb_metric_destroy(gb_metric* m) {
  if (!m) return GB_OK;
  cudaSetDevice(m->ctx->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  m->drop_host_graphs();
  m->release_buffers();  // stream-ordered frees, before the stream goes
  if (m->stream) cudaStreamSynchronize(m->stream);
  if (m->h_params) cudaFreeHost(m->h_params);
  if (m->h_out) cudaFreeHost(m->h_out);
  if (m->h_status) cudaFreeHost(m->h_status);
  if (m->h_consts) cudaFreeHost(m->h_consts);
  if (m->h_opt) cudaFreeHost(m->h_opt);
  if (m->h_halt) cudaFreeHost(m->h_halt);
  for (int i = 0; i < gb_metric::kMaxEvents; ++i)
    if (m->events[i]) cudaEventDestroy(m->events[i]);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
  return GB_OK;
}

extern "C" int gb_metric_set_floating_point_correction(gb_metric* m, int on, double resolution) {
  gb::ErrorScope scope_(m, __func__);
  if (!m) return fail(GB_ERR_BAD_ARG, "null metric");
  if (on && !(resolution > 0.0)) return fail(GB_ERR_BAD_ARG, "floating point correction resolution must be > 0");
  m->fp_res = on ? resolution : 0.0;
  m->initialized = false;
  return GB_OK;
}

extern "C" int gb_metric_set_joint_pdf_smoothing_variance(gb_metric* m, double variance) {
  gb::ErrorScope scope_(m, __func__);
  if (!m) return fail(GB_ERR_BAD_ARG, "null metric");
  if (!(variance == variance)) return fail(GB_ERR_BAD_ARG, "variance is NaN");
  m->jhmi_variance = variance;
  m->initialized = false;
  return GB_OK;
}

extern "C" int gb_metric_set_number_of_histogram_bins(gb_metric* m, uint64_t bins) {
  gb::ErrorScope scope_(m, __func__);
  if (!m) return fail(GB_ERR_BAD_ARG, "null metric");
  if (bins < 5) bins = 5;  // itkSetClampMacro(NumberOfHistogramBins, SizeValueType, 5, max)
  if (bins > 4096) return fail(GB_ERR_BAD_ARG, "number of histogram bins above 4096");
  m->bins = (int64_t)bins;
  m->initialized = false;
  return GB_OK;
}

static int set_image_common(gb_metric* m, int which, const float* src, bool device_src, const int64_t size[3],
                            const double spacing[3], const double origin[3], const double direction[9]) {
  if (!m || !src || !size || !spacing || !origin || !direction) return fail(GB_ERR_BAD_ARG, "null argument");
  if (which != GB_IMAGE_FIXED && which != GB_IMAGE_MOVING) return fail(GB_ERR_BAD_ARG, "unknown image slot");
  GB_CUDA(cudaSetDevice(m->ctx->device));
  Geom g;
  int rc = geom_init(g, size, spacing, origin, direction);
  if (rc) return rc;
  if (g.voxels() > ((int64_t)1 << 31)) return fail(GB_ERR_UNSUPPORTED, "images above 2^31 voxels are not supported");
  DevBuf<float>& buf = which == GB_IMAGE_FIXED ? m->d_fixed : m->d_moving;
  const size_t n = (size_t)g.voxels();
  buf.reset();
  GB_CUDA(buf.alloc_on(m->stream, n));
  GB_CUDA(cudaMemcpyAsync(buf.p, src, n * sizeof(float), device_src ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                          m->stream));
  GB_CUDA(cudaStreamSynchronize(m->stream));
  (which == GB_IMAGE_FIXED ? m->fixed : m->moving) = g;
  if (which == GB_IMAGE_MOVING) m->grad_set = false;
  m->initialized = false;
  return GB_OK;
}

extern "C" int gb_metric_set_image(gb_metric* m, int which, const float* voxels, const int64_t size[3],
                                   const double spacing[3], const double origin[3], const double direction[9]) {
  gb::ErrorScope scope_(m, __func__);
  return set_image_common(m, which, voxels, false, size, spacing, origin, direction);
}

extern "C" int gb_metric_set_image_device(gb_metric* m, int which, const float* device_voxels, const int64_t size[3],
                                          const double spacing[3], const double origin[3],
                                          const double direction[9]) {
  gb::ErrorScope scope_(m, __func__);
  return set_image_common(m, which, device_voxels, true, size, spacing, origin, direction);
}

extern "C" int gb_metric_set_gradient_source(gb_metric* m, int source) {
  gb::ErrorScope scope_(m, __func__);
  if (!m) return fail(GB_ERR_BAD_ARG, "null metric");
  if (source != GB_GRADIENT_IMAGE && source != GB_GRADIENT_CENTRAL_DIFFERENCE &&
      source != GB_GRADIENT_RECURSIVE_GAUSSIAN)
    return fail(GB_ERR_BAD_ARG, "unknown gradient source");
  m->grad_source = source;
  m->initialized = false;
  return GB_OK;
}

extern "C" int gb_metric_set_moving_gradient_image(gb_metric* m, const double* gradient_xyz) {
  gb::ErrorScope scope_(m, __func__);
  if (!m || !gradient_xyz) return fail(GB_ERR_BAD_ARG, "null argument");
  if (!m->moving.set) return fail(GB_ERR_BAD_ARG, "set the moving image before its gradient image");
  GB_CUDA(cudaSetDevice(m->ctx->device));
  const size_t n = (size_t)m->moving.voxels() * 3;
  m->d_grad_in.reset();
  GB_CUDA(m->d_grad_in.alloc_on(m->stream, n));
  GB_CUDA(cudaMemcpyAsync(m->d_grad_in.p, gradient_xyz, n * sizeof(double), cudaMemcpyHostToDevice, m->stream));
  GB_CUDA(cudaStreamSynchronize(m->stream));
  m->grad_set = true;
  m->initialized = false;
  return GB_OK;
}

extern "C" int gb_metric_set_virtual_domain(gb_metric* m, const int64_t size[3], const double spacing[3],
                                            const double origin[3], const double direction[9]) {
  gb::ErrorScope scope_(m, __func__);
  if (!m || !size || !spacing || !origin || !direction) return fail(GB_ERR_BAD_ARG, "null argument");
  Geom g;
  int rc = geom_init(g, size, spacing, origin, direction);
  if (rc) return rc;
  m->virt = g;
  m->virt_user = true;
  m->initialized = false;
  return GB_OK;
}

extern "C" int gb_metric_set_level_smoothing(gb_metric* m, double sigma, int sigma_in_physical_units) {
  gb::ErrorScope scope_(m, __func__);
  if (!m) return fail(GB_ERR_BAD_ARG, "null metric");
  if (!(sigma >= 0.0) || !std::isfinite(sigma)) return fail(GB_ERR_BAD_ARG, "smoothing sigma must be >= 0");
  m->level_sigma = sigma;
  m->level_sigma_physical = sigma_in_physical_units != 0;
  m->initialized = false;
  return GB_OK;
}

extern "C" int gb_metric_set_level_shrink(gb_metric* m, const int64_t factors[3]) {
  gb::ErrorScope scope_(m, __func__);
  if (!m || !factors) return fail(GB_ERR_BAD_ARG, "null argument");
  for (int i = 0; i < 3; ++i) m->level_shrink[i] = factors[i] < 1 ? 1 : factors[i];  // ShrinkImageFilter clamps to 1
  m->initialized = false;
  return GB_OK;
}

extern "C" int gb_metric_set_sampled_points(gb_metric* m, const float* xyz, int64_t n, int virtual_space) {
  gb::ErrorScope scope_(m, __func__);
  if (!m) return fail(GB_ERR_BAD_ARG, "null metric");
  if (n < 0 || (n > 0 && !xyz)) return fail(GB_ERR_BAD_ARG, "bad point array");
  if (n > (int64_t)0x7fffffff) return fail(GB_ERR_BAD_ARG, "more than 2^31-1 sample points");
  m->h_points.assign(xyz, xyz + 3 * n);
  m->points_virtual = virtual_space != 0;
  m->initialized = false;
  return GB_OK;
}

extern "C" int gb_metric_use_sampled_point_set(gb_metric* m, int on) {
  gb::ErrorScope scope_(m, __func__);
  if (!m) return fail(GB_ERR_BAD_ARG, "null metric");
  m->use_sampled = on != 0;
  m->initialized = false;
  return GB_OK;
}

extern "C" int gb_metric_set_moving_transform(gb_metric* m, int kind, const double* params, int64_t nparams,
                                              const double* fixed, int64_t nfixed) {
  gb::ErrorScope scope_(m, __func__);
  if (!m || !params || !fixed) return fail(GB_ERR_BAD_ARG, "null argument");
  if (kind == GB_TRANSFORM_AFFINE) {
    if (nparams != 12 || nfixed != 3) return fail(GB_ERR_BAD_ARG, "affine transform takes 12 parameters and a 3-D centre");
    m->nper = 0;
  } else if (kind == GB_TRANSFORM_BSPLINE || kind == GB_TRANSFORM_COMPOSITE) {
    if (nfixed != (kind == GB_TRANSFORM_BSPLINE ? 18 : 33))
      return fail(GB_ERR_BAD_ARG, "B-spline fixed parameters: 18 (+15 for the initial affine of a composite)");
    int64_t nper = 1;
    for (int i = 0; i < 3; ++i) {
      const double g = fixed[i];
      if (!(g >= 4.0) || g != std::floor(g) || g > 4096.0)
        return fail(GB_ERR_BAD_ARG, "B-spline grid size must be an integer >= 4 (mesh size >= 1)");
      nper *= (int64_t)g;
    }
    if (nparams != 3 * nper) return fail(GB_ERR_BAD_ARG, "B-spline parameter count must be 3 * grid nodes");
    if (nper > 65536) return fail(GB_ERR_UNSUPPORTED, "B-spline grids above 65536 nodes are not supported");
    m->nper = nper;
  } else if (kind == GB_TRANSFORM_DISPLACEMENT_FIELD) {
    // DisplacementFieldTransform fixed parameters: size, origin, spacing, direction
    // (itkDisplacementFieldTransform.hxx:520-570); the parameters are the field
    if (nfixed != 18 && nfixed != 33)
      return fail(GB_ERR_BAD_ARG, "displacement field fixed parameters: size, origin, spacing, direction (18), "
                                  "+ 15 for the initial affine of a composite");
    int64_t nv = 1;
    for (int i = 0; i < 3; ++i) {
      const double g = fixed[i];
      if (!(g >= 1.0) || g != std::floor(g) || g > 2147483647.0)
        return fail(GB_ERR_BAD_ARG, "displacement field size must be a positive integer");
      nv *= (int64_t)g;
      if (nv > (int64_t)0x7fffffff) return fail(GB_ERR_UNSUPPORTED, "displacement fields above 2^31-1 voxels");
    }
    if (nparams != 3 * nv) return fail(GB_ERR_BAD_ARG, "displacement field parameter count must be 3 * field voxels");
    m->nper = 0;
  } else {
    return fail(GB_ERR_BAD_ARG, "unknown transform kind");
  }
  m->tkind = kind;
  m->tparams.assign(params, params + nparams);
  m->tfixed.assign(fixed, fixed + nfixed);
  m->initialized = false;
  return GB_OK;
}

extern "C" int gb_metric_set_parameters(gb_metric* m, const double* params, int64_t nparams) {
  gb::ErrorScope scope_(m, __func__);
  if (!m || !params) return fail(GB_ERR_BAD_ARG, "null argument");
  if (m->tkind < 0) return fail(GB_ERR_BAD_ARG, "no moving transform set");
  if ((size_t)nparams != m->tparams.size()) return fail(GB_ERR_BAD_ARG, "parameter count mismatch");
  copy_parallel(m->tparams.data(), params, sizeof(double) * (size_t)nparams);
  return GB_OK;
}

extern "C" int gb_metric_update_transform_parameters(gb_metric* m, const double* update, int64_t nparams,
                                                     double factor) {
  gb::ErrorScope scope_(m, __func__);
  if (!m || !update) return fail(GB_ERR_BAD_ARG, "null argument");
  if ((size_t)nparams != m->tparams.size())
    return fail(GB_ERR_BAD_ARG, "Parameter update size must be same as transform parameter size");
  if (factor == 1.0)
    for (int64_t k = 0; k < nparams; ++k) m->tparams[k] += update[k];
  else
    for (int64_t k = 0; k < nparams; ++k) m->tparams[k] += update[k] * factor;
  return GB_OK;
}

extern "C" int gb_metric_get_parameters(gb_metric* m, double* params, int64_t nparams) {
  gb::ErrorScope scope_(m, __func__);
  if (!m || !params) return fail(GB_ERR_BAD_ARG, "null argument");
  if ((size_t)nparams != m->tparams.size()) return fail(GB_ERR_BAD_ARG, "parameter count mismatch");
  copy_parallel(params, m->tparams.data(), sizeof(double) * m->tparams.size());
  return GB_OK;
}

extern "C" int gb_metric_get_number_of_parameters(gb_metric* m, int64_t* nparams) {
  gb::ErrorScope scope_(m, __func__);
  if (!m || !nparams) return fail(GB_ERR_BAD_ARG, "null argument");
  *nparams = (int64_t)m->tparams.size();
  return GB_OK;
}

// ===========================================================================
// Initialize

// Accumulators cleared before every evaluation:
// acc_n u64 | tickets kTicketCount u32 | hist B*B u64 | fmarg B u64 | colsum B u64 | 16 bytes
// The histogram starts at a 16-byte boundary and the padding covers the Mattes
// derivative pass's bulk copy of hist..colsum rounded up to 16 bytes.
static size_t acc_offset_tickets() { return 8; }
static size_t acc_offset_hist() { return (8 + sizeof(unsigned) * kTicketCount + 15) / 16 * 16; }
static size_t acc_offset_fmarg(int64_t B) { return acc_offset_hist() + 8 * (size_t)(B * B); }
static size_t acc_offset_colsum(int64_t B) { return acc_offset_fmarg(B) + 8 * (size_t)B; }
static size_t acc_layout_bytes(const gb_metric* m) {
  const int64_t B = (m->kind == GB_METRIC_MATTES || m->kind == GB_METRIC_JOINT_HISTOGRAM_MI) ? m->bins : 0;
  return (acc_offset_colsum(B) + 8 * (size_t)B + 16 + 15) / 16 * 16;
}

extern "C" int gb_metric_initialize(gb_metric* m) {
  gb::ErrorScope scope_(m, __func__);
  if (!m) return fail(GB_ERR_BAD_ARG, "null metric");
  m->drop_host_graphs();  // they hold this level's buffers and arguments
  if (!m->fixed.set) return fail(GB_ERR_BAD_ARG, "FixedImage is not present");
  if (!m->moving.set) return fail(GB_ERR_BAD_ARG, "MovingImage is not present");
  if (m->tkind < 0) return fail(GB_ERR_BAD_ARG, "MovingTransform is not present");
  if (m->grad_source == GB_GRADIENT_IMAGE && !m->grad_set)
    return fail(GB_ERR_BAD_ARG, "gradient source is a gradient image but none was set");
  const bool bspline = is_bspline(m);
  const bool field = is_field(m);
  if (field && m->kind == GB_METRIC_CORRELATION)  // as the reference's constructor refuses it
    return fail(GB_ERR_UNSUPPORTED, "the correlation metric does not support displacement field transforms");
  const bool jhmi = m->kind == GB_METRIC_JOINT_HISTOGRAM_MI;
  if (jhmi && (m->bins < 6 || m->bins > kJhmiMaxBins))
    return fail(GB_ERR_UNSUPPORTED, "the joint-histogram metric takes 6 to 64 bins");
  // the floating point correction acts where points store a global derivative
  // (MeanSquares, joint-histogram MI); Mattes, correlation and local-support
  // transforms accumulate elsewhere, so it has no effect there, as in the reference
  if (m->fp_res > 0.0 && (jhmi || (m->kind == GB_METRIC_MEAN_SQUARES && !field && m->tkind != GB_TRANSFORM_AFFINE)))
    return fail(GB_ERR_UNSUPPORTED, "the floating point correction runs MeanSquares with affine transforms");
  double g_p2i[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  if (bspline) {
    // BSplineTransform fixed parameters: grid size, origin, spacing, direction (itkBSplineTransform.hxx:243-283)
    const double* f = m->tfixed.data();
    double i2p[9];
    for (int i = 0; i < 3; ++i) {
      if (f[i] > 1024.0) return fail(GB_ERR_UNSUPPORTED, "B-spline grids above 1024 nodes per axis are not supported");
      m->grid[i] = (int)f[i];
    }
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) i2p[r * 3 + c] = f[9 + r * 3 + c] * f[6 + c];
    if (inv3(i2p, g_p2i) != GB_OK) return fail(GB_ERR_BAD_ARG, "B-spline grid direction * spacing is singular");
  }
  GB_CUDA(cudaSetDevice(m->ctx->device));
  m->initialized = false;
  cudaStream_t st = m->stream;

  // ---- the level's images: both through SmoothingRecursiveGaussianImageFilter
  // (ImageRegistrationMethodv4.hxx:590-640), kept on the device
  if (m->level_sigma > 0.0) {
    for (int w = 0; w < 2; ++w) {
      const Geom& g = w == 0 ? m->fixed : m->moving;
      const float* src = w == 0 ? m->d_fixed.p : m->d_moving.p;
      DevBuf<float>& dst = w == 0 ? m->d_fixed_s : m->d_moving_s;
      double sig[3];
      for (int i = 0; i < 3; ++i) sig[i] = m->level_sigma_physical ? m->level_sigma : m->level_sigma * g.spacing[i];
      const int64_t nv = g.voxels();
      DevBuf<float> tmp;
      GB_CUDA(dst.alloc_on(m->stream, nv));
      GB_CUDA(tmp.alloc_on(m->stream, 2 * (size_t)nv));
      const int rc = smooth_rg_device(st, src, dst.p, tmp.p, tmp.p + nv, g.size, g.spacing, sig);
      if (rc) return rc;
      GB_CUDA(cudaStreamSynchronize(st));  // tmp is released at the end of this scope
    }
  } else {
    m->d_fixed_s.reset();
    m->d_moving_s.reset();
  }
  // ---- virtual domain: the fixed image's geometry (itkImageToImageMetricv4.hxx:98-112),
  // shrunk for the level (ShrinkImageFilter, ImageRegistrationMethodv4.hxx:448-461)
  if (!m->virt_user) {
    m->virt = m->fixed;
    if (m->level_shrink[0] != 1 || m->level_shrink[1] != 1 || m->level_shrink[2] != 1) {
      int64_t sz[3];
      double sp[3], org[3];
      shrink_geometry(m->fixed.size, m->fixed.spacing, m->fixed.origin, m->fixed.dir, m->level_shrink, sz, sp, org);
      const int rc = geom_init(m->virt, sz, sp, org, m->fixed.dir);
      if (rc) return rc;
    }
  }

  if (field) {
    // VerifyDisplacementFieldSizeAndPhysicalSpace (itkObjectToObjectMetric.hxx:444-503): the
    // derivative field is laid out on the virtual grid, so the two grids must coincide
    const double* f = m->tfixed.data();
    for (int i = 0; i < 3; ++i)
      if ((int64_t)f[i] != m->virt.size[i])
        return fail(GB_ERR_BAD_ARG,
                    "Virtual domain and moving transform displacement field must have the same size and index for "
                    "BufferedRegion.");
    const double ctol = 1.0e-6 * m->virt.spacing[0];
    bool same = true;
    for (int i = 0; i < 3; ++i)
      same = same && std::fabs(f[3 + i] - m->virt.origin[i]) <= ctol && std::fabs(f[6 + i] - m->virt.spacing[i]) <= ctol;
    for (int i = 0; i < 9; ++i) same = same && std::fabs(f[9 + i] - m->virt.dir[i]) <= 1.0e-6;
    if (!same)
      return fail(GB_ERR_BAD_ARG,
                  "Virtual Domain and DisplacementField do not occupy the same physical space! You may be able to "
                  "simply call displacementField->CopyInformation( metric->GetVirtualImage() ) to align them.");
  }

  const bool sampled = m->use_sampled;
  if (sampled && m->h_points.empty()) return fail(GB_ERR_BAD_ARG, "VirtualSampledPointSet must have 1 or more points.");
  const int64_t ncand = sampled ? (int64_t)(m->h_points.size() / 3) : m->virt.voxels();
  if (ncand > (int64_t)0x7fffffff) return fail(GB_ERR_UNSUPPORTED, "more than 2^31-1 domain points");
  m->ndomain = ncand;

  DevBuf<float> d_pts;
  if (sampled) {
    GB_CUDA(d_pts.alloc_on(m->stream, m->h_points.size()));
    GB_CUDA(cudaMemcpyAsync(d_pts.p, m->h_points.data(), m->h_points.size() * sizeof(float), cudaMemcpyHostToDevice, st));
  }

  // ---- Mattes ranges and bins (Mattes...v4.hxx:75-327)
  const DGeom dfixed = to_dgeom(m->fixed), dvirt = to_dgeom(m->virt);
  if (m->kind == GB_METRIC_MATTES) {
    DevBuf<int> d_mm;
    GB_CUDA(d_mm.alloc_on(m->stream, 4));
    int init[4] = {float_to_ordered_host(FLT_MAX), float_to_ordered_host(-FLT_MAX), float_to_ordered_host(FLT_MAX),
                   float_to_ordered_host(-FLT_MAX)};
    GB_CUDA(cudaMemcpyAsync(d_mm.p, init, sizeof(init), cudaMemcpyHostToDevice, st));
    if (sampled) {
      k_minmax_points<<<grid_for(m, ncand, 4), kBlock, 0, st>>>(d_pts.p, ncand, dfixed, m->fixed_img(), d_mm.p);
    } else {
      k_minmax<<<grid_for(m, m->fixed.voxels(), 4), kBlock, 0, st>>>(m->fixed_img(), m->fixed.voxels(), d_mm.p);
    }
    k_minmax<<<grid_for(m, m->moving.voxels(), 4), kBlock, 0, st>>>(m->moving_img(), m->moving.voxels(), d_mm.p + 2);
    GB_CUDA(cudaGetLastError());
    int res[4];
    GB_CUDA(cudaMemcpyAsync(res, d_mm.p, sizeof(res), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    const double fmin = (double)ordered_to_float_host(res[0]), fmax = (double)ordered_to_float_host(res[1]);
    const double mmin = (double)ordered_to_float_host(res[2]), mmax = (double)ordered_to_float_host(res[3]);
    const bool fempty = res[0] == float_to_ordered_host(FLT_MAX) && res[1] == float_to_ordered_host(-FLT_MAX);
    m->mstate[0] = fmin;
    m->mstate[1] = fmax;
    m->mstate[2] = mmin;
    m->mstate[3] = mmax;
    if (fempty || fmax < fmin)
      return fail(GB_ERR_FIXED_EMPTY,
                  "No fixed-image samples were observed in the analysis region. Verify that the fixed image mask or "
                  "sampled point set contains at least one valid pixel that overlaps the fixed image buffered region.");
    if (fmax - fmin <= DBL_EPSILON)
      return fail(GB_ERR_FIXED_CONSTANT,
                  "All fixed-image samples in the analysis region have the same intensity value (" +
                      std::to_string(fmin) +
                      "). Mattes mutual information is undefined for a constant image: the marginal entropy is zero "
                      "and no meaningful gradient can be computed.");
    if (mmax < mmin)
      return fail(GB_ERR_MOVING_EMPTY, "No moving-image samples were observed in the analysis region.");
    if (mmax - mmin <= DBL_EPSILON)
      return fail(GB_ERR_MOVING_CONSTANT,
                  "All moving-image samples in the analysis region have the same intensity value (" +
                      std::to_string(mmin) +
                      "). Mattes mutual information is undefined for a constant image: the marginal entropy is zero "
                      "and no meaningful gradient can be computed.");
    const double padding = 2.0;
    m->mstate[4] = (fmax - fmin) / (double)(m->bins - 2 * 2);
    m->mstate[6] = fmin / m->mstate[4] - padding;
    m->mstate[5] = (mmax - mmin) / (double)(m->bins - 2 * 2);
    m->mstate[7] = mmin / m->mstate[5] - padding;
  }

  // ---- joint-histogram MI: true min / max over the whole level images, joint-PDF
  // geometry, smoothing kernel (itkJointHistogramMutualInformationImageToImageMetricv4.hxx:70-190)
  if (jhmi) {
    DevBuf<int> d_mm;
    GB_CUDA(d_mm.alloc_on(m->stream, 4));
    int init[4] = {float_to_ordered_host(FLT_MAX), float_to_ordered_host(-FLT_MAX), float_to_ordered_host(FLT_MAX),
                   float_to_ordered_host(-FLT_MAX)};
    GB_CUDA(cudaMemcpyAsync(d_mm.p, init, sizeof(init), cudaMemcpyHostToDevice, st));
    k_minmax<<<grid_for(m, m->fixed.voxels(), 4), kBlock, 0, st>>>(m->fixed_img(), m->fixed.voxels(), d_mm.p);
    k_minmax<<<grid_for(m, m->moving.voxels(), 4), kBlock, 0, st>>>(m->moving_img(), m->moving.voxels(), d_mm.p + 2);
    GB_CUDA(cudaGetLastError());
    int res[4];
    GB_CUDA(cudaMemcpyAsync(res, d_mm.p, sizeof(res), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    JhmiConsts C;
    std::memset(&C, 0, sizeof(C));
    C.fmin = (double)ordered_to_float_host(res[0]);
    C.fmax = (double)ordered_to_float_host(res[1]);
    C.mmin = (double)ordered_to_float_host(res[2]);
    C.mmax = (double)ordered_to_float_host(res[3]);
    C.spacing = 1.0 / (double)(m->bins - 2 * 2 - 1);
    C.origin = C.spacing * 2.0 * -1.0;
    C.inv_spacing = 1.0 / C.spacing;
    C.fmin_f = (float)C.fmin;
    C.finv_f = (float)(1.0 / (C.fmax - C.fmin));
    C.mmin_f = (float)C.mmin;
    C.minv_f = (float)(1.0 / (C.mmax - C.mmin));
    C.origin_f = (float)C.origin;
    C.inv_spacing_f = (float)C.inv_spacing;
    C.spacing_f = (float)C.spacing;
    C.radius = m->jhmi_variance > 0.0 ? discrete_gaussian_kernel(m->jhmi_variance, 0.01, 32, C.kernel) : 0;
    m->mstate[0] = C.fmin;
    m->mstate[1] = C.fmax;
    m->mstate[2] = C.mmin;
    m->mstate[3] = C.mmax;
    GB_CUDA(m->d_jhmi.alloc_on(m->stream, sizeof(JhmiConsts)));
    GB_CUDA(cudaMemcpyAsync(m->d_jhmi.p, &C, sizeof(C), cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaStreamSynchronize(st));  // C lives on this stack frame
  }

  // ---- sample list: fixed values / bins in FP64, spatial sort
  DevBuf<uint64_t> keys, keys_sorted;
  DevBuf<uint32_t> vals, vals_sorted;
  DevBuf<float4> recs;
  DevBuf<unsigned long long> d_nvalid;
  GB_CUDA(keys.alloc_on(m->stream, ncand));
  GB_CUDA(keys_sorted.alloc_on(m->stream, ncand));
  GB_CUDA(vals.alloc_on(m->stream, ncand));
  GB_CUDA(vals_sorted.alloc_on(m->stream, ncand));
  GB_CUDA(recs.alloc_on(m->stream, ncand));
  GB_CUDA(d_nvalid.alloc_on(m->stream, 1));
  GB_CUDA(cudaMemsetAsync(d_nvalid.p, 0, sizeof(unsigned long long), st));
  BuildArgs b{};
  b.points = sampled ? d_pts.p : nullptr;
  b.n = ncand;
  b.points_virtual = m->points_virtual ? 1 : 0;
  b.virt = dvirt;
  b.fixed = dfixed;
  b.fixed_img = m->fixed_img();
  b.mattes = m->kind == GB_METRIC_MATTES;
  b.bins = (int)m->bins;
  b.f_bs = m->mstate[4];
  b.f_normmin = m->mstate[6];
  b.bspline = bspline ? 1 : 0;
  DevBuf<float4> sup;
  if (bspline) {
    GB_CUDA(sup.alloc_on(m->stream, ncand));
    for (int i = 0; i < 3; ++i) {
      b.grid[i] = m->grid[i];
      b.g_origin[i] = m->tfixed[3 + i];
    }
    for (int i = 0; i < 9; ++i) b.g_p2i[i] = g_p2i[i];
  }
  DevBuf<uint32_t> voff;
  const bool want_voff = field && sampled;
  if (want_voff) GB_CUDA(voff.alloc_on(m->stream, ncand));
  b.keys = keys.p;
  b.vals = vals.p;
  b.recs = recs.p;
  b.sup = bspline ? sup.p : nullptr;
  b.voff = want_voff ? voff.p : nullptr;
  b.nvalid = d_nvalid.p;
  k_build_samples<<<(unsigned)((ncand + kBlock - 1) / kBlock), kBlock, 0, st>>>(b);
  GB_CUDA(cudaGetLastError());
  GB_CUDA(sort_pairs_u64(keys.p, keys_sorted.p, vals.p, vals_sorted.p, ncand, 64, st));
  unsigned long long nvalid = 0;
  GB_CUDA(cudaMemcpyAsync(&nvalid, d_nvalid.p, sizeof(nvalid), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  m->nsamples = (int64_t)nvalid;
  m->d_samples.reset();
  GB_CUDA(m->d_samples.alloc_on(m->stream, std::max<int64_t>(1, m->nsamples)));
  m->d_sup.reset();
  if (bspline) GB_CUDA(m->d_sup.alloc_on(m->stream, std::max<int64_t>(1, m->nsamples)));
  m->d_voff.reset();
  if (want_voff) GB_CUDA(m->d_voff.alloc_on(m->stream, std::max<int64_t>(1, m->nsamples)));
  if (m->nsamples > 0)
    k_gather_samples<<<(unsigned)((m->nsamples + kBlock - 1) / kBlock), kBlock, 0, st>>>(
        vals_sorted.p, m->nsamples, recs.p, m->d_samples.p, bspline ? sup.p : nullptr,
        bspline ? m->d_sup.p : nullptr, want_voff ? voff.p : nullptr, want_voff ? m->d_voff.p : nullptr);
  GB_CUDA(cudaGetLastError());

  // ---- B-spline: runs of same-cell samples (at most kChunkLen each) for the
  // derivative's per-cell reduction, and each cell's first run
  m->nchunks = 0;
  if (bspline) {
    std::vector<uint64_t> hk((size_t)m->nsamples);
    if (m->nsamples > 0)
      GB_CUDA(cudaMemcpyAsync(hk.data(), keys_sorted.p, sizeof(uint64_t) * m->nsamples, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    std::vector<int4> chunks;
    std::vector<int> cell_first((size_t)m->nper + 2, 0);
    for (int64_t i = 0; i < m->nsamples;) {
      const uint64_t cell = hk[i] >> kCellShift;
      int64_t j = i + 1;
      while (j < m->nsamples && (hk[j] >> kCellShift) == cell && j - i < kChunkLen) ++j;
      if (cell > 0) {
        chunks.push_back(make_int4((int)i, (int)j, (int)cell, 0));
        ++cell_first[cell + 1];
      }
      i = j;
    }
    for (size_t c = 1; c < cell_first.size(); ++c) cell_first[c] += cell_first[c - 1];
    if (chunks.size() > (size_t)(0x7fffffff / 192) || chunks.size() * 64 > (size_t)0x7fffffff)
      return fail(GB_ERR_UNSUPPORTED, "too many B-spline sample chunks for 32-bit chunk-sum indices");
    // per node: the chunk-sum entries (chunk * 192 + support position k) of every
    // cell whose 4x4x4 support holds the node, cells in z, y, x order, chunks in order
    const int gx = m->grid[0], gy = m->grid[1], gz = m->grid[2];
    std::vector<int> node_first((size_t)m->nper + 1, 0);
    std::vector<int> entries;
    entries.reserve(chunks.size() * 64);
    for (int64_t n = 0; n < m->nper; ++n) {
      node_first[n] = (int)entries.size();
      const int ix = (int)(n % gx), iy = (int)((n / gx) % gy), iz = (int)(n / ((int64_t)gx * gy));
      for (int cz = std::max(0, iz - 3); cz <= std::min(iz, gz - 4); ++cz)
        for (int cy = std::max(0, iy - 3); cy <= std::min(iy, gy - 4); ++cy)
          for (int cx = std::max(0, ix - 3); cx <= std::min(ix, gx - 4); ++cx) {
            const int64_t cell = 1 + cx + (int64_t)gx * (cy + (int64_t)gy * cz);
            const int k = (ix - cx) + 4 * (iy - cy) + 16 * (iz - cz);
            for (int q = cell_first[cell]; q < cell_first[cell + 1]; ++q) entries.push_back(q * 192 + k);
          }
    }
    node_first[m->nper] = (int)entries.size();
    m->nchunks = (int64_t)chunks.size();
    m->d_chunks.reset();
    m->d_node_first.reset();
    m->d_node_entries.reset();
    m->d_chunk_part.reset();
    GB_CUDA(m->d_chunks.alloc_on(m->stream, std::max<size_t>(1, chunks.size())));
    GB_CUDA(m->d_node_first.alloc_on(m->stream, node_first.size()));
    GB_CUDA(m->d_node_entries.alloc_on(m->stream, std::max<size_t>(1, entries.size())));
    m->node_entries_count = (int64_t)entries.size();
    GB_CUDA(m->d_chunk_part.alloc_on(m->stream, std::max<size_t>(1, chunks.size()) * 192));
    if (!chunks.empty())
      GB_CUDA(cudaMemcpyAsync(m->d_chunks.p, chunks.data(), sizeof(int4) * chunks.size(), cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(m->d_node_first.p, node_first.data(), sizeof(int) * node_first.size(),
                            cudaMemcpyHostToDevice, st));
    if (!entries.empty())
      GB_CUDA(cudaMemcpyAsync(m->d_node_entries.p, entries.data(), sizeof(int) * entries.size(),
                              cudaMemcpyHostToDevice, st));
    m->d_nodes.reset();
    GB_CUDA(m->d_nodes.alloc_on(m->stream, (size_t)m->nper));
    GB_CUDA(cudaStreamSynchronize(st));  // the host vectors die here
  }

  // ---- moving image: packed (value, gradient) for the gradient-image paths
  if (m->grad_source == GB_GRADIENT_IMAGE) {
    const int64_t nv = m->moving.voxels();
    m->d_mov4.reset();
    GB_CUDA(m->d_mov4.alloc_on(m->stream, nv));
    k_pack_moving<<<(unsigned)((nv + kBlock - 1) / kBlock), kBlock, 0, st>>>(m->moving_img(), m->d_grad_in.p, nv,
                                                                              m->d_mov4.p);
    GB_CUDA(cudaGetLastError());
  } else if (m->grad_source == GB_GRADIENT_RECURSIVE_GAUSSIAN) {
    // the metric's default gradient filter: sigma = max spacing, normalized across
    // scale, image direction applied (itkImageToImageMetricv4.hxx:488-503)
    const int64_t nv = m->moving.voxels();
    m->d_mov4.reset();
    GB_CUDA(m->d_mov4.alloc_on(m->stream, nv));
    const double sigma = std::max(m->moving.spacing[0], std::max(m->moving.spacing[1], m->moving.spacing[2]));
    const int rc = gradient_rg_device(st, m->moving_img(), m->moving.size, m->moving.spacing, m->moving.dir, sigma,
                                      true, true, m->d_mov4.p, nullptr);
    if (rc) return rc;
  }

  // ---- evaluation buffers
  const size_t P = m->tparams.size();
  m->acc_bytes = acc_layout_bytes(m);
  m->d_acc.reset();
  GB_CUDA(m->d_acc.alloc_on(m->stream, m->acc_bytes));
  GB_CUDA(m->d_scratch.alloc_on(m->stream, kScratchDoubles));
  GB_CUDA(m->d_params.alloc_on(m->stream, P));
  m->d_out.reset();
  GB_CUDA(m->d_out.alloc_on(m->stream, 2 + P));
  GB_CUDA(m->d_status.alloc_on(m->stream, 1));
  if (m->kind == GB_METRIC_MATTES || jhmi) {
    m->d_pratio.reset();  // log(p / pm) table; the joint-histogram metric: FP32 PDF and moving marginal
    GB_CUDA(m->d_pratio.alloc_on(m->stream, (size_t)(m->bins * m->bins + m->bins)));
    m->d_pdf.reset();
    GB_CUDA(m->d_pdf.alloc_on(m->stream, (size_t)(m->bins * m->bins)));
    GB_CUDA(cudaMemsetAsync(m->d_pdf.p, 0, sizeof(double) * m->bins * m->bins, st));
  }
  m->d_cache.reset();
  if (m->kind == GB_METRIC_MATTES || jhmi || bspline)
    GB_CUDA(m->d_cache.alloc_on(m->stream, std::max<int64_t>(1, m->nsamples)));
  if (m->h_cap < 2 + P) {  // pinned staging, reused while large enough (cudaFreeHost waits for the device)
    if (m->h_params) cudaFreeHost(m->h_params);
    if (m->h_out) cudaFreeHost(m->h_out);
    m->h_params = nullptr;
    m->h_out = nullptr;
    m->h_cap = 0;
    GB_CUDA(cudaMallocHost(&m->h_params, sizeof(double) * (2 + P)));
    GB_CUDA(cudaMallocHost(&m->h_out, sizeof(double) * (2 + P)));
    m->h_cap = 2 + P;
  }
  GB_CUDA(m->d_consts.alloc_on(m->stream, 1));
  if (!m->h_consts) GB_CUDA(cudaMallocHost(&m->h_consts, sizeof(EvalConsts)));
  if (bspline) {
    // the B-spline paths' constants depend only on the fixed initial affine: once, here
    double p[12], c[3];
    bspline_init_affine(m, p, c);
    affine_consts(p, c, m->moving.p2i, m->moving.origin, sampled ? nullptr : m->virt.i2p, m->virt.origin,
                  *m->h_consts);
    GB_CUDA(cudaMemcpyAsync(m->d_consts.p, m->h_consts, sizeof(EvalConsts), cudaMemcpyHostToDevice, st));
  }
  if (field) {
    // the displacement-field constants are geometry only: the identity transform's
    // map, the moving image's physical-to-index matrix for the displacement and,
    // for a point set, the physical point -> field continuous index map
    // a [affine, field] composite: the map is the initial affine's, the displacement
    // goes through P2I M and the gradient through M^T (K.Mg)
    double p[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0}, c[3] = {0, 0, 0};
    if (m->tfixed.size() == 33) {
      for (int i = 0; i < 12; ++i) p[i] = m->tfixed[18 + i];
      for (int i = 0; i < 3; ++i) c[i] = m->tfixed[30 + i];
    }
    EvalConsts& K = *m->h_consts;
    affine_consts(p, c, m->moving.p2i, m->moving.origin, sampled ? nullptr : m->virt.i2p, m->virt.origin, K);
    for (int r = 0; r < 3; ++r)
      for (int cc = 0; cc < 3; ++cc) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s = gb::dadd(s, gb::dmul(m->moving.p2i[3 * r + k], p[3 * k + cc]));
        split_df(s, K.umap.Ahi[3 * r + cc], K.umap.Alo[3 * r + cc]);
      }
    for (int r = 0; r < 3; ++r) {
      K.umap.bhi[r] = K.umap.blo[r] = 0.f;
      double b = 0.0;
      for (int k = 0; k < 3; ++k) {
        split_df(m->virt.p2i[3 * r + k], K.fmap.Ahi[3 * r + k], K.fmap.Alo[3 * r + k]);
        b = gb::dadd(b, -gb::dmul(m->virt.p2i[3 * r + k], m->virt.origin[k]));
      }
      split_df(b, K.fmap.bhi[r], K.fmap.blo[r]);
    }
    bool diag = true;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c)
        if (r != c)
          diag = diag && K.map.Ahi[3 * r + c] == 0.f && K.map.Alo[3 * r + c] == 0.f && K.umap.Ahi[3 * r + c] == 0.f &&
                 K.umap.Alo[3 * r + c] == 0.f;
    K.fdiag = diag ? 1.f : 0.f;
    GB_CUDA(cudaMemcpyAsync(m->d_consts.p, m->h_consts, sizeof(EvalConsts), cudaMemcpyHostToDevice, st));
  }
  GB_CUDA(cudaStreamSynchronize(st));
  m->initialized = true;
  return GB_OK;
}

// ===========================================================================
// evaluation

static void fill_eval_args(gb_metric* m, EvalArgs& a, const double* d_params, double* d_out, bool deriv) {
  memset(&a, 0, sizeof(a));
  a.samples = m->d_samples.p;
  a.n = m->nsamples;
  a.mov4 = m->d_mov4.p;
  a.mov1 = m->moving_img();
  a.nx = (int)m->moving.size[0];
  a.ny = (int)m->moving.size[1];
  a.nz = (int)m->moving.size[2];
  for (int i = 0; i < 9; ++i) a.m_p2i[i] = m->moving.p2i[i];
  for (int i = 0; i < 3; ++i) a.m_origin[i] = m->moving.origin[i];
  // central difference: +0.5 spacing along physical axis d, in index space
  for (int d = 0; d < 3; ++d) {
    const double off = 0.5 * m->moving.spacing[d];
    for (int k = 0; k < 3; ++k) split_df(m->moving.p2i[3 * k + d] * off, a.cd_hi[3 * d + k], a.cd_lo[3 * d + k]);
    a.cd_inv_delta[d] = (float)(1.0 / ((off) - (-off)));
  }
  a.params = d_params;
  a.nparams = (int)m->tparams.size();
  if (m->tkind == GB_TRANSFORM_AFFINE)
    for (int i = 0; i < 3; ++i) a.center[i] = m->tfixed[i];
  a.dense = m->use_sampled ? 0 : 1;
  for (int i = 0; i < 9; ++i) a.v_i2p[i] = m->virt.i2p[i];
  for (int i = 0; i < 3; ++i) a.v_origin[i] = m->virt.origin[i];
  a.bins = (int)m->bins;
  a.mmin = (float)m->mstate[2];
  a.mmax = (float)m->mstate[3];
  a.m_bs = m->mstate[5];
  a.m_inv_bs = (float)(1.0 / m->mstate[5]);
  unsigned char* base = m->d_acc.p;
  a.acc_n = reinterpret_cast<unsigned long long*>(base);
  a.tickets = reinterpret_cast<unsigned*>(base + acc_offset_tickets());
  a.acc = reinterpret_cast<uint4*>(base);
  a.acc_words = (int)(m->acc_bytes / 16);
  a.hist = reinterpret_cast<unsigned long long*>(base + acc_offset_hist());
  a.fmarg = reinterpret_cast<unsigned long long*>(base + acc_offset_fmarg(m->bins));
  a.colsum = reinterpret_cast<unsigned long long*>(base + acc_offset_colsum(m->bins));
  a.consts = m->d_consts.p;
  a.part = m->d_scratch.p;
  a.grp = m->d_scratch.p + kGroupOffset;
  a.marg = m->d_scratch.p + kMargOffset;
  a.cache = m->d_cache.p;
  a.pratio = m->d_pratio.p;
  a.pdf_out = m->d_pdf.p;
  a.out = d_out;
  a.status = m->d_status.p;
  a.with_derivative = deriv ? 1 : 0;
  a.halt = m->eval_halt;
  a.fp_res = m->fp_res;
  a.inject_stall = m->inject_fault == GB_FAULT_STALLED_COPY ? 1 : 0;
  if (is_bspline(m)) {
    a.sup = m->d_sup.p;
    a.nodes = m->d_nodes.p;
    a.gx = m->grid[0];
    a.gy = m->grid[1];
    a.gz = m->grid[2];
    a.nper = (int)m->nper;
    a.nodes_smem = nodes_in_smem(m) ? 1 : 0;
    a.chunks = m->d_chunks.p;
    a.nchunks = (int)m->nchunks;
    a.node_first = m->d_node_first.p;
    a.node_entries = m->d_node_entries.p;
    a.chunk_part = m->d_chunk_part.p;
  }
  if (is_field(m)) {
    a.field = d_params ? d_params : m->d_params.p;  // the host call uploads the field to d_params
    a.vnx = (int)m->virt.size[0];
    a.vny = (int)m->virt.size[1];
    a.vnz = (int)m->virt.size[2];
    a.voff = m->d_voff.p;
    a.field_full = (!m->use_sampled && m->nsamples == m->virt.voxels()) ? 1 : 0;
  }
}

// Evaluation arguments of the device-resident form (parameters in d_params,
// results in d_out, with the derivative), for the batched engine.
void gb::batch_eval_args(gb_metric* m, EvalArgs& a) { fill_eval_args(m, a, m->d_params.p, m->d_out.p, true); }

// One kernel of the evaluation chain on the handle's stream, launched with
// programmatic stream serialization: its blocks may be scheduled while the
// previous kernel drains, and wait in griddep_wait() for its results.
template <typename... KArgs, typename... Args>
static cudaError_t launch_chain(gb_metric* m, void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem,
                                Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = m->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Grid-stride evaluation kernel with `smem` bytes of dynamic shared memory, one full wave.
template <typename K, typename... Extra>
static cudaError_t launch_wave(gb_metric* m, K kernel, size_t smem, const EvalArgs& a, Extra... extra) {
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return launch_chain(m, kernel, (unsigned)full_wave(m, kernel, smem, m->nsamples), kBlock, smem, a, extra...);
}

// Mattes pass 2 (affine): kPass2Threads threads per block (the streaming threads and
// the value's group warp), one full wave, at most kFlatMaxBlocks blocks (the one-level
// cross-block sums).  The histogram comes into shared memory with one bulk copy where
// that costs no resident block per SM; otherwise each block reads it from global
// memory.
static cudaError_t launch_pass2(gb_metric* m, const EvalArgs& a) {
  const int B = (int)m->bins;
  const size_t plain = mattes_pass2_smem(B);
  const size_t bulk = mattes_pass2_hist_offset(B) + mattes_pass2_hist_bytes(B);
  auto blocks_per_sm = [](size_t smem) {
    int n = 0;
    if (cudaFuncSetAttribute(k_mattes_pass2_affine, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mattes_pass2_affine, kPass2Threads, smem) != cudaSuccess)
      n = 0;
    return n;
  };
  const int n_plain = blocks_per_sm(plain);
  const bool aligned = (reinterpret_cast<uintptr_t>(a.hist) & 15) == 0;
  const int n_bulk = aligned ? blocks_per_sm(bulk) : 0;
  EvalArgs a2 = a;
  a2.hist_bulk = n_bulk >= 1 && n_bulk >= n_plain ? 1 : 0;
  const size_t smem = a2.hist_bulk ? bulk : plain;
  cudaError_t e = cudaFuncSetAttribute(k_mattes_pass2_affine, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = a2.hist_bulk ? n_bulk : n_plain;
  if (per_sm < 1) per_sm = 2;
  const int grid = std::min(grid_for(m, m->nsamples, per_sm), kFlatMaxBlocks);
  return launch_chain(m, k_mattes_pass2_affine, (unsigned)grid, kPass2Threads, smem, a2);
}

// B-spline / composite evaluation: node conversion (large grids), the per-sample
// pass (MeanSquares or Mattes pass 1), then the value (Mattes without the
// derivative: finalize) or the per-chunk and per-parameter reductions.
static int enqueue_eval_bspline(gb_metric* m, const EvalArgs& a, bool cd, bool deriv, bool device_params) {
  const int nper = (int)m->nper;
  const bool sm = a.nodes_smem != 0;
  if (device_params) {  // the host call uploads converted nodes
    GB_CUDA(launch_chain(m, k_prepare_bspline, (unsigned)((nper + kBlock - 1) / kBlock), kBlock, 0, a));
    m->mark();
  }
  const size_t nb = sm ? bspline_node_bytes(m) : 0;
  const bool mattes = m->kind == GB_METRIC_MATTES;
  if (!mattes) {
    cudaError_t e;
    if (cd) e = sm ? launch_wave(m, k_msq_bspline<kGradCentralDifference, true>, nb, a)
                   : launch_wave(m, k_msq_bspline<kGradCentralDifference, false>, nb, a);
    else e = sm ? launch_wave(m, k_msq_bspline<kGradImage, true>, nb, a)
                : launch_wave(m, k_msq_bspline<kGradImage, false>, nb, a);
    GB_CUDA(e);
    m->mark();
  } else {
    const int B = (int)m->bins;
    const size_t sh1 = mattes_bspline_node_offset(B) + nb;
    if (sh1 > 200 * 1024) return fail(GB_ERR_UNSUPPORTED, "histogram too large for shared memory (bins > 160)");
    cudaError_t e;
    if (cd) e = sm ? launch_wave(m, k_mattes_pass1_bspline<kGradCentralDifference, true>, sh1, a)
                   : launch_wave(m, k_mattes_pass1_bspline<kGradCentralDifference, false>, sh1, a);
    else e = sm ? launch_wave(m, k_mattes_pass1_bspline<kGradImage, true>, sh1, a)
                : launch_wave(m, k_mattes_pass1_bspline<kGradImage, false>, sh1, a);
    GB_CUDA(e);
    m->mark();
    if (!deriv) {  // with the derivative the value is formed by the chunk and params kernels
      GB_CUDA(launch_chain(m, k_mattes_finalize, (unsigned)mattes_groups(B), kFinalizeThreads, 0, a));
      m->mark();
    }
  }
  if (!deriv) return GB_OK;
  if (mattes) {  // the derivative's log(p / pm) table
    const int BB = (int)(m->bins * m->bins);
    GB_CUDA(launch_chain(m, k_mattes_table, (unsigned)((BB + kBlock - 1) / kBlock), kBlock, 0, a));
    m->mark();
  }
  // the chunk sums, grid-stride over one full wave (Mattes: at least one block per value
  // group; the table staged in dynamic shared memory)
  const int64_t want = mattes ? std::max<int64_t>(m->nchunks, mattes_groups((int)m->bins)) : m->nchunks;
  if (want > 0) {
    auto kc = mattes ? k_bspline_chunks<true> : k_bspline_chunks<false>;
    const size_t csm = mattes ? sizeof(float) * (size_t)(m->bins * m->bins) : 0;
    GB_CUDA(cudaFuncSetAttribute(kc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csm));
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kc, kChunkLen, csm) != cudaSuccess || per_sm < 1)
      per_sm = 4;
    const int64_t wave = (int64_t)m->ctx->sm_count * per_sm;
    const int64_t cblocks = std::min<int64_t>(want, std::max<int64_t>(wave, mattes ? mattes_groups((int)m->bins) : 1));
    GB_CUDA(launch_chain(m, kc, (unsigned)cblocks, kChunkLen, csm, a));
    m->mark();
  }
  // one warp per node, or one block per node when the nodes hold many chunk entries
  const bool per_block = m->node_entries_count >= (int64_t)kParamsBlock * nper;
  if (per_block) {
    GB_CUDA(mattes ? launch_chain(m, k_bspline_params<true, true>, (unsigned)nper, kParamsBlock, 0, a)
                   : launch_chain(m, k_bspline_params<false, true>, (unsigned)nper, kParamsBlock, 0, a));
  } else {
    const int64_t threads = (int64_t)nper * 32;
    const unsigned pblocks = (unsigned)((threads + kParamsBlock - 1) / kParamsBlock);
    GB_CUDA(mattes ? launch_chain(m, k_bspline_params<true, false>, pblocks, kParamsBlock, 0, a)
                   : launch_chain(m, k_bspline_params<false, false>, pblocks, kParamsBlock, 0, a));
  }
  m->mark();
  return GB_OK;
}

// Displacement-field evaluation: MeanSquares in one pass; Mattes pass 1, the
// value, then the per-sample derivative blocks.  The derivative field is
// cleared first unless every virtual voxel holds a sample (each then stores its
// own block, zeros when invalid).
static int enqueue_eval_field(gb_metric* m, const EvalArgs& a, bool cd, bool deriv) {
  const size_t P = m->tparams.size();
  if (deriv && !a.field_full) GB_CUDA(cudaMemsetAsync(a.out + 2, 0, sizeof(double) * P, m->stream));
  const bool pts = m->use_sampled;
  if (m->kind == GB_METRIC_MEAN_SQUARES) {
    cudaError_t e;
    if (pts) e = cd ? launch_wave(m, k_msq_field<kGradCentralDifference, kMapFieldPoints>, 0, a)
                    : launch_wave(m, k_msq_field<kGradImage, kMapFieldPoints>, 0, a);
    else e = cd ? launch_wave(m, k_msq_field<kGradCentralDifference, kMapFieldDense>, 0, a)
                : launch_wave(m, k_msq_field<kGradImage, kMapFieldDense>, 0, a);
    GB_CUDA(e);
    m->mark();
    return GB_OK;
  }
  const int B = (int)m->bins;
  const size_t sh1 = sizeof(unsigned long long) * (B * B + B) + sizeof(unsigned) * B;
  if (sh1 > 200 * 1024) return fail(GB_ERR_UNSUPPORTED, "histogram too large for shared memory (bins > 160)");
  cudaError_t e;
  if (pts) e = cd ? launch_wave(m, k_mattes_pass1_field<kGradCentralDifference, kMapFieldPoints>, sh1, a)
                  : launch_wave(m, k_mattes_pass1_field<kGradImage, kMapFieldPoints>, sh1, a);
  else e = cd ? launch_wave(m, k_mattes_pass1_field<kGradCentralDifference, kMapFieldDense>, sh1, a)
              : launch_wave(m, k_mattes_pass1_field<kGradImage, kMapFieldDense>, sh1, a);
  GB_CUDA(e);
  m->mark();
  GB_CUDA(launch_chain(m, k_mattes_finalize, (unsigned)mattes_groups(B), kFinalizeThreads, 0, a));
  m->mark();
  if (deriv) {
    const size_t sh2 = sizeof(float) * B * B;
    GB_CUDA(pts ? launch_wave(m, k_mattes_pass2_field<kMapFieldPoints>, sh2, a)
                : launch_wave(m, k_mattes_pass2_field<kMapFieldDense>, sh2, a));
    m->mark();
  }
  return GB_OK;
}

// The B-spline chunk sums and the per-parameter gather of per-sample factors in the
// cache (the MeanSquares form: sums / count).
static int enqueue_bspline_sums(gb_metric* m, const EvalArgs& a) {
  if (m->nchunks > 0) {
    GB_CUDA(launch_chain(m, k_bspline_chunks<false>, (unsigned)m->nchunks, kChunkLen, 0, a));
    m->mark();
  }
  const int nper = (int)m->nper;
  if (m->node_entries_count >= (int64_t)kParamsBlock * nper) {
    GB_CUDA(launch_chain(m, k_bspline_params<false, true>, (unsigned)nper, kParamsBlock, 0, a));
  } else {
    const int64_t threads = (int64_t)nper * 32;
    GB_CUDA(launch_chain(m, k_bspline_params<false, false>, (unsigned)((threads + kParamsBlock - 1) / kParamsBlock),
                         kParamsBlock, 0, a));
  }
  m->mark();
  return GB_OK;
}

// Correlation, B-spline / composite: averages, the sums and value, the per-sample
// factors, the sparse Jacobian sums.
static int enqueue_eval_corr_bspline(gb_metric* m, const EvalArgs& a, bool cd, bool deriv, bool device_params) {
  const bool sm = a.nodes_smem != 0;
  const size_t nb = sm ? bspline_node_bytes(m) : 0;
  if (device_params) {
    GB_CUDA(launch_chain(m, k_prepare_bspline, (unsigned)((m->nper + kBlock - 1) / kBlock), kBlock, 0, a));
    m->mark();
  }
  cudaError_t e;
  if (cd) e = sm ? launch_wave(m, k_corr_mean_bspline<kGradCentralDifference, true>, nb, a)
                 : launch_wave(m, k_corr_mean_bspline<kGradCentralDifference, false>, nb, a);
  else e = sm ? launch_wave(m, k_corr_mean_bspline<kGradImage, true>, nb, a)
              : launch_wave(m, k_corr_mean_bspline<kGradImage, false>, nb, a);
  GB_CUDA(e);
  m->mark();
  if (deriv) e = launch_wave(m, k_corr_sums_bspline<kGradImage, false, false>, 0, a);
  else if (cd) e = sm ? launch_wave(m, k_corr_sums_bspline<kGradCentralDifference, true, true>, nb, a)
                      : launch_wave(m, k_corr_sums_bspline<kGradCentralDifference, false, true>, nb, a);
  else e = sm ? launch_wave(m, k_corr_sums_bspline<kGradImage, true, true>, nb, a)
              : launch_wave(m, k_corr_sums_bspline<kGradImage, false, true>, nb, a);
  GB_CUDA(e);
  m->mark();
  if (!deriv) return GB_OK;
  GB_CUDA(launch_wave(m, k_corr_factor_bspline, 0, a));
  m->mark();
  return enqueue_bspline_sums(m, a);
}

// Joint-histogram MI: the histogram pass, the one-block PDF / value kernel, the
// derivative pass.
static int enqueue_eval_jhmi(gb_metric* m, const EvalArgs& a, bool cd, bool deriv, bool device_params) {
  const int B = (int)m->bins;
  const JhmiConsts* C = reinterpret_cast<const JhmiConsts*>(m->d_jhmi.p);
  const bool bs = is_bspline(m);
  if (is_field(m)) {
    const bool pts = m->use_sampled;
    if (deriv && !a.field_full) GB_CUDA(cudaMemsetAsync(a.out + 2, 0, sizeof(double) * m->tparams.size(), m->stream));
    const size_t sh1 = sizeof(unsigned) * B * B;
    cudaError_t e;
    if (pts) e = cd ? launch_wave(m, k_jhmi_pass1_field<kGradCentralDifference, kMapFieldPoints>, sh1, a, C)
                    : launch_wave(m, k_jhmi_pass1_field<kGradImage, kMapFieldPoints>, sh1, a, C);
    else e = cd ? launch_wave(m, k_jhmi_pass1_field<kGradCentralDifference, kMapFieldDense>, sh1, a, C)
                : launch_wave(m, k_jhmi_pass1_field<kGradImage, kMapFieldDense>, sh1, a, C);
    GB_CUDA(e);
    m->mark();
    const size_t shf = sizeof(double) * (2 * B * B + 2 * B);
    GB_CUDA(cudaFuncSetAttribute(k_jhmi_finalize, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shf));
    GB_CUDA(launch_chain(m, k_jhmi_finalize, (unsigned)kJhmiFinalizeBlocks, kBlock, shf, a, C));
    m->mark();
    if (deriv) {
      const size_t sh2 = sizeof(float) * (B * B + B);
      GB_CUDA(pts ? launch_wave(m, k_jhmi_pass2_field<kMapFieldPoints>, sh2, a, C)
                  : launch_wave(m, k_jhmi_pass2_field<kMapFieldDense>, sh2, a, C));
      m->mark();
    }
    return GB_OK;
  }
  if (bs) {
    const bool sm = a.nodes_smem != 0;
    if (device_params) {  // the host call uploads converted nodes
      GB_CUDA(launch_chain(m, k_prepare_bspline, (unsigned)((m->nper + kBlock - 1) / kBlock), kBlock, 0, a));
      m->mark();
    }
    const size_t sh1 = jhmi_bspline_node_offset(B) + (sm ? bspline_node_bytes(m) : 0);
    cudaError_t e;
    if (cd) e = sm ? launch_wave(m, k_jhmi_pass1_bspline<kGradCentralDifference, true>, sh1, a, C)
                   : launch_wave(m, k_jhmi_pass1_bspline<kGradCentralDifference, false>, sh1, a, C);
    else e = sm ? launch_wave(m, k_jhmi_pass1_bspline<kGradImage, true>, sh1, a, C)
                : launch_wave(m, k_jhmi_pass1_bspline<kGradImage, false>, sh1, a, C);
    GB_CUDA(e);
  } else {
    const size_t sh1 = sizeof(unsigned) * B * B;
    GB_CUDA(cd ? launch_wave(m, k_jhmi_pass1<kGradCentralDifference>, sh1, a, C)
               : launch_wave(m, k_jhmi_pass1<kGradImage>, sh1, a, C));
  }
  m->mark();
  const size_t shf = sizeof(double) * (2 * B * B + 2 * B);
  GB_CUDA(cudaFuncSetAttribute(k_jhmi_finalize, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shf));
  GB_CUDA(launch_chain(m, k_jhmi_finalize, (unsigned)kJhmiFinalizeBlocks, kBlock, shf, a, C));
  m->mark();
  if (deriv && !bs) {
    const size_t sh2 = sizeof(float) * (B * B + B);
    GB_CUDA(cd ? launch_wave(m, k_jhmi_pass2<kGradCentralDifference>, sh2, a, C)
               : launch_wave(m, k_jhmi_pass2<kGradImage>, sh2, a, C));
    m->mark();
  } else if (deriv) {
    // per-sample factors, then the B-spline's sparse Jacobian sums (MeanSquares form)
    const size_t sh2 = sizeof(float) * (B * B + B);
    GB_CUDA(launch_wave(m, k_jhmi_pass2_bspline, sh2, a, C));
    m->mark();
    return enqueue_bspline_sums(m, a);
  }
  return GB_OK;
}

// The evaluation chains whose first kernel can zero the accumulators and whose host
// call can stage its inputs and results through prologue / epilogue kernels.
static bool chain_clears_in_prepare(const gb_metric* m) {
  return (m->kind == GB_METRIC_MATTES || m->kind == GB_METRIC_MEAN_SQUARES) && !is_field(m) && m->nsamples > 0;
}

// Enqueues one evaluation; results land in d_out = [value, nvalid, derivative...].
// device_params: the parameters are in device memory (d_params), so the affine
// constants or the B-spline nodes are formed on the device; otherwise the host
// has uploaded them.
int gb::enqueue_eval(gb_metric* m, const double* d_params, double* d_out, bool deriv, bool device_params,
                     bool acc_cleared) {
  cudaStream_t st = m->stream;
  EvalArgs a;
  fill_eval_args(m, a, d_params, d_out, deriv);
  // MeanSquares / Mattes under an affine or B-spline transform with device parameters:
  // the prepare kernel zeroes the accumulators (one node fewer, and the chain stays
  // kernel-to-kernel); otherwise a memset unless the caller has cleared them
  if (device_params && chain_clears_in_prepare(m)) a.clear_acc = 1;
  else if (!acc_cleared || m->nsamples == 0) GB_CUDA(cudaMemsetAsync(m->d_acc.p, 0, m->acc_bytes, st));
  if (device_params && !is_bspline(m) && !is_field(m))
    GB_CUDA(launch_chain(m, k_prepare_affine, kConstEntries, 32, 0, a, m->d_consts.p));
  if (m->nsamples == 0) {
    // no valid fixed sample at all: every point is invalid
    const int code = GB_ERR_NO_VALID_POINTS;
    GB_CUDA(cudaMemcpyAsync(m->d_status.p, &code, sizeof(int), cudaMemcpyHostToDevice, st));
    const double v[2] = {m->kind != GB_METRIC_MATTES ? DBL_MAX : 0.0, 0.0};
    GB_CUDA(cudaMemcpyAsync(d_out, v, sizeof(v), cudaMemcpyHostToDevice, st));
    if (deriv && !m->tparams.empty()) GB_CUDA(cudaMemsetAsync(d_out + 2, 0, sizeof(double) * m->tparams.size(), st));
    return GB_OK;
  }
  const bool cd = m->grad_source == GB_GRADIENT_CENTRAL_DIFFERENCE;
  m->nevents = 0;
  m->mark();
  if (m->kind == GB_METRIC_JOINT_HISTOGRAM_MI) return enqueue_eval_jhmi(m, a, cd, deriv, device_params);
  if (m->kind == GB_METRIC_CORRELATION && is_bspline(m)) return enqueue_eval_corr_bspline(m, a, cd, deriv, device_params);
  if (is_bspline(m)) return enqueue_eval_bspline(m, a, cd, deriv, device_params);
  if (is_field(m)) return enqueue_eval_field(m, a, cd, deriv);
  if (m->kind == GB_METRIC_CORRELATION) {
    // averages, then the value and derivative (at most kCorrMaxBlocks blocks: 27 partials each)
    GB_CUDA(cd ? launch_wave(m, k_corr_mean_affine<kGradCentralDifference>, 0, a)
               : launch_wave(m, k_corr_mean_affine<kGradImage>, 0, a));
    m->mark();
    const int grid = std::min(kCorrMaxBlocks, cd ? full_wave(m, k_corr_affine<kGradCentralDifference>, 0, m->nsamples)
                                                 : full_wave(m, k_corr_affine<kGradImage>, 0, m->nsamples));
    GB_CUDA(cd ? launch_chain(m, k_corr_affine<kGradCentralDifference>, (unsigned)grid, kBlock, 0, a)
               : launch_chain(m, k_corr_affine<kGradImage>, (unsigned)grid, kBlock, 0, a));
    m->mark();
    return GB_OK;
  }
  if (m->kind == GB_METRIC_MEAN_SQUARES) {
    if (a.fp_res > 0.0)
      GB_CUDA(cd ? launch_wave(m, k_msq_affine<kGradCentralDifference, true>, 0, a)
                 : launch_wave(m, k_msq_affine<kGradImage, true>, 0, a));
    else
      GB_CUDA(cd ? launch_wave(m, k_msq_affine<kGradCentralDifference>, 0, a)
                 : launch_wave(m, k_msq_affine<kGradImage>, 0, a));
    m->mark();
    return GB_OK;
  }
  // Mattes: pass 1, finalize, pass 2
  const int B = (int)m->bins;
  const size_t sh1 = sizeof(unsigned long long) * (B * B + B) + sizeof(unsigned) * B;
  if (sh1 > 200 * 1024) return fail(GB_ERR_UNSUPPORTED, "histogram too large for shared memory (bins > 160)");
  GB_CUDA(cd ? launch_wave(m, k_mattes_pass1_affine<kGradCentralDifference>, sh1, a)
             : launch_wave(m, k_mattes_pass1_affine<kGradImage>, sh1, a));
  m->mark();
  if (!deriv) {  // with the derivative, pass 2 forms the value as well
    GB_CUDA(launch_chain(m, k_mattes_finalize, (unsigned)mattes_groups(B), kFinalizeThreads, 0, a));
    m->mark();
  } else {
    GB_CUDA(launch_pass2(m, a));
    m->mark();
  }
  return GB_OK;
}

extern "C" int gb_metric_set_fault_injection(gb_metric* m, int fault) {
  gb::ErrorScope scope_(m, __func__);
  if (!m) return fail(GB_ERR_BAD_ARG, "null metric");
  if (fault != GB_FAULT_NONE && fault != GB_FAULT_STALLED_COPY) return fail(GB_ERR_BAD_ARG, "unknown fault");
  if (fault != m->inject_fault) m->drop_host_graphs();  // the graphs hold the kernels' arguments
  m->inject_fault = fault;
  return GB_OK;
}

extern "C" int gb_metric_set_profiling(gb_metric* m, int on) {
  gb::ErrorScope scope_(m, __func__);
  if (!m) return fail(GB_ERR_BAD_ARG, "null metric");
  m->profiling = on != 0;
  m->nevents = 0;
  return GB_OK;
}

extern "C" int gb_metric_get_kernel_times(gb_metric* m, double* ms, int max_kernels, int* count) {
  gb::ErrorScope scope_(m, __func__);
  if (!m || !count) return fail(GB_ERR_BAD_ARG, "null argument");
  GB_CUDA(cudaSetDevice(m->ctx->device));
  const int n = m->nevents > 1 ? m->nevents - 1 : 0;
  *count = n;
  if (n == 0) return GB_OK;
  GB_CUDA(cudaEventSynchronize(m->events[m->nevents - 1]));
  for (int i = 0; i < n && i < max_kernels; ++i) {
    float t = 0.f;
    GB_CUDA(cudaEventElapsedTime(&t, m->events[i], m->events[i + 1]));
    if (ms) ms[i] = (double)t;
  }
  return GB_OK;
}

static_assert(sizeof(EvalConsts) % 16 == 0, "the host prologue copies the constants in 16-byte words");

// The host call's prologue: zero the accumulators and bring the constants (affine) or
// float4 nodes (B-spline) from pinned host memory into device memory.
__global__ void k_host_prologue(EvalArgs a, const uint4* src, uint4* dst, int words) {
  griddep_wait();
  griddep_launch_dependents();
  clear_accumulators(a);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < words; k += gridDim.x * blockDim.x) dst[k] = src[k];
}

// The host call's epilogue: value, count, derivative and status into pinned host memory.
__global__ void k_host_epilogue(const double* out, int n, const int* status, double* h_out, int* h_status) {
  griddep_wait();
  griddep_launch_dependents();
  for (int k = threadIdx.x; k < n; k += blockDim.x) h_out[k] = __ldcg(out + k);
  if (threadIdx.x == 0) *h_status = __ldcg(status);
}

// The host call's device work: the constants (affine) or float4 nodes (B-spline)
// up from pinned memory, the evaluation, value / derivative / status down into
// pinned memory.  MeanSquares / Mattes under affine and B-spline transforms do it with
// a prologue and an epilogue kernel (pinned memory read and written by the device), so
// that every node of the chain is a kernel launched with a programmatic dependency;
// the other chains with copies and a memset.
static int host_chain(gb_metric* m, bool deriv) {
  cudaStream_t st = m->stream;
  const size_t P = m->tparams.size();
  if (chain_clears_in_prepare(m)) {
    const void* src = is_bspline(m) ? (const void*)m->h_params : (const void*)m->h_consts;
    void* dst = is_bspline(m) ? (void*)m->d_nodes.p : (void*)m->d_consts.p;
    const size_t bytes = is_bspline(m) ? sizeof(float4) * m->nper : sizeof(EvalConsts);
    void *src_dev = nullptr, *out_dev = nullptr, *status_dev = nullptr;
    GB_CUDA(cudaHostGetDevicePointer(&src_dev, const_cast<void*>(src), 0));
    GB_CUDA(cudaHostGetDevicePointer(&out_dev, m->h_out, 0));
    GB_CUDA(cudaHostGetDevicePointer(&status_dev, m->h_status, 0));
    EvalArgs a;
    fill_eval_args(m, a, nullptr, m->d_out.p, deriv);
    const int words = (int)(bytes / 16);
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(32, (std::max(words, a.acc_words) + 255) / 256));
    GB_CUDA(launch_chain(m, k_host_prologue, grid, 256, 0, a, (const uint4*)src_dev, (uint4*)dst, words));
    int rc = enqueue_eval(m, nullptr, m->d_out.p, deriv, false, true);
    if (rc) return rc;
    GB_CUDA(launch_chain(m, k_host_epilogue, 1u, 256, 0, (const double*)m->d_out.p, (int)(2 + (deriv ? P : 0)),
                         (const int*)m->d_status.p, (double*)out_dev, (int*)status_dev));
    return GB_OK;
  }
  if (is_bspline(m))
    GB_CUDA(cudaMemcpyAsync(m->d_nodes.p, m->h_params, sizeof(float4) * m->nper, cudaMemcpyHostToDevice, st));
  else if (is_field(m))
    GB_CUDA(cudaMemcpyAsync(m->d_params.p, m->h_params, sizeof(double) * P, cudaMemcpyHostToDevice, st));
  else
    GB_CUDA(cudaMemcpyAsync(m->d_consts.p, m->h_consts, sizeof(EvalConsts), cudaMemcpyHostToDevice, st));
  int rc = enqueue_eval(m, nullptr, m->d_out.p, deriv, false);
  if (rc) return rc;
  GB_CUDA(cudaMemcpyAsync(m->h_out, m->d_out.p, sizeof(double) * (2 + (deriv ? P : 0)), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaMemcpyAsync(m->h_status, m->d_status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  return GB_OK;
}

void gb_metric::drop_host_graphs() {
  for (int k = 0; k < 2; ++k) {
    if (host_exec[k]) cudaGraphExecDestroy(host_exec[k]);
    host_exec[k] = nullptr;
    host_graph_tried[k] = false;
  }
}

// host_chain as one CUDA graph per form (value only / with derivative), captured on
// the first call after Initialize: one launch per evaluation instead of about ten
// API calls.  Direct launches when profiling (per-kernel events), when there is no
// sample (that path stages its result from host memory), or if capture fails.
static int run_host_chain(gb_metric* m, bool deriv) {
  const int k = deriv ? 1 : 0;
  if (m->profiling || m->nsamples == 0) return host_chain(m, deriv);
  if (!m->host_exec[k] && !m->host_graph_tried[k]) {
    m->host_graph_tried[k] = true;
    cudaGraph_t g = nullptr;
    bool ok = cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeRelaxed) == cudaSuccess;
    if (ok) {
      const int rc = host_chain(m, deriv);
      const cudaError_t e = cudaStreamEndCapture(m->stream, &g);
      ok = rc == GB_OK && e == cudaSuccess && g != nullptr;
      if (ok) ok = cudaGraphInstantiate(&m->host_exec[k], g, 0) == cudaSuccess;
      if (g) cudaGraphDestroy(g);
    }
    if (!ok) {
      (void)cudaGetLastError();  // a failed capture leaves no sticky error
      m->host_exec[k] = nullptr;
    }
  }
  if (m->host_exec[k]) {
    GB_CUDA(cudaGraphLaunch(m->host_exec[k], m->stream));
    return GB_OK;
  }
  return host_chain(m, deriv);
}

static int eval_host(gb_metric* m, double* value, double* derivative, int64_t nparams, bool deriv) {
  if (!m) return fail(GB_ERR_BAD_ARG, "null metric");
  if (!m->initialized) return fail(GB_ERR_NOT_INITIALIZED, "call gb_metric_initialize first");
  const size_t P = m->tparams.size();
  if (deriv && (size_t)nparams != P) return fail(GB_ERR_BAD_ARG, "derivative size must equal the number of parameters");
  GB_CUDA(cudaSetDevice(m->ctx->device));
  cudaStream_t st = m->stream;
  if (is_bspline(m)) {
    // float4 coefficient nodes converted here (IEEE round to nearest, as the device
    // conversion of the device-resident call), staged in the pinned parameter buffer
    float4* hn = reinterpret_cast<float4*>(m->h_params);
    const int64_t np = m->nper;
    const double* c = m->tparams.data();
    for (int64_t n = 0; n < np; ++n) hn[n] = make_float4((float)c[n], (float)c[np + n], (float)c[2 * np + n], 0.f);
  } else if (is_field(m)) {
    // the field (the parameters), staged in pinned memory for the upload
    copy_parallel(m->h_params, m->tparams.data(), sizeof(double) * P);
  } else {
    // per-evaluation constants in FP64 on the host, uploaded with the parameters
    const bool dense = !m->use_sampled;
    affine_consts(m->tparams.data(), m->tfixed.data(), m->moving.p2i, m->moving.origin, dense ? m->virt.i2p : nullptr,
                  m->virt.origin, *m->h_consts);
  }
  int rc = run_host_chain(m, deriv);
  if (rc) return rc;
  GB_CUDA(cudaStreamSynchronize(st));
  const int status = *m->h_status;
  m->last_status = status;
  m->last_nvalid = (uint64_t)m->h_out[1];
  if (value) *value = m->h_out[0];
  if (deriv) copy_parallel(derivative, m->h_out + 2, sizeof(double) * P);
  if (status == GB_ERR_NO_VALID_POINTS) {
    if (m->kind == GB_METRIC_MATTES)
      return fail(status,
                  "All samples map outside moving image buffer. The images do not sufficiently overlap. They need to "
                  "be initialized to have more overlap before this metric will work. For instance, you can align the "
                  "image centers by translation.");
    return fail(status,
                "No valid points were found during metric evaluation. For image metrics, verify that the images "
                "overlap appropriately.");
  }
  if (status == GB_ERR_JOINT_PDF_SUM_ZERO) return fail(status, "Joint PDF summed to zero");
  if (status == GB_ERR_TIMEOUT)
    return fail(status, "metric evaluation timed out: a streamed copy did not complete within its wait limit");
  if (status != GB_OK) return fail(status, "metric evaluation failed");
  return GB_OK;
}

extern "C" int gb_metric_get_value_and_derivative(gb_metric* m, double* value, double* derivative, int64_t nparams) {
  gb::ErrorScope scope_(m, __func__);
  if (!derivative || !value) return fail(GB_ERR_BAD_ARG, "null output");
  return eval_host(m, value, derivative, nparams, true);
}

extern "C" int gb_metric_get_value(gb_metric* m, double* value) {
  gb::ErrorScope scope_(m, __func__);
  if (!value) return fail(GB_ERR_BAD_ARG, "null output");
  return eval_host(m, value, nullptr, 0, false);
}

extern "C" int gb_metric_get_number_of_valid_points(gb_metric* m, uint64_t* nvalid) {
  gb::ErrorScope scope_(m, __func__);
  if (!m || !nvalid) return fail(GB_ERR_BAD_ARG, "null argument");
  *nvalid = m->last_nvalid;
  return GB_OK;
}

extern "C" int gb_metric_get_number_of_domain_points(gb_metric* m, uint64_t* n) {
  gb::ErrorScope scope_(m, __func__);
  if (!m || !n) return fail(GB_ERR_BAD_ARG, "null argument");
  *n = (uint64_t)m->ndomain;
  return GB_OK;
}

extern "C" int gb_metric_get_joint_pdf(gb_metric* m, double* out, int64_t n) {
  gb::ErrorScope scope_(m, __func__);
  if (!m || !out) return fail(GB_ERR_BAD_ARG, "null argument");
  if (m->kind != GB_METRIC_MATTES && m->kind != GB_METRIC_JOINT_HISTOGRAM_MI)
    return fail(GB_ERR_BAD_ARG, "joint PDF exists for the Mattes and joint-histogram metrics only");
  if (!m->initialized) return fail(GB_ERR_NOT_INITIALIZED, "call gb_metric_initialize first");
  if (n != m->bins * m->bins) return fail(GB_ERR_BAD_ARG, "joint PDF size must be bins*bins");
  GB_CUDA(cudaSetDevice(m->ctx->device));
  GB_CUDA(cudaMemcpyAsync(out, m->d_pdf.p, sizeof(double) * n, cudaMemcpyDeviceToHost, m->stream));
  GB_CUDA(cudaStreamSynchronize(m->stream));
  return GB_OK;
}

extern "C" int gb_metric_get_mattes_state(gb_metric* m, double out8[8]) {
  gb::ErrorScope scope_(m, __func__);
  if (!m || !out8) return fail(GB_ERR_BAD_ARG, "null argument");
  if (m->kind != GB_METRIC_MATTES) return fail(GB_ERR_BAD_ARG, "Mattes metric only");
  for (int i = 0; i < 8; ++i) out8[i] = m->mstate[i];
  return GB_OK;
}

size_t gb_metric::device_bytes() const {
  return d_fixed.bytes() + d_moving.bytes() + d_fixed_s.bytes() + d_moving_s.bytes() + d_grad_in.bytes() +
         d_mov4.bytes() + d_samples.bytes() + d_cache.bytes() + d_sup.bytes() + d_chunks.bytes() +
         d_node_first.bytes() + d_node_entries.bytes() + d_chunk_part.bytes() + d_nodes.bytes() + d_voff.bytes() +
         d_jhmi.bytes() +
         d_params.bytes() +
         d_acc.bytes() + d_scratch.bytes() + d_out.bytes() + d_status.bytes() + d_pratio.bytes() + d_pdf.bytes() +
         d_consts.bytes() + d_opt.bytes() + d_opt_vec.bytes();
}

extern "C" int gb_metric_get_device_bytes(gb_metric* m, uint64_t* bytes) {
  gb::ErrorScope scope_(m, __func__);
  if (!m || !bytes) return fail(GB_ERR_BAD_ARG, "null argument");
  *bytes = (uint64_t)m->device_bytes();
  return GB_OK;
}

extern "C" int gb_metric_get_stream(gb_metric* m, uint64_t* stream) {
  gb::ErrorScope scope_(m, __func__);
  if (!m || !stream) return fail(GB_ERR_BAD_ARG, "null argument");
  *stream = (uint64_t)(uintptr_t)m->stream;
  return GB_OK;
}

extern "C" int gb_metric_evaluate_device(gb_metric* m, const double* device_params, double* device_out,
                                         int with_derivative) {
  gb::ErrorScope scope_(m, __func__);
  if (!m || !device_params || !device_out) return fail(GB_ERR_BAD_ARG, "null argument");
  if (!m->initialized) return fail(GB_ERR_NOT_INITIALIZED, "call gb_metric_initialize first");
  GB_CUDA(cudaSetDevice(m->ctx->device));
  return enqueue_eval(m, device_params, device_out, with_derivative != 0, true);
}

extern "C" int gb_metric_synchronize(gb_metric* m) {
  gb::ErrorScope scope_(m, __func__);
  if (!m) return fail(GB_ERR_BAD_ARG, "null metric");
  GB_CUDA(cudaSetDevice(m->ctx->device));
  GB_CUDA(cudaMemcpyAsync(m->h_status, m->d_status.p, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
  GB_CUDA(cudaStreamSynchronize(m->stream));
  return *m->h_status;
}
