/*
 * itk_oracle.c -- FP64 CPU restatement of ITK's registration-metric hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU library (see itk_oracle.h
 * for the list of reference files restated here, each function below cites
 * the file:line it follows).  Work is split over POSIX threads the way
 * ThreadedIndexedContainerPartitioner splits a sample range into contiguous
 * chunks (Core/Common/src/itkThreadedIndexedContainerPartitioner.cxx:27-57).
 */
#include "itk_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* small helpers                                                       */
/* ------------------------------------------------------------------ */

/* Kahan add, Core/Common/include/itkCompensatedSummation.hxx:38-48 */
static inline void kahan_add(double *sum, double *comp, double element)
{
  const double compensated = element - *comp;
  const double temp = *sum + compensated;
  *comp = (temp - *sum) - compensated;
  *sum = temp;
}

static int inv3(const double a[9], double out[9])
{
  const double c00 = a[4] * a[8] - a[5] * a[7];
  const double c01 = a[5] * a[6] - a[3] * a[8];
  const double c02 = a[3] * a[7] - a[4] * a[6];
  const double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
  if (det == 0.0) return ORC_ERR_BAD_ARG;
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
  return ORC_OK;
}

/* ImageBase::ComputeIndexToPhysicalPointMatrices, Core/Common/include/itkImageBase.hxx:165-180 */
int orc_geom_init(orc_geom *g, const int64_t size[3], const double spacing[3], const double origin[3],
                  const double direction[9])
{
  for (int i = 0; i < 3; ++i) {
    if (size[i] <= 0 || !(spacing[i] > 0.0)) return ORC_ERR_BAD_ARG;
    g->size[i] = size[i];
    g->spacing[i] = spacing[i];
    g->origin[i] = origin[i];
  }
  for (int i = 0; i < 9; ++i) g->direction[i] = direction[i];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) g->i2p[r * 3 + c] = direction[r * 3 + c] * spacing[c];
  return inv3(g->i2p, g->p2i);
}

static void geom_from_flat(orc_geom *g, const int64_t size[3], const double geo[15], int *rc)
{
  *rc = orc_geom_init(g, size, geo, geo + 3, geo + 6);
}

/* ImageBase::TransformPhysicalPointToContinuousIndex, Core/Common/include/itkImageBase.h:515-531 */
static inline void point_to_cindex(const orc_geom *g, const double p[3], double ci[3])
{
  double v[3];
  for (int k = 0; k < 3; ++k) v[k] = p[k] - g->origin[k];
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s += g->p2i[i * 3 + j] * v[j];
    ci[i] = s;
  }
}

/* ImageBase::TransformIndexToPhysicalPoint, Core/Common/include/itkImageBase.h:594-604 */
static inline void index_to_point(const orc_geom *g, const int64_t idx[3], double p[3])
{
  for (int i = 0; i < 3; ++i) {
    p[i] = g->origin[i];
    for (int j = 0; j < 3; ++j) p[i] += g->i2p[i * 3 + j] * (double)idx[j];
  }
}

/* ImageBase::TransformPhysicalPointToIndex (round half up), Core/Common/include/itkImageBase.h:463-479 */
static inline int point_to_index(const orc_geom *g, const double p[3], int64_t idx[3])
{
  int inside = 1;
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s += g->p2i[i * 3 + j] * (p[j] - g->origin[j]);
    idx[i] = (int64_t)floor(s + 0.5);
    if (idx[i] < 0 || idx[i] >= g->size[i]) inside = 0;
  }
  return inside;
}

/* ImageFunction::IsInsideBuffer(ContinuousIndex), Core/Common/../ImageFunction/include/itkImageFunction.h:157-169,
 * bounds [start-0.5, end+0.5) from itkImageFunction.hxx:56-64 */
static inline int inside_buffer(const orc_geom *g, const double ci[3])
{
  for (int j = 0; j < 3; ++j) {
    const double lo = (double)(0 - 0.5);
    const double hi = (double)((g->size[j] - 1) + 0.5);
    if (!(ci[j] >= lo && ci[j] < hi)) return 0;
  }
  return 1;
}

/* LinearInterpolateImageFunction::EvaluateOptimized(Dispatch<3>),
 * Core/ImageFunction/include/itkLinearInterpolateImageFunction.h:227-470.
 * The branchy reference code is equivalent, value for value, to trilinear
 * interpolation with distances clamped to >= 0 and neighbour indices clamped
 * to the buffer end: a skipped axis (distance <= 0 or neighbour past the end)
 * contributes lerp(a, a, d) == a or lerp(a, b, 0) == a exactly. */
static inline void trilinear_setup(const orc_geom *g, const double ci[3], int64_t b0[3], int64_t b1[3], double d[3])
{
  for (int k = 0; k < 3; ++k) {
    int64_t f = (int64_t)floor(ci[k]);
    if (f < 0) f = 0;
    double dist = ci[k] - (double)f;
    b0[k] = f;
    b1[k] = f + 1 <= g->size[k] - 1 ? f + 1 : f;
    if (!(dist > 0.0)) { dist = 0.0; b1[k] = f; }
    d[k] = dist;
  }
}

static inline double interp_scalar(const orc_geom *g, const float *img, const double ci[3])
{
  int64_t b0[3], b1[3];
  double d[3];
  trilinear_setup(g, ci, b0, b1, d);
  const int64_t nx = g->size[0], nxy = g->size[0] * g->size[1];
#define PIX(x, y, z) ((double)img[(x) + (y) * nx + (z) * nxy])
  const double v000 = PIX(b0[0], b0[1], b0[2]), v100 = PIX(b1[0], b0[1], b0[2]);
  const double v010 = PIX(b0[0], b1[1], b0[2]), v110 = PIX(b1[0], b1[1], b0[2]);
  const double v001 = PIX(b0[0], b0[1], b1[2]), v101 = PIX(b1[0], b0[1], b1[2]);
  const double v011 = PIX(b0[0], b1[1], b1[2]), v111 = PIX(b1[0], b1[1], b1[2]);
#undef PIX
  if (d[0] <= 0.0 && d[1] <= 0.0 && d[2] <= 0.0) return v000;
  const double x00 = v000 + (v100 - v000) * d[0];
  const double x10 = v010 + (v110 - v010) * d[0];
  const double x01 = v001 + (v101 - v001) * d[0];
  const double x11 = v011 + (v111 - v011) * d[0];
  const double xx0 = x00 + (x10 - x00) * d[1];
  const double xx1 = x01 + (x11 - x01) * d[1];
  return xx0 + (xx1 - xx0) * d[2];
}

static inline void interp_vec3(const orc_geom *g, const double *img, const double ci[3], double out[3])
{
  int64_t b0[3], b1[3];
  double d[3];
  trilinear_setup(g, ci, b0, b1, d);
  const int64_t nx = g->size[0], nxy = g->size[0] * g->size[1];
  for (int c = 0; c < 3; ++c) {
#define PIX(x, y, z) (img[3 * ((x) + (y) * nx + (z) * nxy) + c])
    const double v000 = PIX(b0[0], b0[1], b0[2]), v100 = PIX(b1[0], b0[1], b0[2]);
    const double v010 = PIX(b0[0], b1[1], b0[2]), v110 = PIX(b1[0], b1[1], b0[2]);
    const double v001 = PIX(b0[0], b0[1], b1[2]), v101 = PIX(b1[0], b0[1], b1[2]);
    const double v011 = PIX(b0[0], b1[1], b1[2]), v111 = PIX(b1[0], b1[1], b1[2]);
#undef PIX
    if (d[0] <= 0.0 && d[1] <= 0.0 && d[2] <= 0.0) { out[c] = v000; continue; }
    const double x00 = v000 + (v100 - v000) * d[0];
    const double x10 = v010 + (v110 - v010) * d[0];
    const double x01 = v001 + (v101 - v001) * d[0];
    const double x11 = v011 + (v111 - v011) * d[0];
    const double xx0 = x00 + (x10 - x00) * d[1];
    const double xx1 = x01 + (x11 - x01) * d[1];
    out[c] = xx0 + (xx1 - xx0) * d[2];
  }
}

int orc_interpolate(const orc_geom *g, const float *img, const double point[3], double *value, int *inside)
{
  double ci[3];
  point_to_cindex(g, point, ci);
  *inside = inside_buffer(g, ci);
  *value = *inside ? interp_scalar(g, img, ci) : 0.0;
  return ORC_OK;
}

/* CentralDifferenceImageFunction::EvaluateSpecialized (scalar pixels, point),
 * Core/ImageFunction/include/itkCentralDifferenceImageFunction.hxx:256-316,
 * with UseImageDirection on (the metric's default calculator,
 * Registration/Metricsv4/include/itkImageToImageMetricv4.hxx:60-61). */
int orc_central_difference(const orc_geom *g, const float *img, const double point[3], double grad[3])
{
  double n1[3] = {point[0], point[1], point[2]};
  double n2[3] = {point[0], point[1], point[2]};
  for (int dim = 0; dim < 3; ++dim) {
    const double off = 0.5 * g->spacing[dim];
    double ci1[3], ci2[3];
    n1[dim] = point[dim] - off;
    point_to_cindex(g, n1, ci1);
    if (!inside_buffer(g, ci1)) {
      grad[dim] = 0.0;
      n1[dim] = point[dim];
      n2[dim] = point[dim];
      continue;
    }
    n2[dim] = point[dim] + off;
    point_to_cindex(g, n2, ci2);
    if (!inside_buffer(g, ci2)) {
      grad[dim] = 0.0;
      n1[dim] = point[dim];
      n2[dim] = point[dim];
      continue;
    }
    const double delta = n2[dim] - n1[dim];
    if (delta > 10.0 * DBL_EPSILON)
      grad[dim] = (interp_scalar(g, img, ci2) - interp_scalar(g, img, ci1)) / delta;
    else
      grad[dim] = 0.0;
    n1[dim] = point[dim];
    n2[dim] = point[dim];
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* cubic B-spline kernels                                              */
/* ------------------------------------------------------------------ */

/* BSplineKernelFunction<3>::Evaluate, Core/Common/include/itkBSplineKernelFunction.h:152-169 */
double orc_bspline3(double u)
{
  const double a = fabs(u);
  if (a < 1.0) {
    const double s = a * a;
    return (4.0 - 6.0 * s + 3.0 * s * a) / 6.0;
  }
  if (a < 2.0) {
    const double s = a * a;
    return (8.0 - 12.0 * a + 6.0 * s - s * a) / 6.0;
  }
  return 0.0;
}

/* BSplineDerivativeKernelFunction<3>::Evaluate, Core/Common/include/itkBSplineDerivativeKernelFunction.h:156-180 */
double orc_bspline3_derivative(double u)
{
  if (u >= 0.0 && u < 1.0) return -2.0 * u + 1.5 * u * u;
  if (u > -1.0 && u < 0.0) return -2.0 * u - 1.5 * u * u;
  if (u >= 1.0 && u < 2.0) return -2.0 + 2.0 * u - 0.5 * u * u;
  if (u > -2.0 && u <= -1.0) return 2.0 + 2.0 * u + 0.5 * u * u;
  return 0.0;
}

/* BSplineInterpolationWeightFunction::Evaluate (order 3, 3-D),
 * Core/Common/include/itkBSplineInterpolationWeightFunction.hxx:43-93.
 * Weight k enumerates the 4x4x4 support x-fastest. */
int orc_bspline_weights(const double ci[3], double weights[64], int64_t start[3])
{
  double w1[3][4];
  for (int j = 0; j < 3; ++j) start[j] = (int64_t)floor(ci[j] + 0.5 - 3.0 / 2.0);
  for (int j = 0; j < 3; ++j) {
    double x = ci[j] - (double)start[j];
    for (int k = 0; k < 4; ++k) {
      w1[j][k] = orc_bspline3(x);
      x -= 1.0;
    }
  }
  for (int k = 0; k < 64; ++k) {
    const int ix = k & 3, iy = (k >> 2) & 3, iz = k >> 4;
    double w = 1.0;
    w *= w1[0][ix];
    w *= w1[1][iy];
    w *= w1[2][iz];
    weights[k] = w;
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* transforms                                                          */
/* ------------------------------------------------------------------ */

/* MatrixOffsetTransformBase::SetParameters + ComputeOffset,
 * Core/Transform/include/itkMatrixOffsetTransformBase.hxx:515-561,612-631 */
static void affine_setup(orc_transform *t, const double p[12], const double c[3])
{
  for (int i = 0; i < 9; ++i) t->M[i] = p[i];
  for (int i = 0; i < 3; ++i) {
    t->translation[i] = p[9 + i];
    t->center[i] = c[i];
  }
  for (int i = 0; i < 3; ++i) {
    double o = t->translation[i] + t->center[i];
    for (int j = 0; j < 3; ++j) o -= t->M[i * 3 + j] * t->center[j];
    t->offset[i] = o;
  }
}

int orc_affine_init(orc_transform *t, const double params12[12], const double center[3])
{
  memset(t, 0, sizeof(*t));
  t->kind = ORC_TRANSFORM_AFFINE;
  affine_setup(t, params12, center);
  return ORC_OK;
}

/* BSplineTransform fixed parameters: grid size, origin, spacing, direction,
 * Core/Transform/include/itkBSplineTransform.hxx:243-283 */
int orc_bspline_init(orc_transform *t, const double f[18], const double *coeff)
{
  memset(t, 0, sizeof(*t));
  t->kind = ORC_TRANSFORM_BSPLINE;
  t->nper = 1;
  for (int i = 0; i < 3; ++i) {
    t->grid[i] = (int64_t)f[i];
    if (t->grid[i] < 4) return ORC_ERR_BAD_ARG;
    t->nper *= t->grid[i];
    t->gorigin[i] = f[3 + i];
    t->gspacing[i] = f[6 + i];
  }
  for (int i = 0; i < 9; ++i) t->gdir[i] = f[9 + i];
  double i2p[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) i2p[r * 3 + c] = t->gdir[r * 3 + c] * t->gspacing[c];
  if (inv3(i2p, t->gp2i) != ORC_OK) return ORC_ERR_BAD_ARG;
  t->coeff = coeff;
  return ORC_OK;
}

int orc_composite_init(orc_transform *t, const double ap[12], const double ac[3], const double f[18],
                       const double *coeff)
{
  int rc = orc_bspline_init(t, f, coeff);
  if (rc) return rc;
  t->kind = ORC_TRANSFORM_COMPOSITE;
  affine_setup(t, ap, ac);
  return ORC_OK;
}

/* DisplacementFieldTransform fixed parameters: size, origin, spacing, direction
 * (Filtering/DisplacementField/include/itkDisplacementFieldTransform.hxx:520-570);
 * the parameters are the field buffer, 3 values per voxel. */
int orc_displacement_init(orc_transform *t, const double f[18], const double *field)
{
  memset(t, 0, sizeof(*t));
  t->kind = ORC_TRANSFORM_DISPLACEMENT;
  int64_t size[3];
  for (int i = 0; i < 3; ++i) {
    if (!(f[i] >= 1.0) || f[i] != floor(f[i])) return ORC_ERR_BAD_ARG;
    size[i] = (int64_t)f[i];
  }
  int rc = orc_geom_init(&t->fgeom, size, f + 6, f + 3, f + 9);
  if (rc) return rc;
  t->nvox = size[0] * size[1] * size[2];
  t->field = field;
  return ORC_OK;
}

int64_t orc_transform_nparams(const orc_transform *t)
{
  if (t->kind == ORC_TRANSFORM_DISPLACEMENT) return 3 * t->nvox;
  return t->kind == ORC_TRANSFORM_AFFINE ? 12 : 3 * t->nper;
}

/* VectorLinearInterpolateImageFunction::EvaluateAtContinuousIndex,
 * Core/ImageFunction/include/itkVectorLinearInterpolateImageFunction.hxx:35-105:
 * the 2^3 neighbours of floor(ci), clamped to the buffer, weighted by their
 * overlap; the loop ends once the overlaps sum to exactly 1. */
static inline void vector_linear(const orc_geom *g, const double *img, const double ci[3], double out[3])
{
  int64_t base[3];
  double dist[3];
  for (int d = 0; d < 3; ++d) {
    base[d] = (int64_t)floor(ci[d]);
    dist[d] = ci[d] - (double)base[d];
  }
  out[0] = out[1] = out[2] = 0.0;
  double total = 0.0;
  const int64_t nx = g->size[0], nxy = g->size[0] * g->size[1];
  for (unsigned counter = 0; counter < 8; ++counter) {
    double overlap = 1.0;
    unsigned upper = counter;
    int64_t nb[3];
    for (int d = 0; d < 3; ++d) {
      if (upper & 1) {
        nb[d] = base[d] + 1 < g->size[d] - 1 ? base[d] + 1 : g->size[d] - 1;
        overlap *= dist[d];
      } else {
        nb[d] = base[d] > 0 ? base[d] : 0;
        overlap *= 1.0 - dist[d];
      }
      upper >>= 1;
    }
    if (overlap != 0.0) {
      const double *px = img + 3 * (nb[0] + nb[1] * nx + nb[2] * nxy);
      for (int k = 0; k < 3; ++k) out[k] += overlap * px[k];
      total += overlap;
    }
    if (total == 1.0) break;
  }
}

/* DisplacementFieldTransform::TransformPoint, itkDisplacementFieldTransform.hxx:67-100:
 * x + field(x) inside the field's buffer, x outside it. */
static inline void displacement_apply(const orc_transform *t, const double x[3], double y[3])
{
  double ci[3];
  point_to_cindex(&t->fgeom, x, ci);
  y[0] = x[0];
  y[1] = x[1];
  y[2] = x[2];
  if (!inside_buffer(&t->fgeom, ci)) return;
  double u[3];
  vector_linear(&t->fgeom, t->field, ci, u);
  for (int k = 0; k < 3; ++k) y[k] += u[k];
}

static inline void affine_apply(const orc_transform *t, const double x[3], double y[3])
{
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s += t->M[i * 3 + j] * x[j];
    y[i] = s + t->offset[i];
  }
}

/* signed-magnitude -> ordered integer, for Math::FloatAlmostEqual / FloatAddULP
 * (Core/Common/include/itkMath.h:274-356) */
static inline int64_t dbl_as_ulp(double x)
{
  int64_t i;
  memcpy(&i, &x, 8);
  if (i < 0) i = (int64_t)0x8000000000000000LL - i;
  return i;
}

static inline int float_almost_equal4(double a, double b)
{
  if (fabs(a - b) <= 0.1 * DBL_EPSILON) return 1;
  if (signbit(a) != signbit(b)) return 0;
  int64_t d = dbl_as_ulp(a) - dbl_as_ulp(b);
  if (d < 0) d = -d;
  return d <= 4;
}

static inline double float_add_ulp(double x, int64_t ulps)
{
  int64_t i;
  memcpy(&i, &x, 8);
  i += ulps;
  double r;
  memcpy(&r, &i, 8);
  return r;
}

/* BSplineTransform::InsideValidRegion, Core/Transform/include/itkBSplineTransform.hxx:478-507 */
static inline int bspline_inside(const orc_transform *t, double ci[3])
{
  const double minLimit = 0.5 * (double)(3 - 1);
  for (int j = 0; j < 3; ++j) {
    const double maxLimit = (double)t->grid[j] - 0.5 * (double)(3 - 1) - 1.0;
    if (float_almost_equal4(ci[j], maxLimit))
      ci[j] = float_add_ulp(maxLimit, -6);
    else if (ci[j] >= maxLimit)
      return 0;
    else if (ci[j] < minLimit)
      return 0;
  }
  return 1;
}

static inline void bspline_cindex(const orc_transform *t, const double p[3], double ci[3])
{
  double v[3];
  for (int k = 0; k < 3; ++k) v[k] = p[k] - t->gorigin[k];
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s += t->gp2i[i * 3 + j] * v[j];
    ci[i] = s;
  }
}

/* BSplineTransform::TransformPoint, Core/Transform/include/itkBSplineTransform.hxx:510-591.
 * Returns 1 when inside the valid region and fills weights / start. */
static inline int bspline_apply(const orc_transform *t, const double x[3], double y[3], double w[64],
                                int64_t start[3])
{
  double ci[3];
  bspline_cindex(t, x, ci);
  if (!bspline_inside(t, ci)) {
    y[0] = x[0]; y[1] = x[1]; y[2] = x[2];
    return 0;
  }
  orc_bspline_weights(ci, w, start);
  double out[3] = {0.0, 0.0, 0.0};
  const int64_t gx = t->grid[0], gxy = t->grid[0] * t->grid[1];
  int k = 0;
  for (int iz = 0; iz < 4; ++iz)
    for (int iy = 0; iy < 4; ++iy)
      for (int ix = 0; ix < 4; ++ix, ++k) {
        const int64_t n = (start[0] + ix) + (start[1] + iy) * gx + (start[2] + iz) * gxy;
        for (int j = 0; j < 3; ++j) out[j] += w[k] * t->coeff[j * t->nper + n];
      }
  for (int j = 0; j < 3; ++j) y[j] = out[j] + x[j];
  return 1;
}

void orc_transform_point(const orc_transform *t, const double x[3], double y[3])
{
  double w[64];
  int64_t st[3];
  if (t->kind == ORC_TRANSFORM_AFFINE) {
    affine_apply(t, x, y);
  } else if (t->kind == ORC_TRANSFORM_DISPLACEMENT) {
    if (t->field_affine) {
      double u[3];
      displacement_apply(t, x, u);
      affine_apply(t, u, y);
    } else {
      displacement_apply(t, x, y);
    }
  } else if (t->kind == ORC_TRANSFORM_BSPLINE) {
    bspline_apply(t, x, y, w, st);
  } else {
    double u[3];
    bspline_apply(t, x, u, w, st);
    affine_apply(t, u, y); /* CompositeTransform applies the queue in reverse, itkCompositeTransform.hxx:60-70 */
  }
}

/* Per-point Jacobian product J^T g in sparse form.  For the affine
 * (itkMatrixOffsetTransformBase.hxx:566-594): J(r, 3r+k) = (x-c)_k, J(r, 9+r) = 1.
 * For the B-spline (itkBSplineTransform.hxx:596-652): J(d, n_k + d*nper) = w_k,
 * zero elsewhere; for the composite the chain rule left-multiplies by the
 * initial affine matrix (itkCompositeTransform.hxx:525-580), so
 * (J^T g)[n_k + d*nper] = w_k (M^T g)_d.  Entries not listed are exactly 0. */
typedef struct {
  int count;
  int64_t idx[192];
  double val[192];
} sparse_row;

/* ------------------------------------------------------------------ */
/* per-point evaluation shared by both metrics                         */
/* ------------------------------------------------------------------ */

typedef struct {
  double fixed_value;  /* FixedImagePixelType: float unless pixel_double */
  double moving_value; /* MovingImagePixelType */
  double grad[3];
  /* Jacobian support */
  int jac_kind; /* 0 affine dense 12, 1 bspline sparse, 2 outside b-spline support (zero), 3 displacement (local) */
  double v[3];  /* x - centre (affine) */
  double w[64];
  int64_t start[3];
} point_eval;

/* ImageToImageMetricv4GetValueAndDerivativeThreaderBase::ProcessVirtualPoint,
 * itkImageToImageMetricv4GetValueAndDerivativeThreaderBase.hxx:176-273, with
 * TransformAndEvaluateFixedPoint / TransformAndEvaluateMovingPoint /
 * ComputeMovingImageGradientAtPoint (itkImageToImageMetricv4.hxx:290-425);
 * the fixed transform is the identity. */
static inline int evaluate_point(const orc_inputs *in, const orc_transform *t, const double vp[3],
                                 int compute_derivative, point_eval *pe)
{
  double ci[3];
  point_to_cindex(&in->fixed_geom, vp, ci);
  if (!inside_buffer(&in->fixed_geom, ci)) return 0;
  pe->fixed_value = interp_scalar(&in->fixed_geom, in->fixed, ci);
  if (!in->pixel_double) pe->fixed_value = (double)(float)pe->fixed_value;

  double mp[3];
  int inside_bs = 0;
  if (t->kind == ORC_TRANSFORM_AFFINE) {
    affine_apply(t, vp, mp);
  } else if (t->kind == ORC_TRANSFORM_DISPLACEMENT) {
    if (t->field_affine) {
      double u[3];
      displacement_apply(t, vp, u);
      affine_apply(t, u, mp); /* CompositeTransform: the field first, then the affine */
    } else {
      displacement_apply(t, vp, mp);
    }
  } else if (t->kind == ORC_TRANSFORM_BSPLINE) {
    inside_bs = bspline_apply(t, vp, mp, pe->w, pe->start);
  } else {
    double u[3];
    inside_bs = bspline_apply(t, vp, u, pe->w, pe->start);
    affine_apply(t, u, mp);
  }
  double mci[3];
  point_to_cindex(&in->moving_geom, mp, mci);
  if (!inside_buffer(&in->moving_geom, mci)) return 0;
  pe->moving_value = interp_scalar(&in->moving_geom, in->moving, mci);
  if (!in->pixel_double) pe->moving_value = (double)(float)pe->moving_value;
  if (compute_derivative) {
    if (in->moving_grad)
      interp_vec3(&in->moving_geom, in->moving_grad, mci, pe->grad);
    else
      orc_central_difference(&in->moving_geom, in->moving, mp, pe->grad);
    if (t->kind == ORC_TRANSFORM_AFFINE) {
      pe->jac_kind = 0;
      for (int k = 0; k < 3; ++k) pe->v[k] = vp[k] - t->center[k];
    } else if (t->kind == ORC_TRANSFORM_DISPLACEMENT) {
      pe->jac_kind = 3; /* identity: J^T g = g at the point's own field voxel */
    } else {
      pe->jac_kind = inside_bs ? 1 : 2;
    }
  }
  return 1;
}

/* Builds the nonzero entries of J^T g for one point. */
static inline void jacobian_product(const orc_transform *t, const point_eval *pe, sparse_row *row)
{
  row->count = 0;
  if (pe->jac_kind == 0) {
    for (int r = 0; r < 3; ++r)
      for (int k = 0; k < 3; ++k) {
        row->idx[row->count] = 3 * r + k;
        row->val[row->count] = pe->v[k] * pe->grad[r];
        row->count++;
      }
    for (int r = 0; r < 3; ++r) {
      row->idx[row->count] = 9 + r;
      row->val[row->count] = pe->grad[r];
      row->count++;
    }
    return;
  }
  if (pe->jac_kind == 2 || pe->jac_kind == 3) return; /* 3: local support, handled by the caller */
  double gd[3];
  if (t->kind == ORC_TRANSFORM_COMPOSITE) {
    /* column d of M * J_bs is M[:,d] w_k; its product with g is w_k (M^T g)_d,
     * summed over dim in the order of the reference's inner product */
    for (int d = 0; d < 3; ++d) {
      double s = 0.0;
      for (int dim = 0; dim < 3; ++dim) s += t->M[dim * 3 + d] * pe->grad[dim];
      gd[d] = s;
    }
  } else {
    for (int d = 0; d < 3; ++d) gd[d] = pe->grad[d];
  }
  const int64_t gx = t->grid[0], gxy = t->grid[0] * t->grid[1];
  int k = 0;
  for (int iz = 0; iz < 4; ++iz)
    for (int iy = 0; iy < 4; ++iy)
      for (int ix = 0; ix < 4; ++ix, ++k) {
        const int64_t n = (pe->start[0] + ix) + (pe->start[1] + iy) * gx + (pe->start[2] + iz) * gxy;
        for (int d = 0; d < 3; ++d) {
          row->idx[row->count] = n + d * t->nper;
          row->val[row->count] = pe->w[k] * gd[d];
          row->count++;
        }
      }
}

static inline int64_t domain_size(const orc_inputs *in)
{
  if (in->points) return in->npoints;
  return in->virtual_geom.size[0] * in->virtual_geom.size[1] * in->virtual_geom.size[2];
}

static inline void domain_point(const orc_inputs *in, int64_t i, double vp[3])
{
  if (in->points) {
    vp[0] = (double)in->points[3 * i + 0];
    vp[1] = (double)in->points[3 * i + 1];
    vp[2] = (double)in->points[3 * i + 2];
  } else {
    const int64_t nx = in->virtual_geom.size[0], ny = in->virtual_geom.size[1];
    int64_t idx[3] = {i % nx, (i / nx) % ny, i / (nx * ny)};
    index_to_point(&in->virtual_geom, idx, vp);
  }
}

/* J^T g of a displacement field's local parameters: g, or M^T g behind an initial
 * affine (the composite's chain rule, itkCompositeTransform.hxx:525-580) */
static inline void field_grad(const orc_transform *t, const double g[3], double out[3])
{
  for (int d = 0; d < 3; ++d) {
    if (!t->field_affine) {
      out[d] = g[d];
      continue;
    }
    double s = 0.0;
    for (int dim = 0; dim < 3; ++dim) s += t->M[dim * 3 + d] * g[dim];
    out[d] = s;
  }
}

/* ComputeParameterOffsetFromVirtualIndex (Numerics/Optimizersv4/include/itkObjectToObjectMetric.hxx:332-343):
 * the point's virtual index (its own index for the dense domain,
 * TransformPhysicalPointToIndex for a point set) times 3.  -1 for a point set
 * point whose nearest index lies outside the virtual grid (the reference
 * indexes past the derivative there; such points add nothing here). */
static inline int64_t local_offset(const orc_inputs *in, int64_t i, const double vp[3])
{
  if (!in->points) return 3 * i;
  int64_t idx[3];
  if (!point_to_index(&in->virtual_geom, vp, idx)) return -1;
  return 3 * (idx[0] + in->virtual_geom.size[0] * (idx[1] + in->virtual_geom.size[1] * idx[2]));
}

/* VerifyDisplacementFieldSizeAndPhysicalSpace, itkObjectToObjectMetric.hxx:444-503 */
static int verify_field_domain(const orc_inputs *in, const orc_transform *t)
{
  if (t->kind != ORC_TRANSFORM_DISPLACEMENT) return ORC_OK;
  const orc_geom *v = &in->virtual_geom, *f = &t->fgeom;
  for (int i = 0; i < 3; ++i)
    if (v->size[i] != f->size[i]) return ORC_ERR_BAD_ARG;
  const double ctol = 1.0e-6 * v->spacing[0];
  for (int i = 0; i < 3; ++i)
    if (fabs(v->origin[i] - f->origin[i]) > ctol || fabs(v->spacing[i] - f->spacing[i]) > ctol) return ORC_ERR_BAD_ARG;
  for (int i = 0; i < 9; ++i)
    if (fabs(v->direction[i] - f->direction[i]) > 1.0e-6) return ORC_ERR_BAD_ARG;
  return ORC_OK;
}

static int resolve_threads(int requested, int64_t n)
{
  int t = requested > 0 ? requested : 1;
  if (t > 256) t = 256;
  if ((int64_t)t > n) t = (int)(n > 0 ? n : 1);
  return t;
}

/* ------------------------------------------------------------------ */
/* MeanSquares                                                         */
/* ------------------------------------------------------------------ */

typedef struct {
  const orc_inputs *in;
  const orc_transform *t;
  int compute_derivative;
  int64_t begin, end;
  double measure;
  uint64_t nvalid;
  int64_t nparams;
  double *dsum, *dcomp; /* per-thread compensated derivatives */
  int64_t *loff;        /* local support: per point, the derivative offset (-1: none) */
  double *lval;         /* local support: per point, 3 local derivatives */
} msq_job;

/* MeanSquaresImageToImageMetricv4GetValueAndDerivativeThreader::ProcessPoint,
 * itkMeanSquaresImageToImageMetricv4GetValueAndDerivativeThreader.hxx:31-84,
 * accumulated as in StorePointDerivativeResult (ThreaderBase.hxx:278-300) */
static void *msq_worker(void *arg)
{
  msq_job *j = (msq_job *)arg;
  point_eval pe;
  sparse_row row;
  for (int64_t i = j->begin; i < j->end; ++i) {
    double vp[3];
    domain_point(j->in, i, vp);
    if (!evaluate_point(j->in, j->t, vp, j->compute_derivative, &pe)) continue;
    /* diff is computed in FixedImagePixelType (float for Image<float,3>) */
    const double diffC = j->in->pixel_double ? pe.fixed_value - pe.moving_value
                                             : (double)((float)pe.fixed_value - (float)pe.moving_value);
    j->measure += diffC * diffC;
    j->nvalid++;
    if (!j->compute_derivative) continue;
    if (j->loff) {
      /* local support: the point's own derivative block, stored at its offset
       * afterwards (StorePointDerivativeResult, ThreaderBase.hxx:301-320) */
      j->loff[i - j->begin] = local_offset(j->in, i, vp);
      double gd[3];
      field_grad(j->t, pe.grad, gd);
      for (int d = 0; d < 3; ++d) j->lval[3 * (i - j->begin) + d] = 2.0 * diffC * gd[d];
      continue;
    }
    jacobian_product(j->t, &pe, &row);
    for (int e = 0; e < row.count; ++e) {
      /* localDerivative[par] = sum_dim 2.0 * diff * J(dim,par) * g[dim]; with one
       * nonzero J entry per (par, dim) pair for affine rows and B-spline rows */
      double ld = 2.0 * diffC * row.val[e];
      if (j->in->fp_resolution > 0.0) {
        /* UseFloatingPointCorrection: each local derivative truncated to the resolution
         * before it is added (StorePointDerivativeResult, ThreaderBase.hxx:284-294) */
        const double r = j->in->fp_resolution;
        ld = (double)(int64_t)(ld * r) / r;
      }
      kahan_add(&j->dsum[row.idx[e]], &j->dcomp[row.idx[e]], ld);
    }
  }
  return NULL;
}

int orc_msq_value_derivative(const orc_inputs *in, const orc_transform *t, int compute_derivative,
                             double *value, double *derivative, uint64_t *nvalid)
{
  const int64_t n = domain_size(in);
  const int64_t P = orc_transform_nparams(t);
  if (n < 1) return ORC_ERR_BAD_ARG;
  if (verify_field_domain(in, t)) return ORC_ERR_BAD_ARG;
  const int local = t->kind == ORC_TRANSFORM_DISPLACEMENT;
  const int T = resolve_threads(in->nthreads, n);
  msq_job *jobs = (msq_job *)calloc((size_t)T, sizeof(msq_job));
  pthread_t *th = (pthread_t *)calloc((size_t)T, sizeof(pthread_t));
  if (!jobs || !th) { free(jobs); free(th); return ORC_ERR_OOM; }
  const int64_t chunk = (n + T - 1) / T;
  int rc = ORC_OK;
  for (int k = 0; k < T; ++k) {
    jobs[k].in = in;
    jobs[k].t = t;
    jobs[k].compute_derivative = compute_derivative;
    jobs[k].begin = k * chunk < n ? k * chunk : n;
    jobs[k].end = (k + 1) * chunk < n ? (k + 1) * chunk : n;
    jobs[k].nparams = P;
    if (compute_derivative && local) {
      const int64_t len = jobs[k].end - jobs[k].begin;
      jobs[k].loff = (int64_t *)malloc(sizeof(int64_t) * (size_t)(len > 0 ? len : 1));
      jobs[k].lval = (double *)malloc(sizeof(double) * 3 * (size_t)(len > 0 ? len : 1));
      if (!jobs[k].loff || !jobs[k].lval) rc = ORC_ERR_OOM;
      for (int64_t q = 0; jobs[k].loff && q < len; ++q) jobs[k].loff[q] = -1;
    } else if (compute_derivative) {
      jobs[k].dsum = (double *)calloc((size_t)P, sizeof(double));
      jobs[k].dcomp = (double *)calloc((size_t)P, sizeof(double));
      if (!jobs[k].dsum || !jobs[k].dcomp) rc = ORC_ERR_OOM;
    }
  }
  if (rc == ORC_OK) {
    for (int k = 0; k < T; ++k) pthread_create(&th[k], NULL, msq_worker, &jobs[k]);
    for (int k = 0; k < T; ++k) pthread_join(th[k], NULL);
    /* AfterThreadedExecution, ThreaderBase.hxx:116-172 */
    uint64_t nv = 0;
    for (int k = 0; k < T; ++k) nv += jobs[k].nvalid;
    *nvalid = nv;
    if (compute_derivative && local) {
      /* local support: Derivatives[offset + i] += LocalDerivatives[i] in point
       * order, no averaging (ThreaderBase.hxx:128-172,301-320) */
      for (int64_t p = 0; p < P; ++p) derivative[p] = 0.0;
      for (int k = 0; k < T; ++k)
        for (int64_t q = 0; q < jobs[k].end - jobs[k].begin; ++q) {
          const int64_t o = jobs[k].loff[q];
          if (o < 0) continue;
          for (int d = 0; d < 3; ++d) derivative[o + d] += jobs[k].lval[3 * q + d];
        }
    } else if (compute_derivative) {
      for (int64_t p = 0; p < P; ++p) {
        double s = 0.0, c = 0.0;
        for (int k = 0; k < T; ++k) kahan_add(&s, &c, jobs[k].dsum[p]);
        derivative[p] = 0.0 + s;
      }
    }
    if (nv == 0) {
      /* VerifyNumberOfValidPoints, Numerics/Optimizersv4/include/itkObjectToObjectMetric.hxx:512-527 */
      *value = DBL_MAX;
      if (compute_derivative)
        for (int64_t p = 0; p < P; ++p) derivative[p] = 0.0;
      rc = ORC_ERR_NO_VALID_POINTS;
    } else {
      double v = 0.0;
      for (int k = 0; k < T; ++k) v += jobs[k].measure;
      *value = v / (double)nv;
      if (compute_derivative && !local)
        for (int64_t p = 0; p < P; ++p) derivative[p] /= (double)nv;
    }
  }
  for (int k = 0; k < T; ++k) { free(jobs[k].dsum); free(jobs[k].dcomp); free(jobs[k].loff); free(jobs[k].lval); }
  free(jobs);
  free(th);
  return rc;
}

/* ------------------------------------------------------------------ */
/* Correlation (normalized cross correlation)                          */
/* ------------------------------------------------------------------ */

typedef struct {
  const orc_inputs *in;
  const orc_transform *t;
  int compute_derivative;
  int64_t begin, end;
  double avg_f, avg_m;         /* helper pass: inputs of the main pass */
  double fix_sum, mov_sum;     /* helper pass: outputs */
  double f, m, f2, m2, fm;     /* main pass */
  uint64_t nvalid;
  int64_t nparams;
  double *fdm, *mdm;
} corr_job;

/* CorrelationImageToImageMetricv4HelperThreader::ProcessVirtualPoint,
 * itkCorrelationImageToImageMetricv4HelperThreader.hxx:104-169: sums of the
 * fixed and moving values over the valid points */
static void *corr_helper_worker(void *arg)
{
  corr_job *j = (corr_job *)arg;
  point_eval pe;
  for (int64_t i = j->begin; i < j->end; ++i) {
    double vp[3];
    domain_point(j->in, i, vp);
    if (!evaluate_point(j->in, j->t, vp, 0, &pe)) continue;
    j->fix_sum += pe.fixed_value;
    j->mov_sum += pe.moving_value;
    j->nvalid++;
  }
  return NULL;
}

/* CorrelationImageToImageMetricv4GetValueAndDerivativeThreader::ProcessPoint,
 * itkCorrelationImageToImageMetricv4GetValueAndDerivativeThreader.hxx:270-325 */
static void *corr_worker(void *arg)
{
  corr_job *j = (corr_job *)arg;
  point_eval pe;
  sparse_row row;
  for (int64_t i = j->begin; i < j->end; ++i) {
    double vp[3];
    domain_point(j->in, i, vp);
    if (!evaluate_point(j->in, j->t, vp, j->compute_derivative, &pe)) continue;
    const double f1 = pe.fixed_value - j->avg_f;
    const double m1 = pe.moving_value - j->avg_m;
    j->f += f1;
    j->m += m1;
    j->f2 += f1 * f1;
    j->m2 += m1 * m1;
    j->fm += f1 * m1;
    j->nvalid++;
    if (!j->compute_derivative) continue;
    /* one nonzero J(dim, par) per parameter for affine and B-spline rows, so the
     * row entry is sum_dim g[dim] J(dim, par) */
    jacobian_product(j->t, &pe, &row);
    for (int e = 0; e < row.count; ++e) {
      j->fdm[row.idx[e]] += f1 * row.val[e];
      j->mdm[row.idx[e]] += m1 * row.val[e];
    }
  }
  return NULL;
}

static int corr_run(corr_job *jobs, int T, void *(*fn)(void *))
{
  pthread_t *th = (pthread_t *)calloc((size_t)T, sizeof(pthread_t));
  if (!th) return ORC_ERR_OOM;
  for (int k = 0; k < T; ++k) pthread_create(&th[k], NULL, fn, &jobs[k]);
  for (int k = 0; k < T; ++k) pthread_join(th[k], NULL);
  free(th);
  return ORC_OK;
}

/* CorrelationImageToImageMetricv4: InitializeForIteration's helper pass for the
 * averages (itkCorrelationImageToImageMetricv4.hxx:69-116,
 * ...HelperThreader.hxx:58-100), then the value and derivative
 * (...GetValueAndDerivativeThreader.hxx:62-130):
 *   value = -fm^2 / (f2 m2),  derivative = 2 fm / (f2 m2) (fdm - fm / m2 mdm),
 * value 0 and a zero derivative when m2 f2 <= epsilon; no valid point: the
 * MeanSquares-style warning (value DBL_MAX, zero derivative). */
int orc_corr_value_derivative(const orc_inputs *in, const orc_transform *t, int compute_derivative, double *value,
                              double *derivative, uint64_t *nvalid)
{
  const int64_t n = domain_size(in);
  const int64_t P = orc_transform_nparams(t);
  if (n < 1) return ORC_ERR_BAD_ARG;
  if (t->kind == ORC_TRANSFORM_DISPLACEMENT) return ORC_ERR_BAD_ARG; /* global-support transforms only here */
  const int T = resolve_threads(in->nthreads, n);
  corr_job *jobs = (corr_job *)calloc((size_t)T, sizeof(corr_job));
  if (!jobs) return ORC_ERR_OOM;
  const int64_t chunk = (n + T - 1) / T;
  int rc = ORC_OK;
  for (int k = 0; k < T; ++k) {
    jobs[k].in = in;
    jobs[k].t = t;
    jobs[k].compute_derivative = compute_derivative;
    jobs[k].begin = k * chunk < n ? k * chunk : n;
    jobs[k].end = (k + 1) * chunk < n ? (k + 1) * chunk : n;
    jobs[k].nparams = P;
    if (compute_derivative) {
      jobs[k].fdm = (double *)calloc((size_t)P, sizeof(double));
      jobs[k].mdm = (double *)calloc((size_t)P, sizeof(double));
      if (!jobs[k].fdm || !jobs[k].mdm) rc = ORC_ERR_OOM;
    }
  }
  if (rc == ORC_OK) rc = corr_run(jobs, T, corr_helper_worker);
  if (compute_derivative)
    for (int64_t p = 0; p < P; ++p) derivative[p] = 0.0;
  *value = 0.0;
  if (rc == ORC_OK) {
    uint64_t nh = 0;
    double sum_f = 0.0, sum_m = 0.0;
    for (int k = 0; k < T; ++k) {
      nh += jobs[k].nvalid;
      sum_f += jobs[k].fix_sum;
      sum_m += jobs[k].mov_sum;
    }
    const double avg_f = nh > 0 ? sum_f / (double)nh : 0.0;
    const double avg_m = nh > 0 ? sum_m / (double)nh : 0.0;
    for (int k = 0; k < T; ++k) {
      jobs[k].avg_f = avg_f;
      jobs[k].avg_m = avg_m;
      jobs[k].nvalid = 0;
    }
    rc = corr_run(jobs, T, corr_worker);
  }
  if (rc == ORC_OK) {
    uint64_t nv = 0;
    for (int k = 0; k < T; ++k) nv += jobs[k].nvalid;
    *nvalid = nv;
    if (nv == 0) {
      *value = DBL_MAX;
      rc = ORC_ERR_NO_VALID_POINTS;
    } else {
      double fm = 0.0, f2 = 0.0, m2 = 0.0;
      for (int k = 0; k < T; ++k) {
        fm += jobs[k].fm;
        m2 += jobs[k].m2;
        f2 += jobs[k].f2;
      }
      const double m2f2 = m2 * f2;
      if (m2f2 > DBL_EPSILON) {
        *value = -1.0 * fm * fm / m2f2;
        if (compute_derivative) {
          for (int64_t p = 0; p < P; ++p) {
            double fd = 0.0, md = 0.0;
            for (int k = 0; k < T; ++k) {
              fd += jobs[k].fdm[p];
              md += jobs[k].mdm[p];
            }
            derivative[p] += 2.0 * fm / (f2 * m2) * (fd - fm / m2 * md);
          }
        }
      }
    }
  }
  for (int k = 0; k < T; ++k) { free(jobs[k].fdm); free(jobs[k].mdm); }
  free(jobs);
  return rc;
}

/* ------------------------------------------------------------------ */
/* Mattes mutual information                                           */
/* ------------------------------------------------------------------ */

/* MattesMutualInformationImageToImageMetricv4::Initialize,
 * itkMattesMutualInformationImageToImageMetricv4.hxx:75-327 (no masks; the
 * sampled point set, when present, is in virtual space with an identity
 * fixed transform). */
int orc_mattes_initialize(const orc_inputs *in, int64_t bins, orc_mattes_state *st)
{
  if (bins < 5) bins = 5; /* itkSetClampMacro(NumberOfHistogramBins, ..., 5, max), .h:146 */
  st->bins = bins;
  double fmin = (double)FLT_MAX, fmax = -(double)FLT_MAX;
  if (in->points) {
    for (int64_t i = 0; i < in->npoints; ++i) {
      double p[3] = {in->points[3 * i], in->points[3 * i + 1], in->points[3 * i + 2]};
      int64_t idx[3];
      if (point_to_index(&in->fixed_geom, p, idx)) {
        const double v = (double)in->fixed[idx[0] + idx[1] * in->fixed_geom.size[0] +
                                           idx[2] * in->fixed_geom.size[0] * in->fixed_geom.size[1]];
        fmin = fmin < v ? fmin : v;
        fmax = fmax > v ? fmax : v;
      }
    }
  } else {
    const int64_t nv = in->fixed_geom.size[0] * in->fixed_geom.size[1] * in->fixed_geom.size[2];
    for (int64_t i = 0; i < nv; ++i) {
      const double v = (double)in->fixed[i];
      fmin = fmin < v ? fmin : v;
      fmax = fmax > v ? fmax : v;
    }
  }
  double mmin = (double)FLT_MAX, mmax = -(double)FLT_MAX;
  {
    const int64_t nv = in->moving_geom.size[0] * in->moving_geom.size[1] * in->moving_geom.size[2];
    for (int64_t i = 0; i < nv; ++i) {
      const double v = (double)in->moving[i];
      mmin = mmin < v ? mmin : v;
      mmax = mmax > v ? mmax : v;
    }
  }
  st->fixed_true_min = fmin;
  st->fixed_true_max = fmax;
  st->moving_true_min = mmin;
  st->moving_true_max = mmax;
  if (fmax < fmin) return ORC_ERR_FIXED_EMPTY;
  if (fmax - fmin <= DBL_EPSILON) return ORC_ERR_FIXED_CONSTANT;
  if (mmax < mmin) return ORC_ERR_MOVING_EMPTY;
  if (mmax - mmin <= DBL_EPSILON) return ORC_ERR_MOVING_CONSTANT;
  const int padding = 2;
  st->fixed_bin_size = (fmax - fmin) / (double)(bins - 2 * padding);
  st->fixed_normalized_min = fmin / st->fixed_bin_size - (double)padding;
  st->moving_bin_size = (mmax - mmin) / (double)(bins - 2 * padding);
  st->moving_normalized_min = mmin / st->moving_bin_size - (double)padding;
  return ORC_OK;
}

/* ComputeSingleFixedImageParzenWindowIndex, itkMattesMutualInformationImageToImageMetricv4.hxx:571-597 */
static inline int64_t fixed_parzen_index(const orc_mattes_state *st, double value)
{
  const double term = value / st->fixed_bin_size - st->fixed_normalized_min;
  int64_t p = (int64_t)term;
  if (p < 2) p = 2;
  else if (p > st->bins - 3) p = st->bins - 3;
  return p;
}

typedef struct {
  const orc_inputs *in;
  const orc_mattes_state *st;
  const orc_transform *t;
  int compute_derivative;
  int64_t begin, end;
  uint64_t nvalid;
  int64_t nparams;
  double *pdf;      /* bins*bins */
  double *fmarg;    /* bins */
  double *pdfd;     /* [f][m][P] */
  int64_t *loff;    /* local support: per point, the derivative offset (-1: none) */
  int64_t *lidx;    /* local support: per point, JointPdfIndex1D of its first moving bin */
  double *lval;     /* local support: per point, [bin][d] local derivative by Parzen bin */
} mattes_job;

/* MattesMutualInformationImageToImageMetricv4GetValueAndDerivativeThreader::ProcessPoint,
 * itkMattesMutualInformationImageToImageMetricv4GetValueAndDerivativeThreader.hxx:220-387
 * (global-support transforms).  Derivative rows go straight into this thread's
 * JointPDFDerivatives, which is what the reference's DerivativeBufferManager
 * eventually adds into the shared array (.hxx:610-757); the per-thread arrays
 * are summed afterwards. */
static void *mattes_worker(void *arg)
{
  mattes_job *j = (mattes_job *)arg;
  const orc_mattes_state *st = j->st;
  const int64_t bins = st->bins;
  const int64_t P = j->nparams;
  point_eval pe;
  sparse_row row;
  for (int64_t i = j->begin; i < j->end; ++i) {
    double vp[3];
    domain_point(j->in, i, vp);
    if (!evaluate_point(j->in, j->t, vp, j->compute_derivative, &pe)) continue;
    const double mv = pe.moving_value;
    if (mv < st->moving_true_min) continue;
    if (mv > st->moving_true_max) continue;
    const double mterm = mv / st->moving_bin_size - st->moving_normalized_min;
    int64_t midx = (int64_t)mterm;
    if (midx < 2) midx = 2;
    else if (midx > bins - 3) midx = bins - 3;
    int64_t pdfm = midx - 1;
    const int64_t pdfmax = midx + 2;
    const int64_t fidx = fixed_parzen_index(st, pe.fixed_value);
    j->fmarg[fidx] += 1;
    double arg = (double)pdfm - mterm;
    double *pdfrow = j->pdf + fidx * bins + pdfm;
    const int64_t q = i - j->begin;
    if (j->compute_derivative && j->loff) {
      /* local support (Mattes...Threader.hxx:300-312): the point's offset and joint-PDF index */
      j->loff[q] = local_offset(j->in, i, vp);
      j->lidx[q] = pdfm + fidx * bins;
    } else if (j->compute_derivative) {
      jacobian_product(j->t, &pe, &row);
    }
    int bin = 0;
    while (pdfm <= pdfmax) {
      const double val = orc_bspline3(arg);
      *(pdfrow++) += val;
      if (j->compute_derivative && j->loff) {
        /* ComputePDFDerivativesLocalSupportTransform (.hxx:394-412) with the
         * identity Jacobian: innerProduct = g[mu] */
        const double dval = orc_bspline3_derivative(arg);
        double gd[3];
        field_grad(j->t, pe.grad, gd);
        for (int d = 0; d < 3; ++d) j->lval[12 * q + 3 * bin + d] = gd[d] * dval;
      } else if (j->compute_derivative) {
        const double dval = orc_bspline3_derivative(arg);
        double *dst = j->pdfd + (fidx * bins + pdfm) * P;
        for (int e = 0; e < row.count; ++e) dst[row.idx[e]] += row.val[e] * dval;
      }
      arg += 1.0;
      ++pdfm;
      ++bin;
    }
    j->nvalid++;
  }
  return NULL;
}

int orc_mattes_value_derivative(const orc_inputs *in, const orc_mattes_state *st, const orc_transform *t,
                                int compute_derivative, double *value, double *derivative, uint64_t *nvalid,
                                double *joint_pdf)
{
  const int64_t n = domain_size(in);
  const int64_t P = orc_transform_nparams(t);
  const int64_t bins = st->bins;
  if (n < 1) return ORC_ERR_BAD_ARG;
  if (verify_field_domain(in, t)) return ORC_ERR_BAD_ARG;
  const int local = t->kind == ORC_TRANSFORM_DISPLACEMENT;
  int T = resolve_threads(in->nthreads, n);
  /* bound the per-thread derivative arrays to ~2 GB in total */
  if (compute_derivative && !local) {
    const double per = (double)P * (double)(bins * bins) * 8.0;
    while (T > 1 && per * T > 2.0e9) --T;
  }
  mattes_job *jobs = (mattes_job *)calloc((size_t)T, sizeof(mattes_job));
  pthread_t *th = (pthread_t *)calloc((size_t)T, sizeof(pthread_t));
  if (!jobs || !th) { free(jobs); free(th); return ORC_ERR_OOM; }
  const int64_t chunk = (n + T - 1) / T;
  int rc = ORC_OK;
  for (int k = 0; k < T; ++k) {
    jobs[k].in = in;
    jobs[k].st = st;
    jobs[k].t = t;
    jobs[k].compute_derivative = compute_derivative;
    jobs[k].begin = k * chunk < n ? k * chunk : n;
    jobs[k].end = (k + 1) * chunk < n ? (k + 1) * chunk : n;
    jobs[k].nparams = P;
    jobs[k].pdf = (double *)calloc((size_t)(bins * bins), sizeof(double));
    jobs[k].fmarg = (double *)calloc((size_t)bins, sizeof(double));
    if (compute_derivative && local) {
      const int64_t len = jobs[k].end - jobs[k].begin > 0 ? jobs[k].end - jobs[k].begin : 1;
      jobs[k].loff = (int64_t *)malloc(sizeof(int64_t) * (size_t)len);
      jobs[k].lidx = (int64_t *)malloc(sizeof(int64_t) * (size_t)len);
      jobs[k].lval = (double *)calloc((size_t)(12 * len), sizeof(double));
      if (!jobs[k].loff || !jobs[k].lidx || !jobs[k].lval) rc = ORC_ERR_OOM;
      for (int64_t q = 0; jobs[k].loff && q < len; ++q) jobs[k].loff[q] = -1;
    } else if (compute_derivative) {
      jobs[k].pdfd = (double *)calloc((size_t)(bins * bins * P), sizeof(double));
      if (!jobs[k].pdfd) rc = ORC_ERR_OOM;
    }
    if (!jobs[k].pdf || !jobs[k].fmarg) rc = ORC_ERR_OOM;
  }
  if (rc == ORC_OK) {
    for (int k = 0; k < T; ++k) pthread_create(&th[k], NULL, mattes_worker, &jobs[k]);
    for (int k = 0; k < T; ++k) pthread_join(th[k], NULL);

    /* AfterThreadedExecution, Mattes...Threader.hxx:418-463 */
    uint64_t nv = 0;
    for (int k = 0; k < T; ++k) nv += jobs[k].nvalid;
    *nvalid = nv;
    /* GetValueCommonAfterThreadedExecution, Mattes...v4.hxx:512-542 */
    double *pdf = jobs[0].pdf, *fm = jobs[0].fmarg;
    for (int k = 1; k < T; ++k) {
      for (int64_t i = 0; i < bins * bins; ++i) pdf[i] += jobs[k].pdf[i];
      for (int64_t i = 0; i < bins; ++i) fm[i] += jobs[k].fmarg[i];
    }
    double jsum = 0.0, jc = 0.0;
    for (int64_t i = 0; i < bins * bins; ++i) kahan_add(&jsum, &jc, pdf[i]);
    double *pdfd = NULL;
    double *lbin = NULL;    /* local support: m_LocalDerivativeByParzenBin[4][P] */
    int64_t *l1d = NULL;    /* local support: m_JointPdfIndex1DArray[P] */
    if (compute_derivative && local) {
      /* the points' blocks in point order: by-bin sums add up, the joint-PDF
       * index is the last point's (Mattes...Threader.hxx:300-312,340-351) */
      lbin = (double *)calloc((size_t)(4 * P), sizeof(double));
      l1d = (int64_t *)calloc((size_t)P, sizeof(int64_t));
      if (!lbin || !l1d) rc = ORC_ERR_OOM;
      for (int k = 0; rc == ORC_OK && k < T; ++k)
        for (int64_t q = 0; q < jobs[k].end - jobs[k].begin; ++q) {
          const int64_t o = jobs[k].loff[q];
          if (o < 0) continue;
          for (int b = 0; b < 4; ++b)
            for (int d = 0; d < 3; ++d) lbin[b * P + o + d] += jobs[k].lval[12 * q + 3 * b + d];
          for (int d = 0; d < 3; ++d) l1d[o + d] = jobs[k].lidx[q];
        }
    } else if (compute_derivative) {
      pdfd = jobs[0].pdfd;
      for (int k = 1; k < T; ++k)
        for (int64_t i = 0; i < bins * bins * P; ++i) pdfd[i] += jobs[k].pdfd[i];
      if (nv > 0) {
        const double nFactor = -1.0 / (st->moving_bin_size * (double)nv);
        for (int64_t i = 0; i < bins * bins * P; ++i) pdfd[i] *= nFactor;
      }
    }
    /* ComputeResults, Mattes...v4.hxx:358-499 */
    if (rc != ORC_OK) {
      /* allocation failure above: no result */
    } else if (nv == 0) {
      rc = ORC_ERR_NO_VALID_POINTS;
    } else if (jsum < DBL_EPSILON) {
      rc = ORC_ERR_JOINT_PDF_SUM_ZERO;
    } else {
      const double nf = 1.0 / jsum;
      for (int64_t i = 0; i < bins * bins; ++i) pdf[i] = pdf[i] * nf;
      for (int64_t i = 0; i < bins; ++i) fm[i] = fm[i] * nf;
      double *mm = (double *)calloc((size_t)bins, sizeof(double));
      if (!mm) {
        rc = ORC_ERR_OOM;
      } else {
        for (int64_t m = 0; m < bins; ++m) {
          double s = 0.0;
          for (int64_t f = 0; f < bins; ++f) s += pdf[f * bins + m];
          mm[m] = s;
        }
        if (compute_derivative)
          for (int64_t p = 0; p < P; ++p) derivative[p] = 0.0;
        const double closeToZero = DBL_EPSILON;
        /* local support: m_PRatioArray, zero where a bin is skipped; nFactor = 1 / (binsize N) */
        double *pra = local && compute_derivative ? (double *)calloc((size_t)(bins * bins), sizeof(double)) : NULL;
        const double nFactorLocal = 1.0 / (st->moving_bin_size * (double)nv);
        double sum = 0.0;
        for (int64_t f = 0; f < bins; ++f) {
          const double fpdf = fm[f];
          if (!(fpdf > closeToZero)) continue;
          const double logf = log(fpdf);
          for (int64_t m = 0; m < bins; ++m) {
            const double mp = mm[m];
            const double jp = pdf[f * bins + m];
            if (mp > closeToZero && jp > closeToZero) {
              const double pRatio = log(jp / mp);
              sum += jp * (pRatio - logf);
              if (compute_derivative && local) {
                if (pra) pra[f * bins + m] = pRatio * nFactorLocal;
              } else if (compute_derivative) {
                const double *dp = pdfd + (f * bins + m) * P;
                for (int64_t p = 0; p < P; ++p) derivative[p] += dp[p] * pRatio;
              }
            }
          }
        }
        if (compute_derivative && local) {
          /* Mattes...v4.hxx:478-495: derivative[i] -= LocalDerivativeByParzenBin[bin][i] * PRatio[index1D + bin] */
          if (!pra) {
            rc = ORC_ERR_OOM;
          } else {
            for (int64_t i = 0; i < P; ++i)
              for (int b = 0; b < 4; ++b) derivative[i] -= lbin[b * P + i] * pra[l1d[i] + b];
          }
          free(pra);
        }
        *value = -1.0 * sum;
        free(mm);
      }
    }
    if (joint_pdf) memcpy(joint_pdf, pdf, sizeof(double) * (size_t)(bins * bins));
    free(lbin);
    free(l1d);
  }
  for (int k = 0; k < T; ++k) {
    free(jobs[k].pdf); free(jobs[k].fmarg); free(jobs[k].pdfd);
    free(jobs[k].loff); free(jobs[k].lidx); free(jobs[k].lval);
  }
  free(jobs);
  free(th);
  return rc;
}

/* ------------------------------------------------------------------ */
/* flat wrappers                                                       */
/* ------------------------------------------------------------------ */

int orc_transform_from_flat(orc_transform *t, int tkind, const double *tparams, int64_t nparams,
                            const double *tfixed, int64_t nfixed)
{
  if (tkind == ORC_TRANSFORM_AFFINE) {
    if (nparams != 12 || nfixed != 3) return ORC_ERR_BAD_ARG;
    return orc_affine_init(t, tparams, tfixed);
  }
  if (tkind == ORC_TRANSFORM_BSPLINE) {
    if (nfixed != 18) return ORC_ERR_BAD_ARG;
    int rc = orc_bspline_init(t, tfixed, tparams);
    if (rc) return rc;
    return nparams == 3 * t->nper ? ORC_OK : ORC_ERR_BAD_ARG;
  }
  if (tkind == ORC_TRANSFORM_DISPLACEMENT) {
    if (nfixed != 18 && nfixed != 33) return ORC_ERR_BAD_ARG;
    int rc = orc_displacement_init(t, tfixed, tparams);
    if (rc) return rc;
    if (nfixed == 33) {
      affine_setup(t, tfixed + 18, tfixed + 30);
      t->field_affine = 1;
    }
    return nparams == 3 * t->nvox ? ORC_OK : ORC_ERR_BAD_ARG;
  }
  if (tkind == ORC_TRANSFORM_COMPOSITE) {
    if (nfixed != 33) return ORC_ERR_BAD_ARG;
    int rc = orc_composite_init(t, tfixed + 18, tfixed + 30, tfixed, tparams);
    if (rc) return rc;
    return nparams == 3 * t->nper ? ORC_OK : ORC_ERR_BAD_ARG;
  }
  return ORC_ERR_BAD_ARG;
}

static int inputs_from_flat(orc_inputs *in, const float *fixed, const int64_t fsize[3], const double fgeo[15],
                            const float *moving, const int64_t msize[3], const double mgeo[15],
                            const double *moving_grad, const float *points, int64_t npoints, int nthreads,
                            const int64_t *vsize, const double *vgeo)
{
  int rc;
  memset(in, 0, sizeof(*in));
  geom_from_flat(&in->fixed_geom, fsize, fgeo, &rc);
  if (rc) return rc;
  geom_from_flat(&in->moving_geom, msize, mgeo, &rc);
  if (rc) return rc;
  in->virtual_geom = in->fixed_geom; /* virtual domain defaults to the fixed image, itkImageToImageMetricv4.hxx:98-112 */
  if (vsize) {
    geom_from_flat(&in->virtual_geom, vsize, vgeo, &rc);
    if (rc) return rc;
  }
  in->fixed = fixed;
  in->moving = moving;
  in->moving_grad = moving_grad;
  in->points = points;
  in->npoints = points ? npoints : 0;
  in->nthreads = nthreads & 0xffff;
  in->pixel_double = (nthreads >> 16) & 1;
  return ORC_OK;
}

int orc_msq_flat(const float *fixed, const int64_t fsize[3], const double fgeo[15], const float *moving,
                 const int64_t msize[3], const double mgeo[15], const double *moving_grad, const float *points,
                 int64_t npoints, int tkind, const double *tparams, int64_t nparams, const double *tfixed,
                 int64_t nfixed, int nthreads, int compute_derivative, double *value, double *derivative,
                 uint64_t *nvalid)
{
  return orc_msq_flat_v(fixed, fsize, fgeo, moving, msize, mgeo, moving_grad, points, npoints, tkind, tparams,
                        nparams, tfixed, nfixed, nthreads, compute_derivative, value, derivative, nvalid, NULL,
                        NULL);
}

int orc_msq_flat_fpc(const float *fixed, const int64_t fsize[3], const double fgeo[15], const float *moving,
                     const int64_t msize[3], const double mgeo[15], const double *moving_grad, const float *points,
                     int64_t npoints, int tkind, const double *tparams, int64_t nparams, const double *tfixed,
                     int64_t nfixed, int nthreads, int compute_derivative, double *value, double *derivative,
                     uint64_t *nvalid, double resolution)
{
  orc_inputs in;
  orc_transform t;
  int rc = inputs_from_flat(&in, fixed, fsize, fgeo, moving, msize, mgeo, moving_grad, points, npoints, nthreads,
                            NULL, NULL);
  if (rc) return rc;
  in.fp_resolution = resolution;
  rc = orc_transform_from_flat(&t, tkind, tparams, nparams, tfixed, nfixed);
  if (rc) return rc;
  return orc_msq_value_derivative(&in, &t, compute_derivative, value, derivative, nvalid);
}

int orc_msq_flat_v(const float *fixed, const int64_t fsize[3], const double fgeo[15], const float *moving,
                   const int64_t msize[3], const double mgeo[15], const double *moving_grad, const float *points,
                   int64_t npoints, int tkind, const double *tparams, int64_t nparams, const double *tfixed,
                   int64_t nfixed, int nthreads, int compute_derivative, double *value, double *derivative,
                   uint64_t *nvalid, const int64_t *vsize, const double *vgeo)
{
  orc_inputs in;
  orc_transform t;
  int rc = inputs_from_flat(&in, fixed, fsize, fgeo, moving, msize, mgeo, moving_grad, points, npoints, nthreads,
                            vsize, vgeo);
  if (rc) return rc;
  rc = orc_transform_from_flat(&t, tkind, tparams, nparams, tfixed, nfixed);
  if (rc) return rc;
  return orc_msq_value_derivative(&in, &t, compute_derivative, value, derivative, nvalid);
}

int orc_corr_flat_v(const float *fixed, const int64_t fsize[3], const double fgeo[15], const float *moving,
                    const int64_t msize[3], const double mgeo[15], const double *moving_grad, const float *points,
                    int64_t npoints, int tkind, const double *tparams, int64_t nparams, const double *tfixed,
                    int64_t nfixed, int nthreads, int compute_derivative, double *value, double *derivative,
                    uint64_t *nvalid, const int64_t *vsize, const double *vgeo)
{
  orc_inputs in;
  orc_transform t;
  int rc = inputs_from_flat(&in, fixed, fsize, fgeo, moving, msize, mgeo, moving_grad, points, npoints, nthreads,
                            vsize, vgeo);
  if (rc) return rc;
  rc = orc_transform_from_flat(&t, tkind, tparams, nparams, tfixed, nfixed);
  if (rc) return rc;
  return orc_corr_value_derivative(&in, &t, compute_derivative, value, derivative, nvalid);
}

int orc_mattes_flat(const float *fixed, const int64_t fsize[3], const double fgeo[15], const float *moving,
                    const int64_t msize[3], const double mgeo[15], const double *moving_grad, const float *points,
                    int64_t npoints, int tkind, const double *tparams, int64_t nparams, const double *tfixed,
                    int64_t nfixed, int64_t bins, int nthreads, int compute_derivative, double *value,
                    double *derivative, uint64_t *nvalid, double *joint_pdf, double *state_out)
{
  return orc_mattes_flat_v(fixed, fsize, fgeo, moving, msize, mgeo, moving_grad, points, npoints, tkind, tparams,
                           nparams, tfixed, nfixed, bins, nthreads, compute_derivative, value, derivative, nvalid,
                           joint_pdf, state_out, NULL, NULL);
}

int orc_mattes_flat_v(const float *fixed, const int64_t fsize[3], const double fgeo[15], const float *moving,
                      const int64_t msize[3], const double mgeo[15], const double *moving_grad, const float *points,
                      int64_t npoints, int tkind, const double *tparams, int64_t nparams, const double *tfixed,
                      int64_t nfixed, int64_t bins, int nthreads, int compute_derivative, double *value,
                      double *derivative, uint64_t *nvalid, double *joint_pdf, double *state_out,
                      const int64_t *vsize, const double *vgeo)
{
  orc_inputs in;
  orc_transform t;
  orc_mattes_state st;
  int rc = inputs_from_flat(&in, fixed, fsize, fgeo, moving, msize, mgeo, moving_grad, points, npoints, nthreads,
                            vsize, vgeo);
  if (rc) return rc;
  rc = orc_transform_from_flat(&t, tkind, tparams, nparams, tfixed, nfixed);
  if (rc) return rc;
  rc = orc_mattes_initialize(&in, bins, &st);
  if (state_out) {
    state_out[0] = st.fixed_true_min;
    state_out[1] = st.fixed_true_max;
    state_out[2] = st.moving_true_min;
    state_out[3] = st.moving_true_max;
    state_out[4] = st.fixed_bin_size;
    state_out[5] = st.moving_bin_size;
    state_out[6] = st.fixed_normalized_min;
    state_out[7] = st.moving_normalized_min;
  }
  if (rc) return rc;
  return orc_mattes_value_derivative(&in, &st, &t, compute_derivative, value, derivative, nvalid, joint_pdf);
}

int orc_transform_point_flat(int tkind, const double *tparams, int64_t nparams, const double *tfixed,
                             int64_t nfixed, const double *x, int64_t n, double *y)
{
  orc_transform t;
  int rc = orc_transform_from_flat(&t, tkind, tparams, nparams, tfixed, nfixed);
  if (rc) return rc;
  for (int64_t i = 0; i < n; ++i) orc_transform_point(&t, x + 3 * i, y + 3 * i);
  return ORC_OK;
}

int orc_interpolate_flat(const float *img, const int64_t size[3], const double geo[15], const double *points,
                         int64_t n, double *values, int *inside)
{
  orc_geom g;
  int rc;
  geom_from_flat(&g, size, geo, &rc);
  if (rc) return rc;
  for (int64_t i = 0; i < n; ++i) orc_interpolate(&g, img, points + 3 * i, values + i, inside + i);
  return ORC_OK;
}

int orc_central_difference_flat(const float *img, const int64_t size[3], const double geo[15],
                                const double *points, int64_t n, double *grads)
{
  orc_geom g;
  int rc;
  geom_from_flat(&g, size, geo, &rc);
  if (rc) return rc;
  for (int64_t i = 0; i < n; ++i) orc_central_difference(&g, img, points + 3 * i, grads + 3 * i);
  return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* JointHistogramMutualInformationImageToImageMetricv4                 */
/* ------------------------------------------------------------------ */

/* Modified Bessel functions of the first kind for the discrete Gaussian kernel
 * (GaussianOperator, Core/Common/include/itkGaussianOperator.hxx:27-180): the
 * polynomial approximations of Abramowitz & Stegun 9.8.1-9.8.4 for orders 0
 * and 1, and Miller's downward recurrence (normalized by I0) for order n >= 2,
 * as published in Numerical Recipes (bessi, accuracy parameter 40, rescaling
 * at 1e10). */
static double bessel_i0(double y)
{
  const double d = fabs(y);
  if (d < 3.75) {
    double t = y / 3.75;
    t *= t;
    return 1.0 + t * (3.5156229 + t * (3.0899424 + t * (1.2067492 + t * (0.2659732 + t * (0.0360768 + t * 0.0045813)))));
  }
  const double t = 3.75 / d;
  return (exp(d) / sqrt(d)) *
         (0.39894228 + t * (0.01328592 + t * (0.00225319 + t * (-0.00157565 + t * (0.00916281 +
          t * (-0.02057706 + t * (0.02635537 + t * (-0.01647633 + t * 0.00392377))))))));
}

static double bessel_i1(double y)
{
  const double d = fabs(y);
  double r;
  if (d < 3.75) {
    double t = y / 3.75;
    t *= t;
    r = d * (0.5 + t * (0.87890594 + t * (0.51498869 + t * (0.15084934 + t * (0.02658733 + t * (0.00301532 +
                                                                                               t * 0.00032411))))));
  } else {
    const double t = 3.75 / d;
    double q = 0.02282967 + t * (-0.02895312 + t * (0.01787654 - t * 0.00420059));
    q = 0.39894228 + t * (-0.03988024 + t * (-0.00362018 + t * (0.00163801 + t * (-0.01031555 + t * q))));
    r = q * (exp(d) / sqrt(d));
  }
  return y < 0.0 ? -r : r;
}

static double bessel_in(int n, double y)
{
  if (y == 0.0) return 0.0;
  const double tox = 2.0 / fabs(y);
  double bip = 0.0, bi = 1.0, ans = 0.0;
  for (int j = 2 * (n + (int)sqrt(40.0 * n)); j > 0; j--) {
    const double bim = bip + j * tox * bi;
    bip = bi;
    bi = bim;
    if (fabs(bi) > 1.0e10) {
      ans *= 1.0e-10;
      bi *= 1.0e-10;
      bip *= 1.0e-10;
    }
    if (j == n) ans = bip;
  }
  ans *= bessel_i0(y) / bi;
  return (y < 0.0 && (n & 1)) ? -ans : ans;
}

/* GaussianOperator::GenerateCoefficients: e^-v I_k(v) for k = 0, 1, ... until the
 * two-sided sum reaches 1 - max_error (or the width limit), normalized by that
 * sum, mirrored.  Returns the radius; c holds 2 r + 1 coefficients. */
int orc_gaussian_kernel(double variance, double max_error, int max_width, double *c, int cap)
{
  double half[64];
  const double et = exp(-variance);
  int n = 0;
  half[n++] = et * bessel_i0(variance);
  double sum = half[0];
  half[n++] = et * bessel_i1(variance);
  sum += half[1] * 2.0;
  const double limit = 1.0 - max_error;
  for (int i = 2; sum < limit && n < 64; ++i) {
    half[n++] = et * bessel_in(i, variance);
    sum += half[i] * 2.0;
    if (half[i] <= 0.0) break;
    if (n > max_width) break;
  }
  for (int i = 0; i < n; ++i) half[i] /= sum;
  const int r = n - 1;
  if (2 * r + 1 > cap) return -1;
  for (int i = 0; i <= r; ++i) {
    c[r + i] = half[i];
    c[r - i] = half[i];
  }
  return r;
}

/* One separable pass of DiscreteGaussianImageFilter over a bins x bins image
 * along axis `dir` (0: the fixed index, x fastest; 1: the moving index), zero-flux
 * Neumann boundary (ZeroFluxNeumannBoundaryCondition: indices clamped), the
 * neighbourhood inner product in operator order. */
static void gauss_pass(const double *in, double *out, int64_t B, int dir, const double *c, int r)
{
  for (int64_t j = 0; j < B; ++j)
    for (int64_t i = 0; i < B; ++i) {
      double s = 0.0;
      for (int k = 0; k <= 2 * r; ++k) {
        int64_t q = (dir == 0 ? i : j) + k - r;
        q = q < 0 ? 0 : (q > B - 1 ? B - 1 : q);
        s += c[k] * (dir == 0 ? in[q + B * j] : in[i + B * q]);
      }
      out[i + B * j] = s;
    }
}

/* LinearInterpolateImageFunction on the bins x bins joint PDF (2-D path) and the
 * 1-D marginal, at a continuous index; neighbours clamped as in 3-D. */
static double interp2(const double *img, int64_t B, const double ci[2])
{
  int64_t b0[2], b1[2];
  double d[2];
  for (int k = 0; k < 2; ++k) {
    int64_t f = (int64_t)floor(ci[k]);
    if (f < 0) f = 0;
    double dist = ci[k] - (double)f;
    b0[k] = f;
    b1[k] = f + 1 <= B - 1 ? f + 1 : f;
    if (!(dist > 0.0)) { dist = 0.0; b1[k] = f; }
    d[k] = dist;
  }
  const double v00 = img[b0[0] + B * b0[1]], v10 = img[b1[0] + B * b0[1]];
  const double v01 = img[b0[0] + B * b1[1]], v11 = img[b1[0] + B * b1[1]];
  if (d[0] <= 0.0 && d[1] <= 0.0) return v00;
  const double x0 = v00 + (v10 - v00) * d[0];
  const double x1 = v01 + (v11 - v01) * d[0];
  return x0 + (x1 - x0) * d[1];
}

static double interp1(const double *v, int64_t B, double ci)
{
  int64_t f = (int64_t)floor(ci);
  if (f < 0) f = 0;
  double dist = ci - (double)f;
  int64_t g = f + 1 <= B - 1 ? f + 1 : f;
  if (!(dist > 0.0)) return v[f];
  return v[f] + (v[g] - v[f]) * dist;
}

/* Initialize: true min / max over the whole fixed and moving images
 * (itkJointHistogramMutualInformationImageToImageMetricv4.hxx:70-135), joint PDF
 * geometry: spacing 1 / (bins - 2 padding - 1), origin -padding * spacing
 * (.hxx:147-163). */
int orc_jhmi_initialize(const orc_inputs *in, int64_t bins, double variance, orc_jhmi_state *st)
{
  if (bins < 6) return ORC_ERR_BAD_ARG;
  st->bins = bins;
  st->variance = variance;
  double fmin = (double)FLT_MAX, fmax = -(double)FLT_MAX, mmin = (double)FLT_MAX, mmax = -(double)FLT_MAX;
  const int64_t nf = in->fixed_geom.size[0] * in->fixed_geom.size[1] * in->fixed_geom.size[2];
  for (int64_t i = 0; i < nf; ++i) {
    const double v = (double)in->fixed[i];
    fmin = v < fmin ? v : fmin;
    fmax = v > fmax ? v : fmax;
  }
  const int64_t nm = in->moving_geom.size[0] * in->moving_geom.size[1] * in->moving_geom.size[2];
  for (int64_t i = 0; i < nm; ++i) {
    const double v = (double)in->moving[i];
    mmin = v < mmin ? v : mmin;
    mmax = v > mmax ? v : mmax;
  }
  st->fmin = fmin;
  st->fmax = fmax;
  st->mmin = mmin;
  st->mmax = mmax;
  st->spacing = 1.0 / (double)(bins - 2 * 2 - 1);
  st->origin = st->spacing * 2.0 * -1.0;
  st->inv_spacing = 1.0 / st->spacing; /* PhysicalPointToIndex of the diagonal joint-PDF geometry */
  return ORC_OK;
}

/* ComputeJointPDFPoint (.hxx:389-401) */
static inline void jhmi_point(const orc_jhmi_state *st, double f, double m, double p[2])
{
  p[0] = (f - st->fmin) / (st->fmax - st->fmin);
  p[1] = (m - st->mmin) / (st->mmax - st->mmin);
}

typedef struct {
  const orc_inputs *in;
  const orc_transform *t;
  const orc_jhmi_state *st;
  int64_t begin, end;
  /* pass 1 */
  uint64_t *hist;
  uint64_t count;
  /* pass 2 */
  const double *pdf, *mmarg;
  double *dsum, *dcomp;
  uint64_t nvalid;
  int64_t nparams;
  int64_t *loff; /* local support: per point, the derivative offset (-1: none) */
  double *lval;  /* local support: per point, 3 local derivatives */
} jhmi_job;

/* JointHistogramMutualInformationComputeJointPDFThreaderBase::ProcessPoint
 * (...ComputeJointPDFThreaderBase.hxx:57-104): valid fixed and moving values,
 * TransformPhysicalPointToIndex on the joint histogram, count inside it. */
static void *jhmi_hist_worker(void *arg)
{
  jhmi_job *j = (jhmi_job *)arg;
  const int64_t B = j->st->bins;
  point_eval pe;
  for (int64_t i = j->begin; i < j->end; ++i) {
    double vp[3];
    domain_point(j->in, i, vp);
    if (!evaluate_point(j->in, j->t, vp, 0, &pe)) continue;
    double p[2];
    jhmi_point(j->st, pe.fixed_value, pe.moving_value, p);
    int64_t idx[2];
    int inside = 1;
    for (int k = 0; k < 2; ++k) {
      const double s = (p[k] - j->st->origin) * j->st->inv_spacing;
      idx[k] = (int64_t)floor(s + 0.5);
      if (!(s == s) || idx[k] < 0 || idx[k] >= B) inside = 0;
    }
    if (!inside) continue;
    j->hist[idx[0] + B * idx[1]]++;
    j->count++;
  }
  return NULL;
}

/* JointHistogramMutualInformationGetValueAndDerivativeThreader::ProcessPoint and
 * its PDF derivatives (...GetValueAndDerivativeThreader.hxx:94-277). */
static void *jhmi_deriv_worker(void *arg)
{
  jhmi_job *j = (jhmi_job *)arg;
  const orc_jhmi_state *st = j->st;
  const int64_t B = st->bins;
  const double s = st->spacing, eps = 1.0e-16;
  const double max_slope = -log(eps) / s;
  const double mrange = st->mmax - st->mmin;
  const double log2 = log(2.0);
  point_eval pe;
  sparse_row row;
  for (int64_t i = j->begin; i < j->end; ++i) {
    double vp[3];
    domain_point(j->in, i, vp);
    if (!evaluate_point(j->in, j->t, vp, 1, &pe)) continue;
    if (pe.moving_value < st->mmin || pe.moving_value > st->mmax) continue;
    double p[2];
    jhmi_point(st, pe.fixed_value, pe.moving_value, p);
    double ci[2];
    int inside = 1;
    for (int k = 0; k < 2; ++k) {
      ci[k] = (p[k] - st->origin) * st->inv_spacing;
      if (!(ci[k] >= -0.5 && ci[k] < (double)B - 0.5)) inside = 0;
    }
    if (!inside) continue;
    const double jv = interp2(j->pdf, B, ci);
    /* ComputeJointPDFDerivative along the moving axis: +-0.5 spacing, clamped to [spacing, 1] */
    double l = p[1] - 0.5 * s, r = p[1] + 0.5 * s;
    l = l < s ? s : (l > 1.0 ? 1.0 : l);
    r = r < s ? s : (r > 1.0 ? 1.0 : r);
    double dj = 0.0;
    if (r - l > 0.0) {
      const double cl[2] = {ci[0], (l - st->origin) * st->inv_spacing};
      const double cr[2] = {ci[0], (r - st->origin) * st->inv_spacing};
      dj = (interp2(j->pdf, B, cr) - interp2(j->pdf, B, cl)) / (r - l);
    }
    const double mv = interp1(j->mmarg, B, ci[1]);
    double dm = 0.0;
    if (r - l > 0.0)
      dm = (interp1(j->mmarg, B, (r - st->origin) * st->inv_spacing) -
            interp1(j->mmarg, B, (l - st->origin) * st->inv_spacing)) / (r - l);
    double sf = 0.0;
    if (jv > eps && mv > eps) {
      double t1 = dj / jv, t2 = dm / mv;
      t1 = t1 < -max_slope ? -max_slope : (t1 > max_slope ? max_slope : t1);
      t2 = t2 < -max_slope ? -max_slope : (t2 > max_slope ? max_slope : t2);
      sf = (t1 - t2) / (log2 * mrange);
    }
    j->nvalid++;
    if (j->loff) {
      /* local support: sf J^T g stored at the point's voxel afterwards, not averaged */
      double gd[3];
      field_grad(j->t, pe.grad, gd);
      j->loff[i - j->begin] = local_offset(j->in, i, vp);
      for (int d = 0; d < 3; ++d) j->lval[3 * (i - j->begin) + d] = sf * gd[d];
      continue;
    }
    jacobian_product(j->t, &pe, &row);
    for (int e = 0; e < row.count; ++e) kahan_add(&j->dsum[row.idx[e]], &j->dcomp[row.idx[e]], sf * row.val[e]);
  }
  return NULL;
}

int orc_jhmi_value_derivative(const orc_inputs *in, const orc_jhmi_state *st, const orc_transform *t,
                              int compute_derivative, double *value, double *derivative, uint64_t *nvalid,
                              double *joint_pdf)
{
  const int64_t n = domain_size(in);
  const int64_t P = orc_transform_nparams(t);
  const int64_t B = st->bins;
  if (n < 1) return ORC_ERR_BAD_ARG;
  if (verify_field_domain(in, t)) return ORC_ERR_BAD_ARG;
  const int local = t->kind == ORC_TRANSFORM_DISPLACEMENT;
  const int T = resolve_threads(in->nthreads, n);
  jhmi_job *jobs = (jhmi_job *)calloc((size_t)T, sizeof(jhmi_job));
  pthread_t *th = (pthread_t *)calloc((size_t)T, sizeof(pthread_t));
  double *pdf = (double *)calloc((size_t)(B * B), sizeof(double));
  double *tmp = (double *)calloc((size_t)(B * B), sizeof(double));
  double *fmarg = (double *)calloc((size_t)B, sizeof(double));
  double *mmarg = (double *)calloc((size_t)B, sizeof(double));
  int rc = (jobs && th && pdf && tmp && fmarg && mmarg) ? ORC_OK : ORC_ERR_OOM;
  const int64_t chunk = (n + T - 1) / T;
  for (int k = 0; rc == ORC_OK && k < T; ++k) {
    jobs[k].in = in;
    jobs[k].t = t;
    jobs[k].st = st;
    jobs[k].begin = k * chunk < n ? k * chunk : n;
    jobs[k].end = (k + 1) * chunk < n ? (k + 1) * chunk : n;
    jobs[k].nparams = P;
    jobs[k].hist = (uint64_t *)calloc((size_t)(B * B), sizeof(uint64_t));
    if (!jobs[k].hist) rc = ORC_ERR_OOM;
  }
  uint64_t count = 0;
  if (rc == ORC_OK) {
    /* InitializeForIteration (.hxx:207-303): the joint histogram, normalized ... */
    for (int k = 0; k < T; ++k) pthread_create(&th[k], NULL, jhmi_hist_worker, &jobs[k]);
    for (int k = 0; k < T; ++k) pthread_join(th[k], NULL);
    for (int k = 0; k < T; ++k) count += jobs[k].count;
    if (count > 0)
      for (int64_t q = 0; q < B * B; ++q) {
        uint64_t h = 0;
        for (int k = 0; k < T; ++k) h += jobs[k].hist[q];
        pdf[q] = (double)h / (double)count;
      }
    /* ... smoothed by DiscreteGaussianImageFilter (variance, maximum error 0.01, no
     * image spacing; the moving axis first, then the fixed axis) ... */
    if (st->variance > 0.0) {
      double c[129];
      const int r = orc_gaussian_kernel(st->variance, 0.01, 32, c, 129);
      if (r < 0) {
        rc = ORC_ERR_BAD_ARG;
      } else {
        gauss_pass(pdf, tmp, B, 1, c, r);
        gauss_pass(tmp, pdf, B, 0, c, r);
      }
    }
    /* ... and its marginals by compensated sums: the moving marginal over the fixed
     * index, the fixed marginal over the moving index */
    for (int64_t jj = 0; jj < B; ++jj) {
      double s = 0.0, cc = 0.0;
      for (int64_t ii = 0; ii < B; ++ii) kahan_add(&s, &cc, pdf[ii + B * jj]);
      mmarg[jj] = s;
    }
    for (int64_t ii = 0; ii < B; ++ii) {
      double s = 0.0, cc = 0.0;
      for (int64_t jj = 0; jj < B; ++jj) kahan_add(&s, &cc, pdf[ii + B * jj]);
      fmarg[ii] = s;
    }
  }
  /* ComputeValue (.hxx:340-378) */
  double mi = 0.0;
  if (rc == ORC_OK) {
    const double eps = DBL_EPSILON;
    double s = 0.0, cc = 0.0;
    for (int64_t ii = 0; ii < B; ++ii) {
      const double px = fmarg[ii];
      for (int64_t jj = 0; jj < B; ++jj) {
        const double py = mmarg[jj];
        const double denom = px * py;
        const double pxy = pdf[ii + B * jj];
        double local = 0.0;
        if (fabs(denom) > eps && pxy / denom > eps) local = pxy * log(pxy / denom);
        kahan_add(&s, &cc, local);
      }
    }
    mi = -1.0 * s / log(2.0);
  }
  if (rc == ORC_OK && !compute_derivative) {
    /* GetValue (.hxx:309-330): the histogram count is the number of valid points */
    *nvalid = count;
    if (count == 0) {
      *value = DBL_MAX;
      rc = ORC_ERR_NO_VALID_POINTS;
    } else {
      *value = mi;
    }
  } else if (rc == ORC_OK) {
    for (int k = 0; k < T && rc == ORC_OK; ++k) {
      jobs[k].pdf = pdf;
      jobs[k].mmarg = mmarg;
      if (local) {
        const int64_t len = jobs[k].end - jobs[k].begin > 0 ? jobs[k].end - jobs[k].begin : 1;
        jobs[k].loff = (int64_t *)malloc(sizeof(int64_t) * (size_t)len);
        jobs[k].lval = (double *)malloc(sizeof(double) * 3 * (size_t)len);
        if (!jobs[k].loff || !jobs[k].lval) rc = ORC_ERR_OOM;
        for (int64_t q = 0; jobs[k].loff && q < len; ++q) jobs[k].loff[q] = -1;
      } else {
        jobs[k].dsum = (double *)calloc((size_t)P, sizeof(double));
        jobs[k].dcomp = (double *)calloc((size_t)P, sizeof(double));
        if (!jobs[k].dsum || !jobs[k].dcomp) rc = ORC_ERR_OOM;
      }
    }
    if (rc == ORC_OK) {
      for (int k = 0; k < T; ++k) pthread_create(&th[k], NULL, jhmi_deriv_worker, &jobs[k]);
      for (int k = 0; k < T; ++k) pthread_join(th[k], NULL);
      uint64_t nv = 0;
      for (int k = 0; k < T; ++k) nv += jobs[k].nvalid;
      *nvalid = nv;
      if (local) {
        /* Derivatives[offset + i] += LocalDerivatives[i] in point order, no averaging */
        for (int64_t p = 0; p < P; ++p) derivative[p] = 0.0;
        for (int k = 0; nv > 0 && k < T; ++k)
          for (int64_t q = 0; q < jobs[k].end - jobs[k].begin; ++q) {
            const int64_t o = jobs[k].loff[q];
            if (o < 0) continue;
            for (int d = 0; d < 3; ++d) derivative[o + d] += jobs[k].lval[3 * q + d];
          }
      } else {
        for (int64_t p = 0; p < P; ++p) {
          double s = 0.0, cc = 0.0;
          for (int k = 0; k < T; ++k) kahan_add(&s, &cc, jobs[k].dsum[p]);
          derivative[p] = nv > 0 ? s / (double)nv : 0.0;
        }
      }
      if (nv == 0) {
        *value = DBL_MAX; /* VerifyNumberOfValidPoints: a warning, value max, zero derivative */
        rc = ORC_ERR_NO_VALID_POINTS;
      } else {
        *value = mi;
      }
    }
  }
  if (joint_pdf && pdf) memcpy(joint_pdf, pdf, sizeof(double) * (size_t)(B * B));
  for (int k = 0; jobs && k < T; ++k) {
    free(jobs[k].hist); free(jobs[k].dsum); free(jobs[k].dcomp); free(jobs[k].loff); free(jobs[k].lval);
  }
  free(jobs);
  free(th);
  free(pdf);
  free(tmp);
  free(fmarg);
  free(mmarg);
  return rc;
}

int orc_jhmi_flat_v(const float *fixed, const int64_t fsize[3], const double fgeo[15], const float *moving,
                    const int64_t msize[3], const double mgeo[15], const double *moving_grad, const float *points,
                    int64_t npoints, int tkind, const double *tparams, int64_t nparams, const double *tfixed,
                    int64_t nfixed, int64_t bins, double variance, int nthreads, int compute_derivative,
                    double *value, double *derivative, uint64_t *nvalid, double *joint_pdf, const int64_t *vsize,
                    const double *vgeo)
{
  orc_inputs in;
  orc_transform t;
  orc_jhmi_state st;
  int rc = inputs_from_flat(&in, fixed, fsize, fgeo, moving, msize, mgeo, moving_grad, points, npoints, nthreads,
                            vsize, vgeo);
  if (rc) return rc;
  rc = orc_transform_from_flat(&t, tkind, tparams, nparams, tfixed, nfixed);
  if (rc) return rc;
  rc = orc_jhmi_initialize(&in, bins, variance, &st);
  if (rc) return rc;
  return orc_jhmi_value_derivative(&in, &st, &t, compute_derivative, value, derivative, nvalid, joint_pdf);
}
