/*
 * itk_oracle_filters.c -- FP64 CPU restatement of the image filters that
 * ImageRegistrationMethodv4 and ImageToImageMetricv4 run per resolution level.
 *
 * TEST INFRASTRUCTURE ONLY, like itk_oracle.c: the checker for the GPU
 * library's device filters.  Paths are relative to ITK's Modules/.
 *
 *   RecursiveGaussianImageFilter::SetUp and coefficient helpers
 *       Filtering/Smoothing/include/itkRecursiveGaussianImageFilter.hxx:56-300
 *   RecursiveSeparableImageFilter::FilterDataArray / line traversal
 *       Filtering/ImageFilterBase/include/itkRecursiveSeparableImageFilter.hxx:60-150,285-330
 *   SmoothingRecursiveGaussianImageFilter (passes z, x, y; float between passes for float images)
 *       Filtering/Smoothing/include/itkSmoothingRecursiveGaussianImageFilter.hxx:25-60,230-283
 *   GradientRecursiveGaussianImageFilter (first order along d, zero order along the others,
 *   double between passes, / spacing, then direction)
 *       Filtering/ImageGradient/include/itkGradientRecursiveGaussianImageFilter.hxx:160-270
 *       Filtering/ImageGradient/include/itkGradientRecursiveGaussianImageFilter.h:211-246
 *   ShrinkImageFilter output geometry and pixel mapping
 *       Filtering/ImageGrid/include/itkShrinkImageFilter.hxx:100-290
 *   ImageBase index <-> point conversions   Core/Common/include/itkImageBase.h:560-604
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "itk_oracle.h"

/* MathEMAMAMAM / MathSMAMAMAM, itkRecursiveSeparableImageFilter.h:175-225 */
static inline void emam(double *out, double a1, double b1, double a2, double b2, double a3, double b3, double a4,
                        double b4)
{
  *out = a1 * b1 + a2 * b2 + a3 * b3 + a4 * b4;
}
static inline void smam(double *out, double a1, double b1, double a2, double b2, double a3, double b3, double a4,
                        double b4)
{
  *out -= a1 * b1 + a2 * b2 + a3 * b3 + a4 * b4;
}

static void rg_d_coefficients(orc_rg_coef *c, double sigmad, double W1, double L1, double W2, double L2, double *SD,
                              double *DD, double *ED)
{
  const double Cos1 = cos(W1 / sigmad);
  const double Cos2 = cos(W2 / sigmad);
  const double Exp1 = exp(L1 / sigmad);
  const double Exp2 = exp(L2 / sigmad);
  c->D4 = Exp1 * Exp1 * Exp2 * Exp2;
  c->D3 = -2 * Cos1 * Exp1 * Exp2 * Exp2;
  c->D3 += -2 * Cos2 * Exp2 * Exp1 * Exp1;
  c->D2 = 4 * Cos2 * Cos1 * Exp1 * Exp2;
  c->D2 += Exp1 * Exp1 + Exp2 * Exp2;
  c->D1 = -2 * (Exp2 * Cos2 + Exp1 * Cos1);
  *SD = 1.0 + c->D1 + c->D2 + c->D3 + c->D4;
  *DD = c->D1 + 2 * c->D2 + 3 * c->D3 + 4 * c->D4;
  *ED = c->D1 + 4 * c->D2 + 9 * c->D3 + 16 * c->D4;
}

static void rg_n_coefficients(double sigmad, double A1, double B1, double W1, double L1, double A2, double B2,
                              double W2, double L2, double *N0, double *N1, double *N2, double *N3, double *SN,
                              double *DN, double *EN)
{
  const double Sin1 = sin(W1 / sigmad);
  const double Sin2 = sin(W2 / sigmad);
  const double Cos1 = cos(W1 / sigmad);
  const double Cos2 = cos(W2 / sigmad);
  const double Exp1 = exp(L1 / sigmad);
  const double Exp2 = exp(L2 / sigmad);
  *N0 = A1 + A2;
  *N1 = Exp2 * (B2 * Sin2 - (A2 + 2 * A1) * Cos2);
  *N1 += Exp1 * (B1 * Sin1 - (A1 + 2 * A2) * Cos1);
  *N2 = (A1 + A2) * Cos2 * Cos1;
  *N2 -= B1 * Cos2 * Sin1 + B2 * Cos1 * Sin2;
  *N2 *= 2 * Exp1 * Exp2;
  *N2 += A2 * Exp1 * Exp1 + A1 * Exp2 * Exp2;
  *N3 = Exp2 * Exp1 * Exp1 * (B2 * Sin2 - A2 * Cos2);
  *N3 += Exp1 * Exp2 * Exp2 * (B1 * Sin1 - A1 * Cos1);
  *SN = *N0 + *N1 + *N2 + *N3;
  *DN = *N1 + 2 * *N2 + 3 * *N3;
  *EN = *N1 + 4 * *N2 + 9 * *N3;
}

static void rg_remaining(orc_rg_coef *c, int symmetric)
{
  if (symmetric) {
    c->M1 = c->N1 - c->D1 * c->N0;
    c->M2 = c->N2 - c->D2 * c->N0;
    c->M3 = c->N3 - c->D3 * c->N0;
    c->M4 = -c->D4 * c->N0;
  } else {
    c->M1 = -(c->N1 - c->D1 * c->N0);
    c->M2 = -(c->N2 - c->D2 * c->N0);
    c->M3 = -(c->N3 - c->D3 * c->N0);
    c->M4 = c->D4 * c->N0;
  }
  const double SN = c->N0 + c->N1 + c->N2 + c->N3;
  const double SM = c->M1 + c->M2 + c->M3 + c->M4;
  const double SD = 1.0 + c->D1 + c->D2 + c->D3 + c->D4;
  c->BN1 = c->D1 * SN / SD;
  c->BN2 = c->D2 * SN / SD;
  c->BN3 = c->D3 * SN / SD;
  c->BN4 = c->D4 * SN / SD;
  c->BM1 = c->D1 * SM / SD;
  c->BM2 = c->D2 * SM / SD;
  c->BM3 = c->D3 * SM / SD;
  c->BM4 = c->D4 * SM / SD;
}

/* RecursiveGaussianImageFilter::SetUp (Farneback's parameters for the Deriche
 * recursive Gaussian), itkRecursiveGaussianImageFilter.hxx:56-200 */
int orc_rg_setup(double sigma, double spacing, int order, int normalize_across_scale, orc_rg_coef *c)
{
  double direction = 1.0;
  if (spacing < 0.0) {
    direction = -1.0;
    spacing *= -1;
  }
  if (spacing < 1e-8 || !(sigma > 0.0)) return ORC_ERR_BAD_ARG;
  memset(c, 0, sizeof(*c));
  const double sigmad = sigma / spacing;
  double across = 1.0;
  const double A1[3] = {1.3530, -0.6724, -1.3563};
  const double B1[3] = {1.8151, -3.4327, 5.2318};
  const double W1 = 0.6681;
  const double L1 = -1.3932;
  const double A2[3] = {-0.3531, 0.6724, 0.3446};
  const double B2[3] = {0.0902, 0.6100, -2.2355};
  const double W2 = 2.0787;
  const double L2 = -1.3732;
  double SD, DD, ED, SN, DN, EN;
  rg_d_coefficients(c, sigmad, W1, L1, W2, L2, &SD, &DD, &ED);
  if (order == 0) {
    rg_n_coefficients(sigmad, A1[0], B1[0], W1, L1, A2[0], B2[0], W2, L2, &c->N0, &c->N1, &c->N2, &c->N3, &SN, &DN,
                      &EN);
    const double alpha0 = 2 * SN / SD - c->N0;
    c->N0 *= across / alpha0;
    c->N1 *= across / alpha0;
    c->N2 *= across / alpha0;
    c->N3 *= across / alpha0;
    rg_remaining(c, 1);
  } else if (order == 1) {
    if (normalize_across_scale) across = sigma;
    rg_n_coefficients(sigmad, A1[1], B1[1], W1, L1, A2[1], B2[1], W2, L2, &c->N0, &c->N1, &c->N2, &c->N3, &SN, &DN,
                      &EN);
    double alpha1 = 2 * (SN * DD - DN * SD) / (SD * SD);
    alpha1 *= direction;
    c->N0 *= across / alpha1;
    c->N1 *= across / alpha1;
    c->N2 *= across / alpha1;
    c->N3 *= across / alpha1;
    rg_remaining(c, 0);
  } else if (order == 2) {
    if (normalize_across_scale) across = sigma * sigma;
    double N0_0, N1_0, N2_0, N3_0, N0_2, N1_2, N2_2, N3_2, SN0, DN0, EN0, SN2, DN2, EN2;
    rg_n_coefficients(sigmad, A1[0], B1[0], W1, L1, A2[0], B2[0], W2, L2, &N0_0, &N1_0, &N2_0, &N3_0, &SN0, &DN0,
                      &EN0);
    rg_n_coefficients(sigmad, A1[2], B1[2], W1, L1, A2[2], B2[2], W2, L2, &N0_2, &N1_2, &N2_2, &N3_2, &SN2, &DN2,
                      &EN2);
    const double beta = -(2 * SN2 - SD * N0_2) / (2 * SN0 - SD * N0_0);
    c->N0 = N0_2 + beta * N0_0;
    c->N1 = N1_2 + beta * N1_0;
    c->N2 = N2_2 + beta * N2_0;
    c->N3 = N3_2 + beta * N3_0;
    SN = SN2 + beta * SN0;
    DN = DN2 + beta * DN0;
    EN = EN2 + beta * EN0;
    double alpha2 = EN * SD * SD - ED * SN * SD - 2 * DN * DD * SD + 2 * DD * DD * SN;
    alpha2 /= SD * SD * SD;
    c->N0 *= across / alpha2;
    c->N1 *= across / alpha2;
    c->N2 *= across / alpha2;
    c->N3 *= across / alpha2;
    rg_remaining(c, 1);
  } else {
    return ORC_ERR_BAD_ARG;
  }
  return ORC_OK;
}

/* RecursiveSeparableImageFilter::FilterDataArray, itkRecursiveSeparableImageFilter.hxx:60-150 */
void orc_rg_filter_line(const orc_rg_coef *c, const double *data, double *outs, double *scratch, int64_t ln)
{
  const double outV1 = data[0];
  emam(&outs[0], outV1, c->N0, outV1, c->N1, outV1, c->N2, outV1, c->N3);
  emam(&outs[1], data[1], c->N0, outV1, c->N1, outV1, c->N2, outV1, c->N3);
  emam(&outs[2], data[2], c->N0, data[1], c->N1, outV1, c->N2, outV1, c->N3);
  emam(&outs[3], data[3], c->N0, data[2], c->N1, data[1], c->N2, outV1, c->N3);
  smam(&outs[0], outV1, c->BN1, outV1, c->BN2, outV1, c->BN3, outV1, c->BN4);
  smam(&outs[1], outs[0], c->D1, outV1, c->BN2, outV1, c->BN3, outV1, c->BN4);
  smam(&outs[2], outs[1], c->D1, outs[0], c->D2, outV1, c->BN3, outV1, c->BN4);
  smam(&outs[3], outs[2], c->D1, outs[1], c->D2, outs[0], c->D3, outV1, c->BN4);
  for (int64_t i = 4; i < ln; ++i) {
    emam(&outs[i], data[i], c->N0, data[i - 1], c->N1, data[i - 2], c->N2, data[i - 3], c->N3);
    smam(&outs[i], outs[i - 1], c->D1, outs[i - 2], c->D2, outs[i - 3], c->D3, outs[i - 4], c->D4);
  }
  const double outV2 = data[ln - 1];
  emam(&scratch[ln - 1], outV2, c->M1, outV2, c->M2, outV2, c->M3, outV2, c->M4);
  emam(&scratch[ln - 2], data[ln - 1], c->M1, outV2, c->M2, outV2, c->M3, outV2, c->M4);
  emam(&scratch[ln - 3], data[ln - 2], c->M1, data[ln - 1], c->M2, outV2, c->M3, outV2, c->M4);
  emam(&scratch[ln - 4], data[ln - 3], c->M1, data[ln - 2], c->M2, data[ln - 1], c->M3, outV2, c->M4);
  smam(&scratch[ln - 1], outV2, c->BM1, outV2, c->BM2, outV2, c->BM3, outV2, c->BM4);
  smam(&scratch[ln - 2], scratch[ln - 1], c->D1, outV2, c->BM2, outV2, c->BM3, outV2, c->BM4);
  smam(&scratch[ln - 3], scratch[ln - 2], c->D1, scratch[ln - 1], c->D2, outV2, c->BM3, outV2, c->BM4);
  smam(&scratch[ln - 4], scratch[ln - 3], c->D1, scratch[ln - 2], c->D2, scratch[ln - 1], c->D3, outV2, c->BM4);
  for (int64_t i = ln - 4; i > 0; i--) {
    emam(&scratch[i - 1], data[i], c->M1, data[i + 1], c->M2, data[i + 2], c->M3, data[i + 3], c->M4);
    smam(&scratch[i - 1], scratch[i], c->D1, scratch[i + 1], c->D2, scratch[i + 2], c->D3, scratch[i + 3], c->D4);
  }
  for (int64_t i = 0; i < ln; ++i) outs[i] += scratch[i];
}

/* One RecursiveGaussianImageFilter pass along `axis` over a 3-D buffer; input and
 * output are float (is_double 0) or double (1) images; the line is filtered in
 * double (RealType) and stored with a cast to the output pixel type. */
static int rg_pass(const void *in, int in_double, void *out, int out_double, const int64_t size[3], int axis,
                   const orc_rg_coef *c)
{
  const int64_t ln = size[axis];
  if (ln < 4) return ORC_ERR_BAD_ARG;
  const int64_t stride = axis == 0 ? 1 : (axis == 1 ? size[0] : size[0] * size[1]);
  const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
  const int64_t s1 = a1 == 0 ? 1 : size[0], s2 = a2 == 1 ? size[0] : size[0] * size[1];
  double *data = (double *)malloc(sizeof(double) * 3 * (size_t)ln);
  if (!data) return ORC_ERR_OOM;
  double *outs = data + ln, *scratch = data + 2 * ln;
  for (int64_t j2 = 0; j2 < size[a2]; ++j2)
    for (int64_t j1 = 0; j1 < size[a1]; ++j1) {
      const int64_t base = j1 * s1 + j2 * s2;
      for (int64_t i = 0; i < ln; ++i)
        data[i] = in_double ? ((const double *)in)[base + i * stride] : (double)((const float *)in)[base + i * stride];
      orc_rg_filter_line(c, data, outs, scratch, ln);
      for (int64_t i = 0; i < ln; ++i) {
        if (out_double) ((double *)out)[base + i * stride] = outs[i];
        else ((float *)out)[base + i * stride] = (float)outs[i];
      }
    }
  free(data);
  return ORC_OK;
}

/* SmoothingRecursiveGaussianImageFilter<Image<float,3>, Image<float,3>>: zero-order
 * passes along z, x, y (the first filter takes the last direction), float images
 * in between (InternalRealType = FloatType of float). */
int orc_smooth_recursive_gaussian(const float *in, float *out, const int64_t size[3], const double spacing[3],
                                  const double sigma[3])
{
  for (int d = 0; d < 3; ++d)
    if (size[d] < 4) return ORC_ERR_BAD_ARG;
  const int64_t n = size[0] * size[1] * size[2];
  float *tmp = (float *)malloc(sizeof(float) * (size_t)n);
  if (!tmp) return ORC_ERR_OOM;
  orc_rg_coef c;
  int rc = orc_rg_setup(sigma[2], spacing[2], 0, 0, &c);
  if (!rc) rc = rg_pass(in, 0, tmp, 0, size, 2, &c);
  if (!rc) rc = orc_rg_setup(sigma[0], spacing[0], 0, 0, &c);
  if (!rc) rc = rg_pass(tmp, 0, out, 0, size, 0, &c);
  if (!rc) rc = orc_rg_setup(sigma[1], spacing[1], 0, 0, &c);
  if (!rc) rc = rg_pass(out, 0, tmp, 0, size, 1, &c);
  if (!rc) memcpy(out, tmp, sizeof(float) * (size_t)n);
  free(tmp);
  return rc;
}

/* GradientRecursiveGaussianImageFilter<Image<float,3>> (double intermediates):
 * component d = first order along d, then zero order along the other axes in
 * increasing order, divided by spacing[d]; with use_image_direction the vector
 * is mapped by the direction matrix (TransformLocalVectorToPhysicalVector).
 * out: 3 doubles per voxel. */
int orc_gradient_recursive_gaussian(const float *in, double *out, const int64_t size[3], const double spacing[3],
                                    const double direction[9], double sigma, int normalize_across_scale,
                                    int use_image_direction)
{
  for (int d = 0; d < 3; ++d)
    if (size[d] < 4) return ORC_ERR_BAD_ARG;
  const int64_t n = size[0] * size[1] * size[2];
  double *a = (double *)malloc(sizeof(double) * (size_t)n);
  double *b = (double *)malloc(sizeof(double) * (size_t)n);
  if (!a || !b) {
    free(a);
    free(b);
    return ORC_ERR_OOM;
  }
  int rc = ORC_OK;
  for (int dim = 0; dim < 3 && !rc; ++dim) {
    orc_rg_coef c;
    rc = orc_rg_setup(sigma, spacing[dim], 1, normalize_across_scale, &c);
    if (!rc) rc = rg_pass(in, 0, a, 1, size, dim, &c);
    double *src = a, *dst = b;
    for (int j = 0; j < 3 && !rc; ++j) {
      if (j == dim) continue;
      rc = orc_rg_setup(sigma, spacing[j], 0, normalize_across_scale, &c);
      if (!rc) rc = rg_pass(src, 1, dst, 1, size, j, &c);
      double *t = src;
      src = dst;
      dst = t;
    }
    if (!rc)
      for (int64_t v = 0; v < n; ++v) out[3 * v + dim] = src[v] / spacing[dim];
  }
  free(a);
  free(b);
  if (rc || !use_image_direction) return rc;
  for (int64_t v = 0; v < n; ++v) {
    double g[3] = {out[3 * v], out[3 * v + 1], out[3 * v + 2]};
    for (int r = 0; r < 3; ++r) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += direction[r * 3 + k] * g[k];
      out[3 * v + r] = s;
    }
  }
  return ORC_OK;
}

/* ShrinkImageFilter::GenerateOutputInformation (start index 0), itkShrinkImageFilter.hxx:230-290 */
int orc_shrink_geometry(const int64_t size[3], const double spacing[3], const double origin[3],
                        const double direction[9], const int64_t factors[3], int64_t out_size[3],
                        double out_spacing[3], double out_origin[3])
{
  int64_t f[3];
  for (int i = 0; i < 3; ++i) {
    f[i] = factors[i] < 1 ? 1 : factors[i];
    out_spacing[i] = spacing[i] * (double)f[i];
    out_size[i] = (int64_t)floor((double)size[i] / (double)f[i]);
    if (out_size[i] < 1) out_size[i] = 1;
  }
  double in_c[3], out_c[3], in_p[3], out_p[3];
  for (int i = 0; i < 3; ++i) {
    in_c[i] = 0 + (double)(size[i] - 1) / 2.0;
    out_c[i] = 0 + (double)(out_size[i] - 1) / 2.0;
  }
  /* TransformContinuousIndexToPhysicalPoint: the sum first, then the origin (the
   * output image still carries the input origin at this point) */
  for (int r = 0; r < 3; ++r) {
    double s_in = 0.0, s_out = 0.0;
    for (int c = 0; c < 3; ++c) {
      s_in += direction[r * 3 + c] * spacing[c] * in_c[c];
      s_out += direction[r * 3 + c] * out_spacing[c] * out_c[c];
    }
    in_p[r] = s_in + origin[r];
    out_p[r] = s_out + origin[r];
  }
  for (int r = 0; r < 3; ++r) out_origin[r] = origin[r] + (in_p[r] - out_p[r]);
  return ORC_OK;
}
