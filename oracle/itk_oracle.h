/*
 * itk_oracle.h -- FP64 CPU restatement of ITK's registration-metric hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU
 * library: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * and reference legs load it.  The product path (itk_gb300/) never calls it.
 *
 * What it restates (paths relative to the ITK source tree, Modules/):
 *   - ImageToImageMetricv4 value/derivative skeleton
 *       Registration/Metricsv4/include/itkImageToImageMetricv4.hxx:218-373
 *       Registration/Metricsv4/include/itkImageToImageMetricv4GetValueAndDerivativeThreaderBase.hxx:38-327
 *   - MeanSquares per-point math
 *       Registration/Metricsv4/include/itkMeanSquaresImageToImageMetricv4GetValueAndDerivativeThreader.hxx:31-84
 *   - Mattes mutual information (bins, Parzen windows, PDFs, ComputeResults)
 *       Registration/Metricsv4/include/itkMattesMutualInformationImageToImageMetricv4.hxx:75-597
 *       Registration/Metricsv4/include/itkMattesMutualInformationImageToImageMetricv4GetValueAndDerivativeThreader.hxx:220-463
 *   - trilinear interpolation and buffer bounds
 *       Core/ImageFunction/include/itkLinearInterpolateImageFunction.h:227-470
 *       Core/ImageFunction/include/itkImageFunction.h:139-184, itkImageFunction.hxx:52-66
 *   - central-difference gradient calculator
 *       Core/ImageFunction/include/itkCentralDifferenceImageFunction.hxx:256-316
 *   - affine / B-spline (order 3) / composite transforms
 *       Core/Transform/include/itkMatrixOffsetTransformBase.hxx:126-130,566-631
 *       Core/Transform/include/itkBSplineTransform.hxx:478-652
 *       Core/Transform/include/itkCompositeTransform.hxx:60-70,466-580
 *       Core/Common/include/itkBSplineInterpolationWeightFunction.hxx:43-93
 *       Core/Common/include/itkBSplineKernelFunction.h:152-175
 *       Core/Common/include/itkBSplineDerivativeKernelFunction.h:156-180
 *   - Kahan summation  Core/Common/include/itkCompensatedSummation.hxx:38-48
 *   - displacement-field transform and the local-support derivative
 *       Filtering/DisplacementField/include/itkDisplacementFieldTransform.hxx:67-100,520-570
 *       Filtering/DisplacementField/include/itkDisplacementFieldTransform.h:336-351 (identity Jacobian)
 *       Core/ImageFunction/include/itkVectorLinearInterpolateImageFunction.hxx:35-105
 *       Numerics/Optimizersv4/include/itkObjectToObjectMetric.hxx:332-343,444-503
 *       Registration/Metricsv4/include/itkImageToImageMetricv4GetValueAndDerivativeThreaderBase.hxx:128-172,276-327
 *       Registration/Metricsv4/include/itkMattesMutualInformationImageToImageMetricv4GetValueAndDerivativeThreader.hxx:139-157,300-351,394-412
 *       Registration/Metricsv4/include/itkMattesMutualInformationImageToImageMetricv4.hxx:446-495
 *   - JointHistogram mutual information
 *       Registration/Metricsv4/include/itkJointHistogramMutualInformationImageToImageMetricv4.hxx:70-401
 *       Registration/Metricsv4/include/itkJointHistogramMutualInformationComputeJointPDFThreaderBase.hxx:57-150
 *       Registration/Metricsv4/include/itkJointHistogramMutualInformationGetValueAndDerivativeThreader.hxx:41-277
 *       Core/Common/include/itkGaussianOperator.hxx:27-180 (kernel; Abramowitz & Stegun 9.8.1-9.8.4 Bessel
 *       approximations, Numerical Recipes' downward recurrence), Filtering/Smoothing/include/itkDiscreteGaussianImageFilter.hxx:152-300
 *   - Correlation metric
 *       Registration/Metricsv4/include/itkCorrelationImageToImageMetricv4.hxx:69-116
 *       Registration/Metricsv4/include/itkCorrelationImageToImageMetricv4HelperThreader.hxx:58-169
 *       Registration/Metricsv4/include/itkCorrelationImageToImageMetricv4GetValueAndDerivativeThreader.hxx:62-325
 *
 * All arithmetic is double, as in the reference (TInternalComputationValueType
 * = double); interpolated pixel values are rounded to float where the
 * reference stores them in FixedImagePixelType / MovingImagePixelType = float.
 */
#ifndef ITK_ORACLE_H
#define ITK_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes: identical numbering to include/itk_gb300.h */
enum {
  ORC_OK = 0,
  ORC_ERR_BAD_ARG = 1,
  ORC_ERR_NO_VALID_POINTS = 2,
  ORC_ERR_JOINT_PDF_SUM_ZERO = 3,
  ORC_ERR_FIXED_CONSTANT = 4,
  ORC_ERR_MOVING_CONSTANT = 5,
  ORC_ERR_FIXED_EMPTY = 6,
  ORC_ERR_MOVING_EMPTY = 7,
  ORC_ERR_OOM = 8
};

enum { ORC_TRANSFORM_AFFINE = 0, ORC_TRANSFORM_BSPLINE = 1, ORC_TRANSFORM_COMPOSITE = 2, ORC_TRANSFORM_DISPLACEMENT = 3 };

/* Image geometry: x-fastest buffer, start index 0. */
typedef struct {
  int64_t size[3];
  double spacing[3];
  double origin[3];
  double direction[9]; /* row-major */
  double i2p[9];       /* direction * diag(spacing) */
  double p2i[9];       /* inverse of i2p */
} orc_geom;

/* Moving transform.  kind AFFINE: y = M x + offset (12 params).
 * kind BSPLINE: order-3 B-spline over a coefficient grid (3*nper params).
 * kind COMPOSITE: y = affine(bspline(x)); only the B-spline is optimized,
 * which is the [MovingInitialTransform, OutputTransform] queue of
 * ImageRegistrationMethodv4.
 * kind DISPLACEMENT: y = x + field(x) (vector linear interpolation, zero
 * outside the field's buffer); 3 parameters per field voxel, local support:
 * the derivative is a field over the virtual domain (same geometry). */
typedef struct {
  int kind;
  /* affine part (active for AFFINE, fixed initial for COMPOSITE) */
  double M[9];
  double center[3];
  double translation[3];
  double offset[3];
  /* B-spline part */
  int64_t grid[3];
  int64_t nper;
  double gorigin[3];
  double gspacing[3];
  double gdir[9];
  double gp2i[9];
  const double *coeff; /* 3*nper, dimension-major, x-fastest inside */
  /* displacement field */
  orc_geom fgeom;
  int64_t nvox;
  const double *field; /* 3*nvox, voxel-major (x, y, z per voxel), x-fastest voxels */
  int field_affine;    /* 1: [affine, displacement field] composite, y = affine(x + field(x)) */
} orc_transform;

typedef struct {
  const float *fixed;          orc_geom fixed_geom;
  const float *moving;         orc_geom moving_geom;
  const double *moving_grad;   /* 3 doubles / voxel, or NULL: central difference */
  orc_geom virtual_geom;       /* dense domain */
  const float *points;         /* virtual-space sample points (xyz float), or NULL = dense */
  int64_t npoints;
  int nthreads;
  int pixel_double;            /* 1: keep interpolated values in double, as for Image<double,N> */
  double fp_resolution;        /* > 0: UseFloatingPointCorrection at this resolution (MeanSquares) */
} orc_inputs;

typedef struct {
  int64_t bins;
  double fixed_true_min, fixed_true_max;
  double moving_true_min, moving_true_max;
  double fixed_bin_size, moving_bin_size;
  double fixed_normalized_min, moving_normalized_min;
} orc_mattes_state;

int orc_geom_init(orc_geom *g, const int64_t size[3], const double spacing[3],
                  const double origin[3], const double direction[9]);

/* transforms */
int orc_affine_init(orc_transform *t, const double params12[12], const double center[3]);
int orc_bspline_init(orc_transform *t, const double fixed18[18], const double *coeff);
int orc_composite_init(orc_transform *t, const double affine_params12[12], const double affine_center[3],
                       const double fixed18[18], const double *coeff);
/* fixed18: field size, origin, spacing, direction (row-major) */
int orc_displacement_init(orc_transform *t, const double fixed18[18], const double *field);
int64_t orc_transform_nparams(const orc_transform *t);
/* y = T(x); returns 1 always (identity outside the B-spline valid region) */
void orc_transform_point(const orc_transform *t, const double x[3], double y[3]);

/* single-function probes used by the golden tests */
int orc_interpolate(const orc_geom *g, const float *img, const double point[3], double *value, int *inside);
int orc_bspline_weights(const double cindex[3], double weights[64], int64_t start[3]);
double orc_bspline3(double u);
double orc_bspline3_derivative(double u);
int orc_central_difference(const orc_geom *g, const float *img, const double point[3], double grad[3]);

/* metrics */
int orc_msq_value_derivative(const orc_inputs *in, const orc_transform *t, int compute_derivative,
                             double *value, double *derivative, uint64_t *nvalid);
int orc_mattes_initialize(const orc_inputs *in, int64_t bins, orc_mattes_state *st);
int orc_mattes_value_derivative(const orc_inputs *in, const orc_mattes_state *st, const orc_transform *t,
                                int compute_derivative, double *value, double *derivative, uint64_t *nvalid,
                                double *joint_pdf /* bins*bins or NULL */);

/* flat-argument wrappers for ctypes callers (arrays, no structs) */
/* Transform flat encoding:
 *   AFFINE:    tparams = 12 (row-major matrix, translation), tfixed = centre (3)
 *   BSPLINE:   tparams = 3*nper coefficients, tfixed = 18 fixed parameters
 *              (grid size, grid origin, grid spacing, grid direction)
 *   COMPOSITE: tparams = 3*nper B-spline coefficients (the optimized part),
 *              tfixed = 18 B-spline fixed parameters, 12 initial-affine
 *              parameters, 3 initial-affine centre (33 values)
 *   DISPLACEMENT: tparams = 3*voxels field values, tfixed = 18 (field size,
 *              origin, spacing, direction); the field must share the virtual
 *              domain's grid (VerifyDisplacementFieldSizeAndPhysicalSpace);
 *              tfixed = 33 adds an initial affine (12 parameters, centre 3):
 *              the [affine, displacement field] composite, field applied first
 * Geometry flat encoding (15 doubles): spacing(3), origin(3), direction(9).
 * nthreads: low 16 bits = thread count; bit 16 set = double pixel type
 * (interpolated values are not rounded to float, as for Image<double,N>). */
int orc_transform_from_flat(orc_transform *t, int tkind, const double *tparams, int64_t nparams,
                            const double *tfixed, int64_t nfixed);
int orc_msq_flat(const float *fixed, const int64_t fsize[3], const double fgeo[15],
                 const float *moving, const int64_t msize[3], const double mgeo[15], const double *moving_grad,
                 const float *points, int64_t npoints, int tkind, const double *tparams, int64_t nparams,
                 const double *tfixed, int64_t nfixed, int nthreads, int compute_derivative,
                 double *value, double *derivative, uint64_t *nvalid);
/* state_out (8 doubles): fixed min, fixed max, moving min, moving max,
 * fixed bin size, moving bin size, fixed normalized min, moving normalized min */
int orc_mattes_flat(const float *fixed, const int64_t fsize[3], const double fgeo[15],
                    const float *moving, const int64_t msize[3], const double mgeo[15], const double *moving_grad,
                    const float *points, int64_t npoints, int tkind, const double *tparams, int64_t nparams,
                    const double *tfixed, int64_t nfixed, int64_t bins, int nthreads, int compute_derivative,
                    double *value, double *derivative, uint64_t *nvalid, double *joint_pdf, double *state_out);
/* the same with a virtual domain geometry (vsize, vgeo = spacing, origin, direction);
 * NULL = the fixed image's geometry */
int orc_msq_flat_v(const float *fixed, const int64_t fsize[3], const double fgeo[15],
                   const float *moving, const int64_t msize[3], const double mgeo[15], const double *moving_grad,
                   const float *points, int64_t npoints, int tkind, const double *tparams, int64_t nparams,
                   const double *tfixed, int64_t nfixed, int nthreads, int compute_derivative,
                   double *value, double *derivative, uint64_t *nvalid, const int64_t *vsize, const double *vgeo);
int orc_mattes_flat_v(const float *fixed, const int64_t fsize[3], const double fgeo[15],
                      const float *moving, const int64_t msize[3], const double mgeo[15], const double *moving_grad,
                      const float *points, int64_t npoints, int tkind, const double *tparams, int64_t nparams,
                      const double *tfixed, int64_t nfixed, int64_t bins, int nthreads, int compute_derivative,
                      double *value, double *derivative, uint64_t *nvalid, double *joint_pdf, double *state_out,
                      const int64_t *vsize, const double *vgeo);
/* orc_msq_flat_v with UseFloatingPointCorrection at `resolution` (> 0) */
int orc_msq_flat_fpc(const float *fixed, const int64_t fsize[3], const double fgeo[15],
                     const float *moving, const int64_t msize[3], const double mgeo[15], const double *moving_grad,
                     const float *points, int64_t npoints, int tkind, const double *tparams, int64_t nparams,
                     const double *tfixed, int64_t nfixed, int nthreads, int compute_derivative,
                     double *value, double *derivative, uint64_t *nvalid, double resolution);
int orc_transform_point_flat(int tkind, const double *tparams, int64_t nparams, const double *tfixed,
                             int64_t nfixed, const double *x, int64_t n, double *y);
int orc_interpolate_flat(const float *img, const int64_t size[3], const double geo[15], const double *points,
                         int64_t n, double *values, int *inside);
int orc_central_difference_flat(const float *img, const int64_t size[3], const double geo[15],
                                const double *points, int64_t n, double *grads);

/* ---- per-level image filters (itk_oracle_filters.c) ---- */

/* RecursiveGaussianImageFilter coefficients (Farneback / Deriche IIR), order 0, 1 or 2 */
typedef struct {
  double N0, N1, N2, N3;
  double D1, D2, D3, D4;
  double M1, M2, M3, M4;
  double BN1, BN2, BN3, BN4;
  double BM1, BM2, BM3, BM4;
} orc_rg_coef;

int orc_rg_setup(double sigma, double spacing, int order, int normalize_across_scale, orc_rg_coef *c);
/* RecursiveSeparableImageFilter::FilterDataArray on one line of length ln >= 4 */
void orc_rg_filter_line(const orc_rg_coef *c, const double *data, double *outs, double *scratch, int64_t ln);
/* SmoothingRecursiveGaussianImageFilter on Image<float,3> (sigma in physical units per axis) */
int orc_smooth_recursive_gaussian(const float *in, float *out, const int64_t size[3], const double spacing[3],
                                  const double sigma[3]);
/* GradientRecursiveGaussianImageFilter on Image<float,3>: 3 doubles per voxel */
int orc_gradient_recursive_gaussian(const float *in, double *out, const int64_t size[3], const double spacing[3],
                                    const double direction[9], double sigma, int normalize_across_scale,
                                    int use_image_direction);
/* ShrinkImageFilter output geometry (start index 0) */
int orc_shrink_geometry(const int64_t size[3], const double spacing[3], const double origin[3],
                        const double direction[9], const int64_t factors[3], int64_t out_size[3],
                        double out_spacing[3], double out_origin[3]);

/* CorrelationImageToImageMetricv4 (normalized cross correlation): averages over
 * the valid points, then value -fm^2/(f2 m2) and its derivative; flat inputs as
 * orc_msq_flat_v */
int orc_corr_value_derivative(const orc_inputs *in, const orc_transform *t, int compute_derivative, double *value,
                              double *derivative, uint64_t *nvalid);
int orc_corr_flat_v(const float *fixed, const int64_t fsize[3], const double fgeo[15], const float *moving,
                    const int64_t msize[3], const double mgeo[15], const double *moving_grad, const float *points,
                    int64_t npoints, int tkind, const double *tparams, int64_t nparams, const double *tfixed,
                    int64_t nfixed, int nthreads, int compute_derivative, double *value, double *derivative,
                    uint64_t *nvalid, const int64_t *vsize, const double *vgeo);

/* JointHistogramMutualInformationImageToImageMetricv4: joint histogram of
 * (fixed, moving) bins, normalized, smoothed by a discrete Gaussian, MI in bits;
 * derivative from the smoothed PDF's moving-axis slope (flat inputs as
 * orc_msq_flat_v; joint_pdf = the smoothed bins x bins PDF, fixed index fastest,
 * or NULL).  A displacement field stores sf J^T g at each point's voxel, not averaged. */
typedef struct {
  int64_t bins;
  double variance;
  double fmin, fmax, mmin, mmax;
  double spacing, origin, inv_spacing;
} orc_jhmi_state;
int orc_gaussian_kernel(double variance, double max_error, int max_width, double *c, int cap);
int orc_jhmi_initialize(const orc_inputs *in, int64_t bins, double variance, orc_jhmi_state *st);
int orc_jhmi_value_derivative(const orc_inputs *in, const orc_jhmi_state *st, const orc_transform *t,
                              int compute_derivative, double *value, double *derivative, uint64_t *nvalid,
                              double *joint_pdf);
int orc_jhmi_flat_v(const float *fixed, const int64_t fsize[3], const double fgeo[15], const float *moving,
                    const int64_t msize[3], const double mgeo[15], const double *moving_grad, const float *points,
                    int64_t npoints, int tkind, const double *tparams, int64_t nparams, const double *tfixed,
                    int64_t nfixed, int64_t bins, double variance, int nthreads, int compute_derivative,
                    double *value, double *derivative, uint64_t *nvalid, double *joint_pdf, const int64_t *vsize,
                    const double *vgeo);

/* ---- metric sample points (itk_oracle_sampling.c) ---------------------- */
/* MT19937 32-bit outputs after `skip` draws from a fresh seed */
int orc_mt_sequence(uint32_t seed, int64_t skip, uint32_t *out, int64_t n);
/* GetNormalVariate(0, 1) sequence from a fresh seed */
int orc_mt_normals(uint32_t seed, double *out, int64_t n);
/* SetMetricSamplePoints: strategy 1 REGULAR, 2 RANDOM; geometry = spacing[3],
 * origin[3], direction[9]; float points (x, y, z) */
int orc_sample_points(int strategy, const int64_t size[3], const double *geometry, double percentage, int32_t seed,
                      float *xyz, int64_t capacity, int64_t *count);

#ifdef __cplusplus
}
#endif
#endif
