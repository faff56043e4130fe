/*
 * itk_gb300.h -- C ABI of the GB300 registration-metric library.
 *
 * One GPU, one process.  Plain pointers and sizes only: no C++ or torch types
 * cross this boundary.  Every function returns an int status (GB_OK = 0).
 * Caller buffers are borrowed for the duration of a call; device memory
 * belongs to the handle that allocated it.  Handles are independent and may
 * be used from different host threads; one call at a time per handle.
 *
 * Each entry point names the reference interface it replaces (paths relative
 * to the ITK source tree, Modules/).  On the ITK side these entry points sit
 * behind itk::ObjectFactoryBase overrides of the metric classes.
 */
#ifndef ITK_GB300_H
#define ITK_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  GB_OK = 0,
  GB_ERR_BAD_ARG = 1,
  /* no sample mapped inside both buffers.  MeanSquares still returns
   * value = DBL_MAX and a zero derivative (ObjectToObjectMetric::
   * VerifyNumberOfValidPoints, Numerics/Optimizersv4/include/itkObjectToObjectMetric.hxx:512-527);
   * Mattes raises (itkMattesMutualInformationImageToImageMetricv4.hxx:360-366). */
  GB_ERR_NO_VALID_POINTS = 2,
  GB_ERR_JOINT_PDF_SUM_ZERO = 3, /* itkMattesMutualInformationImageToImageMetricv4.hxx:367-370 */
  GB_ERR_FIXED_CONSTANT = 4,     /* itkMattesMutualInformationImageToImageMetricv4.hxx:284-292 */
  GB_ERR_MOVING_CONSTANT = 5,    /* itkMattesMutualInformationImageToImageMetricv4.hxx:299-307 */
  GB_ERR_FIXED_EMPTY = 6,        /* itkMattesMutualInformationImageToImageMetricv4.hxx:278-283 */
  GB_ERR_MOVING_EMPTY = 7,       /* itkMattesMutualInformationImageToImageMetricv4.hxx:293-298 */
  GB_ERR_OUT_OF_MEMORY = 8,
  GB_ERR_CUDA = 9,
  GB_ERR_TIMEOUT = 10,
  GB_ERR_NOT_INITIALIZED = 11,
  GB_ERR_UNSUPPORTED = 12,
  GB_ERR_ADMISSION = 13
};

/* metric kinds; CORRELATION is CorrelationImageToImageMetricv4 (affine transforms)
 * (Registration/Metricsv4/include/itkCorrelationImageToImageMetricv4.hxx) */
enum { GB_METRIC_MEAN_SQUARES = 0, GB_METRIC_MATTES = 1, GB_METRIC_CORRELATION = 2, GB_METRIC_JOINT_HISTOGRAM_MI = 3 };
/* image slots */
enum { GB_IMAGE_FIXED = 0, GB_IMAGE_MOVING = 1 };
/* moving transform kinds (flat encodings below) */
enum { GB_TRANSFORM_AFFINE = 0, GB_TRANSFORM_BSPLINE = 1, GB_TRANSFORM_COMPOSITE = 2, GB_TRANSFORM_DISPLACEMENT_FIELD = 3 };
/* moving-gradient source */
enum {
  GB_GRADIENT_IMAGE = 0,              /* caller-supplied gradient image (filter output) */
  GB_GRADIENT_CENTRAL_DIFFERENCE = 1, /* per-point CentralDifferenceImageFunction */
  GB_GRADIENT_RECURSIVE_GAUSSIAN = 2  /* gradient image computed on the device */
};

typedef struct gb_ctx gb_ctx;
typedef struct gb_metric gb_metric;

/* Text of the last error raised on the calling host thread (never NULL).
 * Mattes/MeanSquares errors reuse the reference's exception text. */
const char *gb_last_error(void);
/* Text of the last error raised by a call on metric handle m (never NULL; ""
 * before any error), so that errors are not mis-attributed when one thread
 * drives several handles.  This is the per-handle error text of the drop-in's
 * exceptions (itkExceptionMacro in the metric, Core/Common/include/itkMacro.h:608). */
const char *gb_metric_last_error(gb_metric *m);
/* Library version string. */
const char *gb_version(void);

/* ---- device context ---------------------------------------------------- */
/* Binds a CUDA device; the context owns no stream of its own. */
int gb_ctx_create(int device, gb_ctx **out);
int gb_ctx_destroy(gb_ctx *ctx);
/* Number of SMs and total/free device memory in bytes. */
int gb_ctx_info(gb_ctx *ctx, int *sm_count, uint64_t *total_bytes, uint64_t *free_bytes);

/* ---- metric handle ----------------------------------------------------- */
/* Replaces MeanSquaresImageToImageMetricv4<Image<float,3>,...>::New() and
 * MattesMutualInformationImageToImageMetricv4<Image<float,3>,...>::New()
 * (Registration/Metricsv4/include/itkMattesMutualInformationImageToImageMetricv4.hxx:31-60).
 * Each handle owns a CUDA stream and its device buffers. */
int gb_metric_create(gb_ctx *ctx, int kind, gb_metric **out);
int gb_metric_destroy(gb_metric *m);

/* SetNumberOfHistogramBins, clamped to >= 5
 * (itkMattesMutualInformationImageToImageMetricv4.h:146). */
int gb_metric_set_number_of_histogram_bins(gb_metric *m, uint64_t bins);
/* JointHistogramMutualInformationImageToImageMetricv4::SetVarianceForJointPDFSmoothing
 * (default 1.5; <= 0: no smoothing), Registration/Metricsv4/include/itkJointHistogramMutualInformationImageToImageMetricv4.h:141.
 * The joint-histogram metric takes affine, B-spline, [affine, B-spline] and
 * displacement-field transforms and 6 to 64 bins (default 20). */
int gb_metric_set_joint_pdf_smoothing_variance(gb_metric *m, double variance);
/* SetUseFloatingPointCorrection(on) / SetFloatingPointCorrectionResolution(resolution)
 * (Registration/Metricsv4/include/itkImageToImageMetricv4.h:604-621; applied in
 * ...GetValueAndDerivativeThreaderBase.hxx:284-294): each point's local derivative
 * truncated to 1 / resolution before it is summed.  Runs MeanSquares with affine
 * transforms (summed in FP64); no effect on Mattes, correlation and displacement
 * fields, as in the reference; other combinations are GB_ERR_UNSUPPORTED at Initialize. */
int gb_metric_set_floating_point_correction(gb_metric *m, int on, double resolution);

/* SetFixedImage / SetMovingImage (itkImageToImageMetricv4.h SetFixedImage /
 * SetMovingImage): float voxels, x fastest, size[3] = (nx, ny, nz), start
 * index 0, direction row-major 3x3.  The voxels are copied into HBM. */
int gb_metric_set_image(gb_metric *m, int which, const float *voxels, const int64_t size[3],
                        const double spacing[3], const double origin[3], const double direction[9]);
/* Same, from a device pointer (no host round trip; copied device-to-device). */
int gb_metric_set_image_device(gb_metric *m, int which, const float *device_voxels, const int64_t size[3],
                               const double spacing[3], const double origin[3], const double direction[9]);

/* Moving-image gradient.  GB_GRADIENT_IMAGE expects a call to
 * gb_metric_set_moving_gradient_image (the CovariantVector<double,3> image the
 * metric's gradient filter produces, itkImageToImageMetricv4.hxx:449-455);
 * GB_GRADIENT_CENTRAL_DIFFERENCE evaluates CentralDifferenceImageFunction at
 * each mapped point (SetUseMovingImageGradientFilter(false),
 * Core/ImageFunction/include/itkCentralDifferenceImageFunction.hxx:256-316);
 * GB_GRADIENT_RECURSIVE_GAUSSIAN runs GradientRecursiveGaussianImageFilter on
 * the device (sigma = max spacing, normalized across scale, image direction
 * applied; itkImageToImageMetricv4.hxx:488-503). */
int gb_metric_set_gradient_source(gb_metric *m, int source);
/* gradient: 3 doubles per voxel (x, y, z), same grid as the moving image */
int gb_metric_set_moving_gradient_image(gb_metric *m, const double *gradient_xyz);

/* Virtual domain (SetVirtualDomain, itkImageToImageMetricv4.h); when never
 * set, the fixed image geometry is used (itkImageToImageMetricv4.hxx:98-112). */
int gb_metric_set_virtual_domain(gb_metric *m, const int64_t size[3], const double spacing[3],
                                 const double origin[3], const double direction[9]);

/* Per-level set-up of ImageRegistrationMethodv4::InitializeRegistrationAtEachLevel
 * (Registration/RegistrationMethodsv4/include/itkImageRegistrationMethodv4.hxx:262-640),
 * done on the device by gb_metric_initialize, so a level's images never leave HBM:
 *   level smoothing: the fixed and moving images pass through
 *     SmoothingRecursiveGaussianImageFilter with sigma in physical units, or in
 *     voxels (times each axis' spacing) when sigma_in_physical_units = 0
 *     (SetSmoothingSigmasAreSpecifiedInPhysicalUnits); 0 = no smoothing;
 *   level shrink: the virtual domain is the fixed image's geometry through
 *     ShrinkImageFilter with these factors ({1,1,1} = full resolution); a domain
 *     set with gb_metric_set_virtual_domain takes precedence.
 * The images given with gb_metric_set_image stay unmodified. */
int gb_metric_set_level_smoothing(gb_metric *m, double sigma, int sigma_in_physical_units);
int gb_metric_set_level_shrink(gb_metric *m, const int64_t factors[3]);

/* Sampled point sets: float xyz, n points.  virtual_space = 1 replaces
 * SetVirtualSampledPointSet + UseVirtualSampledPointSetOn (what
 * ImageRegistrationMethodv4::SetMetricSamplePoints installs,
 * Registration/RegistrationMethodsv4/include/itkImageRegistrationMethodv4.hxx:1010-1021);
 * virtual_space = 0 replaces SetFixedSampledPointSet (mapped to the virtual
 * domain by MapFixedSampledPointSetToVirtual, itkImageToImageMetricv4.hxx:568-612). */
int gb_metric_set_sampled_points(gb_metric *m, const float *xyz, int64_t n, int virtual_space);
/* SetUseSampledPointSet(on) */
int gb_metric_use_sampled_point_set(gb_metric *m, int on);

/* Moving transform (SetMovingTransform).  Flat encodings:
 *   AFFINE    params = 12 (row-major matrix, translation), fixed = centre (3)
 *             -- AffineTransform<double,3>, Core/Transform/include/itkMatrixOffsetTransformBase.hxx:464-561
 *   BSPLINE   params = 3*nper coefficients, fixed = 18 (grid size, origin,
 *             spacing, direction) -- BSplineTransform<double,3,3>,
 *             Core/Transform/include/itkBSplineTransform.hxx:243-283
 *   COMPOSITE params = 3*nper B-spline coefficients (optimized), fixed = 18
 *             B-spline fixed parameters + 12 initial-affine parameters + 3
 *             initial-affine centre -- CompositeTransform [affine, bspline]
 *             with only the B-spline optimized, Core/Transform/include/itkCompositeTransform.hxx:60-70,466-580
 *   DISPLACEMENT_FIELD params = 3 per field voxel (x, y, z; voxels x fastest),
 *             fixed = 18 (field size, origin, spacing, direction) --
 *             DisplacementFieldTransform<double,3>,
 *             Filtering/DisplacementField/include/itkDisplacementFieldTransform.hxx:67-100,520-570.
 *             Local support: Initialize requires the field to share the virtual
 *             domain's grid (Numerics/Optimizersv4/include/itkObjectToObjectMetric.hxx:444-503);
 *             the derivative is a field too, each point's block added at its
 *             virtual voxel and not divided by the number of valid points
 *             (Registration/Metricsv4/include/itkImageToImageMetricv4GetValueAndDerivativeThreaderBase.hxx:128-172,276-327).
 *             fixed = 33 appends an initial affine (12 parameters, centre 3): the
 *             CompositeTransform [affine, displacement field], the field applied
 *             first and optimized, the local derivative M^T-mapped.
 *             MeanSquares and Mattes only. */
int gb_metric_set_moving_transform(gb_metric *m, int kind, const double *params, int64_t nparams,
                                   const double *fixed, int64_t nfixed);
/* SetParameters of the optimized transform (per optimizer iteration). */
int gb_metric_set_parameters(gb_metric *m, const double *params, int64_t nparams);
/* UpdateTransformParameters(update, factor): params += factor*update
 * (Core/Transform/include/itkTransform.hxx:71-120). */
int gb_metric_update_transform_parameters(gb_metric *m, const double *update, int64_t nparams, double factor);
int gb_metric_get_parameters(gb_metric *m, double *params, int64_t nparams);
int gb_metric_get_number_of_parameters(gb_metric *m, int64_t *nparams);

/* Initialize() (itkImageToImageMetricv4.hxx:72-172; Mattes bins and ranges
 * itkMattesMutualInformationImageToImageMetricv4.hxx:75-327).  Builds the
 * device sample list, the fixed values / fixed Parzen bins, the packed moving
 * image and its gradient. */
int gb_metric_initialize(gb_metric *m);

/* GetValueAndDerivative(value, derivative) (itkImageToImageMetricv4.hxx:218-231):
 * derivative has nparams entries and is overwritten. */
int gb_metric_get_value_and_derivative(gb_metric *m, double *value, double *derivative, int64_t nparams);
/* GetValue() (itkImageToImageMetricv4.hxx:182-196). */
int gb_metric_get_value(gb_metric *m, double *value);
/* GetNumberOfValidPoints() of the last evaluation. */
int gb_metric_get_number_of_valid_points(gb_metric *m, uint64_t *nvalid);
/* GetNumberOfDomainPoints(): samples (or virtual voxels) evaluated per call. */
int gb_metric_get_number_of_domain_points(gb_metric *m, uint64_t *n);
/* GetJointPDF() of the last Mattes evaluation: bins*bins doubles, row = fixed bin. */
int gb_metric_get_joint_pdf(gb_metric *m, double *out, int64_t n);
/* Mattes ranges: fixed min, fixed max, moving min, moving max, fixed bin size,
 * moving bin size, fixed normalized min, moving normalized min. */
int gb_metric_get_mattes_state(gb_metric *m, double out8[8]);

/* ---- device-resident form (no host copies) ----------------------------- */
/* Device memory the handle holds (images, pyramids, samples, caches, optimizer state), in bytes. */
int gb_metric_get_device_bytes(gb_metric *m, uint64_t *bytes);
/* CUDA stream the handle launches on (cudaStream_t as an integer). */
int gb_metric_get_stream(gb_metric *m, uint64_t *stream);
/* Enqueue one evaluation on the handle's stream with the parameters already
 * in device memory (nparams doubles) and write value, derivative and the
 * valid-point count (as a double) to device memory: out = [value, nvalid,
 * derivative...].  Asynchronous; use gb_metric_status_device for the status. */
int gb_metric_evaluate_device(gb_metric *m, const double *device_params, double *device_out, int with_derivative);
/* Synchronize the handle's stream and return the status of the last enqueued evaluation. */
int gb_metric_synchronize(gb_metric *m);

/* ---- allocation-free MeanSquares --------------------------------------- */
/* No counterpart in the reference: an extra entry point of this library.
 *
 * For callers that cannot call cudaMalloc -- code running inside another
 * framework's memory pool or arena, real-time loops that forbid allocation
 * after start-up, hosts that account for every device allocation -- this
 * evaluates MeanSquares value and derivative under an affine transform
 * without allocating anything.  The caller passes device pointers to:
 *   samples  n float4 records (x, y, z, fixed value): virtual-space points
 *            and the fixed image's value there, 16-byte aligned;
 *   moving   one float4 per moving voxel (value, gx, gy, gz), x fastest,
 *            16-byte aligned;
 *   out      14 doubles: value, number of valid points, derivative[12].
 * Geometry, the 12 affine parameters and the centre are host arrays.  The
 * call is asynchronous on `stream` (a cudaStream_t, 0 for the default
 * stream), so the return code covers only the arguments and the launch.
 * When no sample maps inside the moving image the call still succeeds and
 * leaves out = [DBL_MAX, 0, 0...], as VerifyNumberOfValidPoints leaves the
 * reference metric: out[1] == 0 is the only "no valid points" signal.
 * Scratch: one static device array of GB_NOALLOC_SCRATCH_BYTES bytes that
 * every GPU loading this library holds until the process exits.  The first
 * call under each CUDA context (the device's primary context, again after a
 * cudaDeviceReset, or a context the caller made current) looks up the array's
 * device address (cudaGetSymbolAddress) with that context current, so make
 * that first call before any stream capture.  All calls share the array:
 * calls that overlap on the GPU (other streams, other host threads) race;
 * serialize them.
 * Limits: n <= GB_NOALLOC_MAX_SAMPLES, moving voxels <= GB_NOALLOC_MAX_VOXELS;
 * larger sizes are rejected with GB_ERR_BAD_ARG. */
#define GB_NOALLOC_SCRATCH_BYTES 114176
#define GB_NOALLOC_MAX_SAMPLES 2147483647LL
#define GB_NOALLOC_MAX_VOXELS 2147483648LL
int gb_msq_affine_noalloc(const void *device_samples, int64_t n, const void *device_moving,
                          const int64_t moving_size[3], const double moving_spacing[3],
                          const double moving_origin[3], const double moving_direction[9],
                          const double params[12], const double center[3], double *device_out, uint64_t stream);

/* ---- device image filters ---------------------------------------------- */
/* Device forms of the filters the registration method and the metric run per
 * level; device buffers in, device buffers out, enqueued on `stream` (0: the
 * legacy default stream); scratch comes from the stream-ordered allocator.
 * Images are x-fastest float buffers of size[0] x size[1] x size[2], each axis >= 4.
 *
 * SmoothingRecursiveGaussianImageFilter<Image<float,3>> with a sigma per axis in
 * physical units (Filtering/Smoothing/include/itkSmoothingRecursiveGaussianImageFilter.hxx);
 * d_in and d_out may be the same buffer. */
int gb_smooth_recursive_gaussian(gb_ctx *ctx, uint64_t stream, const float *d_in, float *d_out, const int64_t size[3],
                                 const double spacing[3], const double sigma[3]);
/* GradientRecursiveGaussianImageFilter<Image<float,3>>
 * (Filtering/ImageGradient/include/itkGradientRecursiveGaussianImageFilter.hxx):
 * 3 floats (x, y, z) per voxel in d_out_xyz. */
int gb_gradient_recursive_gaussian(gb_ctx *ctx, uint64_t stream, const float *d_in, float *d_out_xyz,
                                   const int64_t size[3], const double spacing[3], const double direction[9],
                                   double sigma, int normalize_across_scale, int use_image_direction);
/* The same two filters on host buffers (copied in and out; synchronous). */
int gb_smooth_recursive_gaussian_host(gb_ctx *ctx, const float *in, float *out, const int64_t size[3],
                                      const double spacing[3], const double sigma[3]);
int gb_gradient_recursive_gaussian_host(gb_ctx *ctx, const float *in, float *out_xyz, const int64_t size[3],
                                        const double spacing[3], const double direction[9], double sigma,
                                        int normalize_across_scale, int use_image_direction);
/* ShrinkImageFilter output geometry for start index 0
 * (Filtering/ImageGrid/include/itkShrinkImageFilter.hxx:230-290). */
int gb_shrink_geometry(const int64_t size[3], const double spacing[3], const double origin[3],
                       const double direction[9], const int64_t factors[3], int64_t out_size[3],
                       double out_spacing[3], double out_origin[3]);

/* ---- device optimizer --------------------------------------------------- */
/* Stop conditions, numbered as StopConditionObjectToObjectOptimizerEnum
 * (Numerics/Optimizersv4/include/itkObjectToObjectOptimizerBase.h:42-51). */
enum {
  GB_STOP_MAXIMUM_NUMBER_OF_ITERATIONS = 0,
  GB_STOP_COSTFUNCTION_ERROR = 1,
  GB_STOP_UPDATE_PARAMETERS_ERROR = 2,
  GB_STOP_STEP_TOO_SMALL = 3,
  GB_STOP_CONVERGENCE_CHECKER_PASSED = 4,
  GB_STOP_GRADIENT_MAGNITUDE_TOLERANCE = 5,
  GB_STOP_OTHER_ERROR = 6
};

/* RegularStepGradientDescentOptimizerv4 settings; the reference's defaults are
 * learning rate 1, relaxation 0.5, minimum step 1e-4, gradient tolerance 1e-4,
 * 100 iterations, return-best off. */
typedef struct {
  double learning_rate;
  double relaxation_factor;
  double minimum_step_length;
  double gradient_magnitude_tolerance;
  int64_t number_of_iterations;
  int return_best_parameters_and_value;
} gb_regular_step_settings;

typedef struct {
  int stop_condition;          /* GB_STOP_* */
  int metric_status;           /* status of the evaluation that stopped it (GB_OK unless COSTFUNCTION_ERROR) */
  int64_t iterations;          /* GetCurrentIteration() */
  double value;                /* GetValue(): the current (or, with return-best, the best) metric value */
  double current_step_length;  /* GetCurrentStepLength() */
  double gradient_magnitude;   /* magnitude of the last scaled gradient */
  double learning_rate_relaxation;
} gb_optimizer_report;

/* RegularStepGradientDescentOptimizerv4::StartOptimization on an initialized
 * metric (Numerics/Optimizersv4/include/itkRegularStepGradientDescentOptimizerv4.hxx:39-171,
 * the loop of itkGradientDescentOptimizerv4.hxx:72-169): every iteration is one
 * GetValueAndDerivative at the current parameters and one AdvanceOneStep
 * (gradient / scales, ||g|| and g . g_prev by compensated sums, relaxation,
 * update of the moving transform's parameters by g * relaxation * rate / ||g||),
 * all in device memory on the handle's stream; the host only enqueues batches
 * of iterations and reads the stop flag between batches.  scales: nscales = the
 * number of parameters (each > DBL_EPSILON; within 0.01 of 1 everywhere counts as
 * identity, as ObjectToObjectOptimizerBase does), or nscales = 0 for identity.
 * On return the handle's parameters are the optimizer's final position
 * (gb_metric_get_parameters).  A metric error during the loop stops it with
 * GB_STOP_COSTFUNCTION_ERROR and is returned as the metric's status. */
int gb_metric_optimize_regular_step(gb_metric *m, const gb_regular_step_settings *settings, const double *scales,
                                    int64_t nscales, gb_optimizer_report *report);
/* Capture each optimizer iteration in a CUDA graph (default on). */
int gb_metric_set_optimizer_graphs(gb_metric *m, int on);

/* ---- batched registrations ---------------------------------------------- */
/* No counterpart in the reference (which runs one registration per optimizer):
 * many affine registrations, each an initialized metric handle with its own
 * RegularStepGradientDescentOptimizerv4 settings, advance together -- one
 * launch per phase of an iteration for all of them (accumulator clear,
 * transform constants, MeanSquares pass, Mattes pass 1, Mattes pass 2,
 * AdvanceOneStep), captured as a CUDA graph -- or, in the persistent form, one
 * launch for several iterations.  A registration's results do not depend on which others share
 * the batch.  While a metric is in a batch, make
 * no other call on it. */
typedef struct gb_batch gb_batch;
int gb_batch_create(gb_ctx *ctx, gb_batch **out);
int gb_batch_destroy(gb_batch *b);
/* StartOptimization of one registration in the batch; *slot identifies it. */
int gb_batch_add(gb_batch *b, gb_metric *m, const gb_regular_step_settings *settings, const double *scales,
                 int64_t nscales, int64_t *slot);
/* Advance every running registration by up to max_iterations iterations
 * (<= 0: until all have stopped); *running (may be null) = those still running. */
int gb_batch_run(gb_batch *b, int64_t max_iterations, int64_t *running);
/* *finished = 1 once registration `slot` has stopped; then *report is filled,
 * the metric handle holds the final parameters, and the return value is the
 * registration's status (as gb_metric_optimize_regular_step returns it). */
int gb_batch_result(gb_batch *b, int64_t slot, int *finished, gb_optimizer_report *report);
/* Samples per block of the MeanSquares pass, Mattes pass 1 and Mattes pass 2
 * (default 8192 each); gb_batch_autotune picks them by timing the batch's
 * evaluations (no optimizer state changes) and leaves the fastest set. */
int gb_batch_set_samples_per_block(gb_batch *b, const int64_t spb[3]);
int gb_batch_get_samples_per_block(gb_batch *b, int64_t spb[3]);
int gb_batch_autotune(gb_batch *b, int iterations, int64_t spb[3]);
/* Capture the iteration in a CUDA graph (default on; the per-phase form). */
int gb_batch_set_graphs(gb_batch *b, int on);
/* The persistent form (default off): every iteration of every running
 * registration -- clears, constants, metric passes, steps -- in one kernel
 * launch that runs several iterations, each work item waiting (bounded) only
 * for its own registration's earlier items; off: one launch per phase and
 * iteration, captured as a CUDA graph.  A registration's results are bitwise
 * the same in both forms. */
int gb_batch_set_persistent(gb_batch *b, int on);
/* Iterations launched, table rebuilds (registrations joining or leaving) and
 * the host seconds they took, since the batch was created. */
int gb_batch_get_stats(gb_batch *b, int64_t *iterations, int64_t *rebuilds, double *rebuild_seconds);

/* ---- metric sample points ----------------------------------------------- */
/* ImageRegistrationMethodv4's sampling strategies
 * (Registration/RegistrationMethodsv4/include/itkImageRegistrationMethodv4.h, MetricSamplingStrategyEnum). */
enum { GB_SAMPLING_NONE = 0, GB_SAMPLING_REGULAR = 1, GB_SAMPLING_RANDOM = 2 };
/* Number of points gb_sample_points makes for a virtual domain of `size`
 * voxels: RANDOM (unsigned long)((float)voxels * percentage), REGULAR every
 * ceil(1 / percentage)-th voxel in scan order, NONE every voxel. */
int gb_sample_count(int strategy, const int64_t size[3], double percentage, int64_t *count);
/* ImageRegistrationMethodv4::SetMetricSamplePoints for one image metric and no
 * fixed mask (Registration/RegistrationMethodsv4/include/itkImageRegistrationMethodv4.hxx:869-1024),
 * bit for bit: REGULAR or RANDOM voxels of the virtual domain (geometry given),
 * each moved by N(0,1) * spacing / 3 per axis, as float points (x, y, z) in
 * xyz[0 .. 3 * count).  seed is the method's current random seed at this
 * level: the jitter generator takes seed, RANDOM's voxel iterator seed + 1;
 * *next_seed (may be null) receives the seed the next level starts from. */
int gb_sample_points(int strategy, const int64_t size[3], const double spacing[3], const double origin[3],
                     const double direction[9], double percentage, int32_t seed, float *xyz, int64_t capacity,
                     int64_t *count, int32_t *next_seed);

/* ---- observability ----------------------------------------------------- */
/* Per-kernel CUDA-event timing of evaluations (the reference's TimeProbe,
 * Core/Common/include/itkTimeProbe.h:44, at kernel granularity).  When on,
 * each evaluation records an event before and after every kernel it launches. */
int gb_metric_set_profiling(gb_metric *m, int on);
/* Device milliseconds of each kernel of the last evaluation, in launch order
 * (affine MeanSquares: 1 kernel; affine Mattes: pass 1 then pass 2, or the
 * value-only finalize; B-spline: [node conversion], the sample pass, [Mattes
 * finalize], chunk sums, parameter gather).  Synchronizes. */
int gb_metric_get_kernel_times(gb_metric *m, double *ms, int max_kernels, int *count);

/* ---- failure detection ------------------------------------------------- */
/* No counterpart in the reference (whose failures are exceptions thrown by
 * the metric): a test hook for the device-side failure path.  Every wait of
 * the kernels on an asynchronous copy is bounded; when one runs out the
 * kernel records GB_ERR_TIMEOUT, waits (bounded) for its other copies in
 * flight and returns, so the context stays usable and the call reports the
 * status.  GB_FAULT_STALLED_COPY makes the affine Mattes derivative pass
 * issue none of its streamed record copies (with a short wait limit), so its
 * waits run out: GetValueAndDerivative then returns GB_ERR_TIMEOUT.
 * GB_FAULT_NONE restores normal evaluations. */
enum { GB_FAULT_NONE = 0, GB_FAULT_STALLED_COPY = 1 };
int gb_metric_set_fault_injection(gb_metric *m, int fault);

#ifdef __cplusplus
}
#endif
#endif /* ITK_GB300_H */
