"""Host-side mirror of ITK's v4 image metrics over the GB300 C ABI.

Class and method names follow ``itk::MeanSquaresImageToImageMetricv4`` and
``itk::MattesMutualInformationImageToImageMetricv4`` on ``Image<float,3>``
(Registration/Metricsv4/include/itkImageToImageMetricv4.h,
itkMattesMutualInformationImageToImageMetricv4.h) so code written against
ITK reads the same: SetFixedImage / SetMovingImage / SetMovingTransform /
Initialize / GetValueAndDerivative.  Every evaluation runs on the GPU; errors
come back as ``ExceptionObject`` carrying the reference's message text.
"""
from __future__ import annotations

import ctypes
import warnings

import numpy as np

from . import _capi
from ._capi import ExceptionObject, check, f64, i64, ptr
from .image import GradientImage, Image

_ctx_cache = {}


def context(device: int = 0):
    """One ``gb_ctx`` per device, created on first use."""
    if device not in _ctx_cache:
        L = _capi.lib()
        h = ctypes.c_void_p()
        check(L.gb_ctx_create(device, ctypes.byref(h)))
        _ctx_cache[device] = h
    return _ctx_cache[device]


class ImageToImageMetricv4:
    """Common part of the two metrics (itkImageToImageMetricv4.h)."""

    _kind = None

    def __init__(self, device: int = 0):
        self._L = _capi.lib()
        self._h = ctypes.c_void_p()
        check(self._L.gb_metric_create(context(device), self._kind, ctypes.byref(self._h)))
        self._fixed = None
        self._moving = None
        self._transform = None
        self._gradient = None
        self._use_moving_gradient_filter = True
        self._use_sampled = False
        self._points = None
        self._points_virtual = True
        self._virtual = None
        self._value = np.finfo(np.float64).max
        self._nparams = 0
        self._level_sigma = 0.0
        self._level_sigma_physical = True
        self._level_shrink = (1, 1, 1)

    def __del__(self):
        try:
            if getattr(self, "_h", None) and self._h.value:
                self._L.gb_metric_destroy(self._h)
                self._h = ctypes.c_void_p()
        except Exception:
            pass

    # ---- inputs
    def SetFixedImage(self, image: Image):
        self._fixed = image
        self._set_image(_capi.GB_IMAGE_FIXED, image)

    def SetMovingImage(self, image: Image):
        self._moving = image
        self._set_image(_capi.GB_IMAGE_MOVING, image)

    def _set_image(self, which, image):
        a = image.array
        check(self._L.gb_metric_set_image(self._h, which, ptr(a), ptr(i64(image.GetSize())), ptr(f64(image.spacing)),
                                          ptr(f64(image.origin)), ptr(f64(image.direction.reshape(9)))))

    def GetFixedImage(self):
        return self._fixed

    def GetMovingImage(self):
        return self._moving

    def SetMovingTransform(self, transform):
        self._transform = transform

    def GetMovingTransform(self):
        return self._transform

    def SetUseFloatingPointCorrection(self, on: bool):
        """Truncate each point's local derivative to 1 / resolution before summing
        (MeanSquares with affine transforms; no effect on Mattes, correlation and
        displacement fields, as in the reference)."""
        self._fp_correction = bool(on)

    def GetUseFloatingPointCorrection(self):
        return getattr(self, "_fp_correction", False)

    def SetFloatingPointCorrectionResolution(self, resolution: float):
        self._fp_resolution = float(resolution)

    def GetFloatingPointCorrectionResolution(self):
        return getattr(self, "_fp_resolution", 1e6)  # the reference's default

    def SetUseMovingImageGradientFilter(self, on: bool):
        """False selects CentralDifferenceImageFunction at each mapped point."""
        self._use_moving_gradient_filter = bool(on)

    def GetUseMovingImageGradientFilter(self):
        return self._use_moving_gradient_filter

    def SetMovingImageGradientImage(self, gradient):
        """Supplies the gradient image the metric's gradient filter would compute."""
        self._gradient = gradient if isinstance(gradient, GradientImage) else GradientImage(gradient)

    def SetVirtualDomainFromImage(self, image: Image):
        self._virtual = image
        check(self._L.gb_metric_set_virtual_domain(self._h, ptr(i64(image.GetSize())), ptr(f64(image.spacing)),
                                                   ptr(f64(image.origin)), ptr(f64(image.direction.reshape(9)))))

    def SetFixedSampledPointSet(self, points):
        self._points = np.ascontiguousarray(np.asarray(points, np.float32).reshape(-1, 3))
        self._points_virtual = False

    def SetVirtualSampledPointSet(self, points):
        self._points = np.ascontiguousarray(np.asarray(points, np.float32).reshape(-1, 3))
        self._points_virtual = True

    def SetUseSampledPointSet(self, on: bool):
        self._use_sampled = bool(on)

    def UseSampledPointSetOn(self):
        self.SetUseSampledPointSet(True)

    def UseVirtualSampledPointSetOn(self):
        self._points_virtual = True

    # ---- per-level set-up of ImageRegistrationMethodv4 (done on the device at Initialize)
    def SetLevelSmoothingSigma(self, sigma: float, in_physical_units: bool = True):
        """Smooth both images with SmoothingRecursiveGaussianImageFilter(sigma) at Initialize
        (ImageRegistrationMethodv4.hxx:590-640); 0 = no smoothing.  The inputs stay unmodified."""
        self._level_sigma = float(sigma)
        self._level_sigma_physical = bool(in_physical_units)

    def SetLevelShrinkFactors(self, factors):
        """Virtual domain = the fixed image's geometry through ShrinkImageFilter(factors)
        (ImageRegistrationMethodv4.hxx:448-461), unless a virtual domain was set."""
        self._level_shrink = tuple(int(f) for f in np.broadcast_to(np.asarray(factors), (3,)))

    # ---- set-up
    def _push_transform(self):
        kind, params, fixed = self._transform.flat()
        params, fixed = f64(params), f64(fixed)
        check(self._L.gb_metric_set_moving_transform(self._h, kind, ptr(params), params.size, ptr(fixed), fixed.size))
        self._nparams = params.size

    def Initialize(self):
        if self._fixed is None:
            raise ExceptionObject(_capi.GB_ERR_BAD_ARG, "FixedImage is not present")
        if self._moving is None:
            raise ExceptionObject(_capi.GB_ERR_BAD_ARG, "MovingImage is not present")
        if self._transform is None:
            raise ExceptionObject(_capi.GB_ERR_BAD_ARG, "MovingTransform is not present")
        self._push_transform()
        if self._use_moving_gradient_filter:
            if self._gradient is not None:
                check(self._L.gb_metric_set_gradient_source(self._h, _capi.GB_GRADIENT_IMAGE))
                check(self._L.gb_metric_set_moving_gradient_image(self._h, ptr(self._gradient.array)))
            else:
                check(self._L.gb_metric_set_gradient_source(self._h, _capi.GB_GRADIENT_RECURSIVE_GAUSSIAN))
        else:
            check(self._L.gb_metric_set_gradient_source(self._h, _capi.GB_GRADIENT_CENTRAL_DIFFERENCE))
        if self._use_sampled:
            if self._points is None or len(self._points) == 0:
                raise ExceptionObject(_capi.GB_ERR_BAD_ARG, "VirtualSampledPointSet must have 1 or more points.")
            check(self._L.gb_metric_set_sampled_points(self._h, ptr(self._points), self._points.shape[0],
                                                       int(self._points_virtual)))
        check(self._L.gb_metric_use_sampled_point_set(self._h, int(self._use_sampled)))
        check(self._L.gb_metric_set_floating_point_correction(self._h, int(self.GetUseFloatingPointCorrection()),
                                                               self.GetFloatingPointCorrectionResolution()))
        check(self._L.gb_metric_set_level_smoothing(self._h, self._level_sigma, int(self._level_sigma_physical)))
        check(self._L.gb_metric_set_level_shrink(self._h, ptr(i64(self._level_shrink))))
        self._pre_initialize()
        check(self._L.gb_metric_initialize(self._h))

    def _pre_initialize(self):
        pass

    # ---- evaluation
    def _sync_params(self):
        view = getattr(self._transform, "parameters_view", None)  # a displacement field: no copy
        p = view() if view is not None else f64(self._transform.GetParameters())
        if p.size != self._nparams:
            raise ExceptionObject(_capi.GB_ERR_BAD_ARG, "transform parameter count changed; call Initialize()")
        # .ctypes.data: the array is held by the local name for the call (data_as costs ~2 us)
        check(self._L.gb_metric_set_parameters(self._h, p.ctypes.data, p.size))

    def _handle_status(self, rc):
        if rc == _capi.GB_OK:
            return
        if rc == _capi.GB_ERR_NO_VALID_POINTS and self._kind != _capi.GB_METRIC_MATTES:
            warnings.warn(_capi.last_error())
            return
        raise ExceptionObject(rc, _capi.last_error())

    def GetValueAndDerivative(self):
        """Returns (value, derivative) like GetValueAndDerivative(value, derivative)."""
        self._sync_params()
        value = np.zeros(1)
        deriv = np.empty(self._nparams)  # every entry is written by the call
        rc = self._L.gb_metric_get_value_and_derivative(self._h, value.ctypes.data, deriv.ctypes.data, self._nparams)
        self._handle_status(rc)
        self._value = float(value[0])
        return self._value, deriv

    def GetValue(self):
        self._sync_params()
        value = np.zeros(1)
        rc = self._L.gb_metric_get_value(self._h, ptr(value))
        self._handle_status(rc)
        self._value = float(value[0])
        return self._value

    def GetDerivative(self):
        return self.GetValueAndDerivative()[1]

    def GetCurrentValue(self):
        return self._value

    def GetNumberOfValidPoints(self):
        n = ctypes.c_uint64()
        check(self._L.gb_metric_get_number_of_valid_points(self._h, ctypes.byref(n)))
        return int(n.value)

    def GetNumberOfDomainPoints(self):
        n = ctypes.c_uint64()
        check(self._L.gb_metric_get_number_of_domain_points(self._h, ctypes.byref(n)))
        return int(n.value)

    def GetDeviceBytes(self) -> int:
        """Device memory this metric holds (images, pyramid, samples, caches, optimizer state)."""
        n = ctypes.c_uint64()
        check(self._L.gb_metric_get_device_bytes(self._h, ctypes.byref(n)))
        return int(n.value)

    def GetNumberOfParameters(self):
        return self._transform.GetNumberOfParameters()

    def HasLocalSupport(self) -> bool:
        """True under a displacement field: the derivative is a field over the virtual domain."""
        return getattr(self._transform, "kind", None) == _capi.GB_TRANSFORM_DISPLACEMENT_FIELD

    def GetNumberOfLocalParameters(self):
        return 3 if self.HasLocalSupport() else self.GetNumberOfParameters()

    def UpdateTransformParameters(self, update, factor=1.0):
        self._transform.UpdateTransformParameters(update, factor)

    # ---- device-resident form
    @property
    def handle(self):
        return self._h

    def stream(self) -> int:
        s = ctypes.c_uint64()
        check(self._L.gb_metric_get_stream(self._h, ctypes.byref(s)))
        return int(s.value)

    def evaluate_device(self, device_params_ptr: int, device_out_ptr: int, with_derivative: bool = True):
        check(self._L.gb_metric_evaluate_device(self._h, ctypes.c_void_p(device_params_ptr),
                                                ctypes.c_void_p(device_out_ptr), int(with_derivative)))

    def synchronize(self) -> int:
        return self._L.gb_metric_synchronize(self._h)

    def set_fault_injection(self, fault: int):
        """Failure-detection test hook (gb_metric_set_fault_injection): GB_FAULT_STALLED_COPY makes
        the affine Mattes derivative pass's bounded copy waits run out (GB_ERR_TIMEOUT);
        GB_FAULT_NONE restores normal evaluations."""
        check(self._L.gb_metric_set_fault_injection(self._h, int(fault)))

    def set_profiling(self, on: bool = True):
        check(self._L.gb_metric_set_profiling(self._h, int(on)))

    def kernel_times_ms(self):
        """Device milliseconds of each kernel of the last evaluation (profiling on)."""
        buf = np.zeros(8)
        n = ctypes.c_int()
        check(self._L.gb_metric_get_kernel_times(self._h, ptr(buf), 8, ctypes.byref(n)))
        return buf[:n.value].copy()


class MeanSquaresImageToImageMetricv4(ImageToImageMetricv4):
    """Mean of squared intensity differences; derivative 2 (f - m) J^T grad m / N."""

    _kind = _capi.GB_METRIC_MEAN_SQUARES


class CorrelationImageToImageMetricv4(ImageToImageMetricv4):
    """Normalized cross correlation: value -(sum f1 m1)^2 / (sum f1^2 sum m1^2) with
    f1, m1 the intensities less their averages over the valid points (affine,
    B-spline and [affine, B-spline] transforms)."""

    _kind = _capi.GB_METRIC_CORRELATION


class JointHistogramMutualInformationImageToImageMetricv4(ImageToImageMetricv4):
    """Joint-histogram mutual information (value -MI in bits): counts of (fixed, moving)
    intensity bins over the valid points, normalized and smoothed by a discrete
    Gaussian; the derivative from the smoothed PDF's slope along the moving axis
    (affine, B-spline, [affine, B-spline] and displacement-field transforms; default
    20 bins, variance 1.5)."""

    _kind = _capi.GB_METRIC_JOINT_HISTOGRAM_MI

    def __init__(self, device: int = 0):
        super().__init__(device)
        self._bins = 20
        self._variance = 1.5

    def SetNumberOfHistogramBins(self, bins: int):
        self._bins = max(int(bins), 5)  # itkSetClampMacro(..., 5, max)

    def GetNumberOfHistogramBins(self):
        return self._bins

    def SetVarianceForJointPDFSmoothing(self, variance: float):
        self._variance = float(variance)

    def GetVarianceForJointPDFSmoothing(self):
        return self._variance

    def _pre_initialize(self):
        check(self._L.gb_metric_set_number_of_histogram_bins(self._h, self._bins))
        check(self._L.gb_metric_set_joint_pdf_smoothing_variance(self._h, self._variance))

    def GetJointPDF(self):
        """The smoothed joint PDF of the last evaluation as the reference's image buffer
        (fixed bin fastest): out[moving bin, fixed bin]."""
        out = np.zeros((self._bins, self._bins))
        check(self._L.gb_metric_get_joint_pdf(self._h, ptr(out), out.size))
        return out


class MattesMutualInformationImageToImageMetricv4(ImageToImageMetricv4):
    """Mattes mutual information with cubic B-spline Parzen windows (default 50 bins)."""

    _kind = _capi.GB_METRIC_MATTES

    def __init__(self, device: int = 0):
        super().__init__(device)
        self._bins = 50

    def SetNumberOfHistogramBins(self, bins: int):
        self._bins = max(int(bins), 5)  # itkSetClampMacro(..., 5, max)

    def GetNumberOfHistogramBins(self):
        return self._bins

    def _pre_initialize(self):
        check(self._L.gb_metric_set_number_of_histogram_bins(self._h, self._bins))

    def GetJointPDF(self):
        out = np.zeros((self._bins, self._bins))
        check(self._L.gb_metric_get_joint_pdf(self._h, ptr(out), out.size))
        return out

    def GetHistogramState(self):
        """(fixed min, fixed max, moving min, moving max, fixed bin size, moving bin size,
        fixed normalized min, moving normalized min)."""
        out = np.zeros(8)
        check(self._L.gb_metric_get_mattes_state(self._h, ptr(out)))
        return out
