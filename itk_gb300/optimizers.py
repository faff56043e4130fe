"""RegularStepGradientDescentOptimizerv4 with its loop on the device.

Mirrors itk::RegularStepGradientDescentOptimizerv4<double>
(Modules/Numerics/Optimizersv4/include/itkRegularStepGradientDescentOptimizerv4.h):
the same settings, defaults, stop conditions and stop-condition texts.
StartOptimization runs every iteration -- the metric evaluation and
AdvanceOneStep -- in device memory through gb_metric_optimize_regular_step;
the metric must have been initialized (the registration method initializes it
per level, as the reference does).  The moving transform's parameters are
updated in place when the loop ends.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import ExceptionObject, OptimizerReport, RegularStepSettings, check, f64, ptr

_STOP_NAMES = {
    _capi.GB_STOP_MAXIMUM_NUMBER_OF_ITERATIONS: "MAXIMUM_NUMBER_OF_ITERATIONS",
    _capi.GB_STOP_COSTFUNCTION_ERROR: "COSTFUNCTION_ERROR",
    _capi.GB_STOP_UPDATE_PARAMETERS_ERROR: "UPDATE_PARAMETERS_ERROR",
    _capi.GB_STOP_STEP_TOO_SMALL: "STEP_TOO_SMALL",
    _capi.GB_STOP_CONVERGENCE_CHECKER_PASSED: "CONVERGENCE_CHECKER_PASSED",
    _capi.GB_STOP_GRADIENT_MAGNITUDE_TOLERANCE: "GRADIENT_MAGNITUDE_TOLEARANCE",
    _capi.GB_STOP_OTHER_ERROR: "OTHER_ERROR",
}


class RegularStepGradientDescentOptimizerv4:
    """Defaults as the reference's constructors set them: learning rate 1,
    relaxation factor 0.5, minimum step length 1e-4, gradient magnitude
    tolerance 1e-4, 100 iterations, return-best off, identity scales."""

    def __init__(self):
        self._metric = None
        self._learning_rate = 1.0
        self._relaxation_factor = 0.5
        self._minimum_step_length = 1e-4
        self._gradient_magnitude_tolerance = 1e-4
        self._number_of_iterations = 100
        self._return_best = False
        self._scales = None
        self._report = OptimizerReport()
        self._report.stop_condition = _capi.GB_STOP_MAXIMUM_NUMBER_OF_ITERATIONS
        self._report.learning_rate_relaxation = 0.0
        self._use_graphs = True

    # ---- settings
    def SetMetric(self, metric):
        self._metric = metric

    def GetMetric(self):
        return self._metric

    def SetLearningRate(self, v: float):
        self._learning_rate = float(v)

    def GetLearningRate(self) -> float:
        return self._learning_rate

    def SetRelaxationFactor(self, v: float):
        self._relaxation_factor = float(v)

    def GetRelaxationFactor(self) -> float:
        return self._relaxation_factor

    def SetMinimumStepLength(self, v: float):
        self._minimum_step_length = float(v)

    def GetMinimumStepLength(self) -> float:
        return self._minimum_step_length

    def SetGradientMagnitudeTolerance(self, v: float):
        self._gradient_magnitude_tolerance = float(v)

    def GetGradientMagnitudeTolerance(self) -> float:
        return self._gradient_magnitude_tolerance

    def SetNumberOfIterations(self, n: int):
        self._number_of_iterations = int(n)

    def GetNumberOfIterations(self) -> int:
        return self._number_of_iterations

    def SetReturnBestParametersAndValue(self, on: bool):
        self._return_best = bool(on)

    def ReturnBestParametersAndValueOn(self):
        self._return_best = True

    def ReturnBestParametersAndValueOff(self):
        self._return_best = False

    def GetReturnBestParametersAndValue(self) -> bool:
        return self._return_best

    def SetScales(self, scales):
        self._scales = None if scales is None else f64(scales)

    def GetScales(self):
        return self._scales

    def SetScalesEstimator(self, estimator):
        """A RegistrationParameterScalesFromPhysicalShift: with DoEstimateScales on (the
        default), StartOptimization sets the scales from it (GradientDescentOptimizerBasev4::
        StartOptimization, Numerics/Optimizersv4/include/itkGradientDescentOptimizerBasev4.hxx:132-143)."""
        self._scales_estimator = estimator

    def GetScalesEstimator(self):
        return getattr(self, "_scales_estimator", None)

    def SetDoEstimateScales(self, on: bool):
        self._do_estimate_scales = bool(on)

    def GetDoEstimateScales(self):
        return getattr(self, "_do_estimate_scales", True)

    def SetUseCudaGraphs(self, on: bool):
        """Capture each iteration in a CUDA graph (default on); off launches the kernels directly."""
        self._use_graphs = bool(on)

    # ---- run
    def StartOptimization(self, doOnlyInitialization: bool = False):
        m = self._metric
        if m is None:
            raise ExceptionObject(_capi.GB_ERR_BAD_ARG, "m_Metric must be set.")
        m._sync_params()
        est = self.GetScalesEstimator()
        if est is not None and self.GetDoEstimateScales():
            self._scales = f64(est.EstimateScales())
        if doOnlyInitialization:
            return
        s = RegularStepSettings(self._learning_rate, self._relaxation_factor, self._minimum_step_length,
                                self._gradient_magnitude_tolerance, self._number_of_iterations,
                                int(self._return_best))
        scales = self._scales
        L = _capi.lib()
        self._report = OptimizerReport()
        self._report.stop_condition = -1  # set by the call once the loop has run
        check(L.gb_metric_set_optimizer_graphs(m.handle, int(self._use_graphs)))
        rc = L.gb_metric_optimize_regular_step(m.handle, ctypes.byref(s), ptr(scales),
                                               0 if scales is None else scales.size, ctypes.byref(self._report))
        if rc != _capi.GB_OK and self._report.stop_condition != _capi.GB_STOP_COSTFUNCTION_ERROR:
            raise ExceptionObject(rc, _capi.last_error())
        # the transform now holds the optimizer's final position
        p = np.zeros(m._nparams)
        check(L.gb_metric_get_parameters(m.handle, ptr(p), p.size))
        m.GetMovingTransform().SetParameters(p)
        m._value = self._report.value
        if rc != _capi.GB_OK:  # the metric threw inside the loop; pass it on as the reference does
            raise ExceptionObject(rc, _capi.last_error())

    # ---- results
    def GetCurrentIteration(self) -> int:
        return int(self._report.iterations)

    def GetValue(self) -> float:
        return float(self._report.value)

    def GetCurrentMetricValue(self) -> float:
        return float(self._report.value)

    def GetCurrentStepLength(self) -> float:
        return float(self._report.current_step_length)

    def GetGradientMagnitude(self) -> float:
        return float(self._report.gradient_magnitude)

    def GetCurrentLearningRateRelaxation(self) -> float:
        return float(self._report.learning_rate_relaxation)

    def GetStopCondition(self) -> int:
        return int(self._report.stop_condition)

    def GetStopConditionName(self) -> str:
        return _STOP_NAMES.get(self.GetStopCondition(), "OTHER_ERROR")

    def GetCurrentPosition(self):
        return np.asarray(self._metric.GetMovingTransform().GetParameters(), dtype=np.float64)

    def GetStopConditionDescription(self) -> str:
        """The reference's texts (itkRegularStepGradientDescentOptimizerv4.hxx:117-148,
        itkGradientDescentOptimizerv4.hxx:84-104)."""
        r = self._report
        head = "RegularStepGradientDescentOptimizerv4Template: "
        c = r.stop_condition
        if c == _capi.GB_STOP_MAXIMUM_NUMBER_OF_ITERATIONS:
            return head + f"Maximum number of iterations ({self._number_of_iterations}) exceeded."
        if c == _capi.GB_STOP_GRADIENT_MAGNITUDE_TOLERANCE:
            return head + (f"Gradient magnitude tolerance met after {r.iterations - 1} iterations. Gradient magnitude "
                           f"({r.gradient_magnitude:g}) is less than gradient magnitude tolerance "
                           f"({self._gradient_magnitude_tolerance:g}).")
        if c == _capi.GB_STOP_STEP_TOO_SMALL:
            return head + (f"Step too small after {r.iterations - 1} iterations. Current step "
                           f"({r.current_step_length:g}) is less than minimum step ({self._minimum_step_length:g}).")
        if c == _capi.GB_STOP_COSTFUNCTION_ERROR:
            return head + "Metric error during optimization"
        return head + self.GetStopConditionName()
