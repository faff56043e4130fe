"""ImageRegistrationMethodv4: the multi-resolution loop around the metric and
the device optimizer.

Mirrors itk::ImageRegistrationMethodv4
(Modules/Registration/RegistrationMethodsv4/include/itkImageRegistrationMethodv4.h/.hxx):
per level (GenerateData, :786-804; InitializeRegistrationAtEachLevel, :262-717)
the fixed and moving images are smoothed with the level's sigma, the virtual
domain is the fixed geometry shrunk by the level's factors, the metric's
sample points are drawn (SetMetricSamplePoints, :869-1024, bit for bit through
gb_sample_points), the metric is initialized and the optimizer runs.  The
smoothing, shrink and gradient filtering happen inside the metric's Initialize
on the device; the optimizer loop runs on the device.
"""
from __future__ import annotations

import time

import numpy as np

from . import _capi
from ._capi import ExceptionObject, check, f64, i64, ptr
from .filters import shrink_geometry
from .image import Image
from .transforms import AffineTransform, CompositeTransform

NONE = _capi.GB_SAMPLING_NONE
REGULAR = _capi.GB_SAMPLING_REGULAR
RANDOM = _capi.GB_SAMPLING_RANDOM


def sample_count(strategy, size_xyz, percentage) -> int:
    n = np.zeros(1, np.int64)
    check(_capi.lib().gb_sample_count(int(strategy), ptr(i64(size_xyz)), float(percentage), ptr(n)))
    return int(n[0])


def sample_points(strategy, size_xyz, spacing, origin, direction, percentage, seed):
    """SetMetricSamplePoints over a virtual domain geometry: (float32 points (n, 3), next seed)."""
    size = i64(size_xyz)
    cap = sample_count(strategy, size, percentage)
    out = np.zeros((max(cap, 1), 3), np.float32)
    n = np.zeros(1, np.int64)
    nxt = np.zeros(1, np.int32)
    check(_capi.lib().gb_sample_points(int(strategy), ptr(size), ptr(f64(spacing)), ptr(f64(origin)),
                                       ptr(f64(np.asarray(direction).reshape(9))), float(percentage), int(seed),
                                       ptr(out), cap, ptr(n), ptr(nxt)))
    return out[:int(n[0])].copy(), int(nxt[0])


def setup_level(metric, fixed: Image, shrink, sigma, sigma_physical, strategy, percentage, seed):
    """InitializeRegistrationAtEachLevel for one image metric: the level's smoothing
    and virtual-domain shrink (done on the device by Initialize), the metric sample
    points (SetMetricSamplePoints), then Initialize.  Returns (points or None, the
    seed the next level starts from)."""
    metric.SetLevelShrinkFactors(shrink)
    metric.SetLevelSmoothingSigma(sigma, sigma_physical)
    pts = None
    if strategy != NONE:
        size, sp, org = shrink_geometry(fixed, shrink)
        pts, seed = sample_points(strategy, size, sp, org, fixed.direction, percentage, seed)
        metric.SetVirtualSampledPointSet(pts)
        metric.SetUseSampledPointSet(True)
    else:
        metric.SetUseSampledPointSet(False)
    metric.Initialize()
    return pts, seed


class ImageRegistrationMethodv4:
    """Defaults as the reference's: one level, shrink 1, sigma 0 in physical
    units, no sampling (the dense virtual domain), percentage 1."""

    def __init__(self):
        self._fixed = None
        self._moving = None
        self._metric = None
        self._optimizer = None
        self._transform = None
        self._moving_initial = None
        self._levels = 1
        self._shrink = [np.ones(3, np.int64)]
        self._sigmas = [0.0]
        self._sigmas_physical = True
        self._strategy = NONE
        self._percentages = [1.0]
        # MetricSamplingReinitializeSeed(int) fixes it; otherwise a clock-derived seed, as the reference
        self._random_seed = int(time.time_ns() & 0x7FFFFFFF)
        self._reseed_from_clock = False
        self._current_level = 0
        self._level_points = []
        self._composite = None

    # ---- inputs
    def SetFixedImage(self, image: Image):
        self._fixed = image

    def SetMovingImage(self, image: Image):
        self._moving = image

    def SetMetric(self, metric):
        self._metric = metric

    def GetMetric(self):
        return self._metric

    def SetOptimizer(self, optimizer):
        self._optimizer = optimizer

    def GetOptimizer(self):
        return self._optimizer

    def SetInitialTransform(self, transform):
        """The transform being optimized (updated in place, as with InPlace on)."""
        self._transform = transform

    def SetMovingInitialTransform(self, transform):
        self._moving_initial = transform

    def SetNumberOfLevels(self, n: int):
        n = int(n)
        self._levels = n
        self._shrink = [np.ones(3, np.int64)] * n
        self._sigmas = [0.0] * n
        self._percentages = [self._percentages[0]] * n

    def GetNumberOfLevels(self) -> int:
        return self._levels

    def SetShrinkFactorsPerLevel(self, factors):
        """One integer per level (all axes) or a triple per level."""
        out = []
        for f in factors:
            f = np.asarray(f, np.int64)
            out.append(np.full(3, int(f)) if f.ndim == 0 else f.reshape(3))
        self._shrink = out

    def SetSmoothingSigmasPerLevel(self, sigmas):
        self._sigmas = [float(s) for s in sigmas]

    def SetSmoothingSigmasAreSpecifiedInPhysicalUnits(self, on: bool):
        self._sigmas_physical = bool(on)

    def SetMetricSamplingStrategy(self, strategy: int):
        if strategy not in (NONE, REGULAR, RANDOM):
            raise ExceptionObject(_capi.GB_ERR_BAD_ARG, "Invalid sampling strategy requested.")
        self._strategy = strategy

    def SetMetricSamplingPercentage(self, p: float):
        self.SetMetricSamplingPercentagePerLevel([float(p)] * self._levels)

    def SetMetricSamplingPercentagePerLevel(self, ps):
        """Every percentage must lie in (0, 1]
        (RegistrationMethodsv4/include/itkImageRegistrationMethodv4.hxx:1266-1283)."""
        ps = [float(p) for p in ps]
        if ps != self._percentages:
            if any(not (0.0 < p <= 1.0) for p in ps):
                raise ExceptionObject(_capi.GB_ERR_BAD_ARG, "sampling percentage outside expected (0,1] range")
            self._percentages = ps

    def MetricSamplingReinitializeSeed(self, seed=None):
        if seed is None:
            self._reseed_from_clock = True
        else:
            self._reseed_from_clock = False
            self._random_seed = int(seed)

    # ---- outputs
    def GetTransform(self):
        return self._transform

    def GetModifiableTransform(self):
        return self._transform

    def GetCurrentLevel(self) -> int:
        return self._current_level

    def GetMetricSamplePoints(self, level: int):
        """The float points the metric sampled at a level (None for the dense domain)."""
        return self._level_points[level]

    # ---- run
    def _check(self):
        if self._fixed is None or self._moving is None:
            raise ExceptionObject(_capi.GB_ERR_BAD_ARG, "Fixed and moving images must be set.")
        if self._metric is None or self._optimizer is None or self._transform is None:
            raise ExceptionObject(_capi.GB_ERR_BAD_ARG, "Metric, optimizer and initial transform must be set.")
        for name, v in (("shrink factors", self._shrink), ("smoothing sigmas", self._sigmas)):
            if len(v) != self._levels:
                raise ExceptionObject(_capi.GB_ERR_BAD_ARG, f"The number of {name} does not match the number of "
                                                            f"levels.")
        if self._strategy != NONE and len(self._percentages) != self._levels:
            raise ExceptionObject(_capi.GB_ERR_BAD_ARG, "sampling percentages do not match the number of levels")

    def _compose(self):
        """Level 0's composite: [moving initial (unless absent), output transform]
        (itkImageRegistrationMethodv4.hxx:335-360); a linear output transform takes the
        centre of a linear moving initial transform (InitializeCenterOfLinearOutputTransform)."""
        if self._moving_initial is None:
            return self._transform
        if isinstance(self._transform, AffineTransform) and isinstance(self._moving_initial, AffineTransform):
            self._transform.SetCenter(self._moving_initial.GetCenter())
        c = CompositeTransform()
        c.AddTransform(self._moving_initial)
        c.AddTransform(self._transform)
        return c

    def Update(self):
        self._check()
        self._composite = self._compose()
        m, opt = self._metric, self._optimizer
        m.SetFixedImage(self._fixed)
        m.SetMovingImage(self._moving)
        m.SetMovingTransform(self._composite)
        seed = self._random_seed  # GenerateData: the same seed for every Update
        self._level_points = []
        for level in range(self._levels):
            self._current_level = level
            s = int(time.time_ns() & 0x7FFFFFFF) if self._reseed_from_clock else seed
            pts, seed = setup_level(m, self._fixed, self._shrink[level], self._sigmas[level], self._sigmas_physical,
                                    self._strategy, self._percentages[level] if self._strategy != NONE else 1.0, s)
            self._level_points.append(pts)
            opt.SetMetric(m)
            opt.StartOptimization()
        return self._transform
