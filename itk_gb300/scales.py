"""``RegistrationParameterScalesFromPhysicalShift``: optimizer scales from the physical
shift that a small change of each parameter causes.

Restates Numerics/Optimizersv4/include/itkRegistrationParameterScalesFromShiftBase.hxx:31-213
and itkRegistrationParameterScalesFromPhysicalShift.hxx:27-90 with the sampling of
itkRegistrationParameterScalesEstimator.hxx:296-580: each parameter in turn is moved
by the small variation (0.01); its scale is the largest Euclidean shift of the
mapped sample points, squared and divided by the squared variation (a zero shift
takes the smallest nonzero shift squared); a B-spline takes the smallest nonzero
shift for every parameter.  Sample points: the 8 corners of the virtual domain for
an affine transform, the central region (radius 5 voxels) for transforms with
local support (B-spline, displacement field), or a given virtual-domain point set.
Host code: it runs once per level, on a handful of points.
"""
from __future__ import annotations

import numpy as np

from .transforms import TRANSFORM_BSPLINE, TRANSFORM_COMPOSITE, TRANSFORM_DISPLACEMENT_FIELD

CENTRAL_REGION_RADIUS = 5


class RegistrationParameterScalesFromPhysicalShift:
    def __init__(self):
        self._metric = None
        self._variation = 0.01
        self._points = None

    def SetMetric(self, metric):
        self._metric = metric

    def GetMetric(self):
        return self._metric

    def SetSmallParameterVariation(self, v: float):
        self._variation = float(v)

    def GetSmallParameterVariation(self):
        return self._variation

    def SetVirtualDomainPointSet(self, points):
        self._points = None if points is None else np.asarray(points, np.float64).reshape(-1, 3)

    # ---- the virtual domain and its samples
    def _virtual_grid(self):
        """(size xyz, spacing, origin, direction) of the metric's virtual domain at its level."""
        from .filters import shrink_geometry
        m = self._metric
        img = m._virtual if m._virtual is not None else m._fixed
        if img is None:
            raise ValueError("the metric has no virtual domain (set the fixed image)")
        size = np.asarray(img.GetSize(), np.int64)
        spacing, origin = np.asarray(img.spacing, np.float64), np.asarray(img.origin, np.float64)
        if m._virtual is None and tuple(m._level_shrink) != (1, 1, 1):
            size, spacing, origin = shrink_geometry(img, m._level_shrink)
        return size, spacing, origin, np.asarray(img.direction, np.float64).reshape(3, 3)

    def _local_support(self):
        return self._metric.GetMovingTransform().kind in (TRANSFORM_BSPLINE, TRANSFORM_COMPOSITE,
                                                            TRANSFORM_DISPLACEMENT_FIELD)

    def _sample_points(self, size, spacing, origin, direction):
        if self._points is not None:
            return self._points
        i2p = direction @ np.diag(spacing)
        if self._local_support():
            # SampleVirtualDomainWithCentralRegion: the voxels within the radius of the central
            # index (lower + upper) / 2 (itkRegistrationParameterScalesEstimator.hxx:429-478)
            c = (size - 1) // 2
            lo = np.maximum(c - CENTRAL_REGION_RADIUS, 0)
            hi = np.minimum(c + CENTRAL_REGION_RADIUS, size - 1)
            axes = [np.arange(lo[d], hi[d] + 1) for d in range(3)]
            kz, ky, kx = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
            idx = np.stack([kx.ravel(), ky.ravel(), kz.ravel()], 1).astype(np.float64)
        else:
            # SampleVirtualDomainWithCorners: the 2^3 corners, bit d selects the far end of axis d
            idx = np.array([[(i >> d) & 1 for d in range(3)] for i in range(8)], np.float64) * (size - 1)
        return idx @ i2p.T + origin

    def _max_shift(self, T, points, delta):
        """ComputeMaximumVoxelShift: the largest distance between the points mapped before
        and after UpdateTransformParameters(delta); the parameters are restored."""
        old = T.GetParameters().copy()
        y0 = T.TransformPoint(points)
        T.UpdateTransformParameters(delta)
        y1 = T.TransformPoint(points)
        T.SetParameters(old)
        return float(np.max(np.sqrt(np.sum((y1 - y0) ** 2, axis=1))))

    # ---- estimates
    def EstimateScales(self):
        m = self._metric
        if m is None:
            raise ValueError("the scales estimator has no metric")
        T = m.GetMovingTransform()
        size, spacing, origin, direction = self._virtual_grid()
        pts = self._sample_points(size, spacing, origin, direction)
        P = T.GetNumberOfParameters()
        field = T.kind == TRANSFORM_DISPLACEMENT_FIELD
        nlocal = 3 if field else P
        offset = 0
        if field:
            # the central voxel's parameters (ComputeParameterOffsetFromVirtualIndex)
            c = (size - 1) // 2
            offset = 3 * int(c[0] + size[0] * (c[1] + size[1] * c[2]))
        scales = np.zeros(nlocal)
        min_nonzero = np.finfo(np.float64).max
        eps = np.finfo(np.float64).eps
        for i in range(nlocal):
            delta = np.zeros(P)
            delta[offset + i] = self._variation
            s = self._max_shift(T, pts, delta)
            scales[i] = s
            if eps < s < min_nonzero:
                min_nonzero = s
        if min_nonzero == np.finfo(np.float64).max:
            return np.ones(nlocal)  # no parameter moves a point: the reference's default
        if T.kind in (TRANSFORM_BSPLINE, TRANSFORM_COMPOSITE):
            return np.full(nlocal, min_nonzero)
        scales = np.where(scales <= eps, min_nonzero * min_nonzero, scales * scales)
        return scales / (self._variation * self._variation)

    def EstimateStepScale(self, step):
        """The largest physical shift of the sample points for a step of the parameters
        (linearized by a step scaled to the small variation for global transforms)."""
        T = self._metric.GetMovingTransform()
        size, spacing, origin, direction = self._virtual_grid()
        step = np.asarray(step, np.float64)
        if self._local_support():
            i2p = direction @ np.diag(spacing)
            kz, ky, kx = np.meshgrid(*[np.arange(n) for n in size[::-1]], indexing="ij")
            pts = np.stack([kx.ravel(), ky.ravel(), kz.ravel()], 1) @ i2p.T + origin
            return self._max_shift(T, pts, step)
        pts = self._sample_points(size, spacing, origin, direction)
        max_step = float(np.max(np.abs(step))) if step.size else 0.0
        if max_step <= np.finfo(np.float64).eps:
            return 0.0
        factor = self._variation / max_step
        return self._max_shift(T, pts, step * factor) / factor
