"""Moving transforms with ITK's parameter layouts.

* ``AffineTransform`` -- ``AffineTransform<double,3>``: 12 parameters (row-major
  matrix, then translation), fixed parameters = centre
  (Core/Transform/include/itkMatrixOffsetTransformBase.hxx:464-561, offset
  from ComputeOffset :612-631).
* ``BSplineTransform`` -- ``BSplineTransform<double,3,3>``: 3*prod(mesh+3)
  coefficients (dimension-major, x fastest), 18 fixed parameters: grid size,
  grid origin, grid spacing, grid direction
  (Core/Transform/include/itkBSplineTransform.hxx:243-330).
* ``DisplacementFieldTransform`` -- ``DisplacementFieldTransform<double,3>``:
  y = x + u(x), u linearly interpolated from a vector field and zero outside
  its buffer; the parameters are the field itself (3 per voxel), 18 fixed
  parameters: field size, origin, spacing, direction
  (Filtering/DisplacementField/include/itkDisplacementFieldTransform.hxx:67-100,520-570).
* ``CompositeTransform`` -- queue applied in reverse
  (Core/Transform/include/itkCompositeTransform.hxx:60-70), the most recently
  added transform optimized; supported queues: [T], [affine, B-spline] and
  [affine, displacement field].
"""
from __future__ import annotations

import numpy as np

from . import _capi
from .image import DisplacementFieldImage

TRANSFORM_AFFINE = _capi.GB_TRANSFORM_AFFINE
TRANSFORM_BSPLINE = _capi.GB_TRANSFORM_BSPLINE
TRANSFORM_COMPOSITE = _capi.GB_TRANSFORM_COMPOSITE
TRANSFORM_DISPLACEMENT_FIELD = _capi.GB_TRANSFORM_DISPLACEMENT_FIELD


class AffineTransform:
    kind = TRANSFORM_AFFINE

    def __init__(self):
        self.matrix = np.eye(3)
        self.translation = np.zeros(3)
        self.center = np.zeros(3)

    def SetIdentity(self):
        self.matrix = np.eye(3)
        self.translation = np.zeros(3)

    def SetCenter(self, c):
        self.center = np.asarray(c, dtype=np.float64).reshape(3).copy()

    def GetCenter(self):
        return self.center.copy()

    def SetMatrix(self, m):
        self.matrix = np.asarray(m, dtype=np.float64).reshape(3, 3).copy()

    def GetMatrix(self):
        return self.matrix.copy()

    def SetTranslation(self, t):
        self.translation = np.asarray(t, dtype=np.float64).reshape(3).copy()

    def GetTranslation(self):
        return self.translation.copy()

    def GetOffset(self):
        # ComputeOffset: offset = t + c - M c (itkMatrixOffsetTransformBase.hxx:612-631)
        return self.translation + self.center - self.matrix @ self.center

    def GetNumberOfParameters(self):
        return 12

    def GetParameters(self):
        return np.concatenate([self.matrix.reshape(9), self.translation])

    def SetParameters(self, p):
        p = np.asarray(p, dtype=np.float64).reshape(12)
        self.matrix = p[:9].reshape(3, 3).copy()
        self.translation = p[9:].copy()

    def GetFixedParameters(self):
        return self.center.copy()

    def SetFixedParameters(self, f):
        self.SetCenter(f)

    def UpdateTransformParameters(self, update, factor=1.0):
        self.SetParameters(self.GetParameters() + np.asarray(update, np.float64) * factor)

    def TransformPoint(self, x):
        x = np.asarray(x, dtype=np.float64)
        return x @ self.matrix.T + self.GetOffset()

    def flat(self):
        return self.kind, self.GetParameters(), self.GetFixedParameters()


class BSplineTransform:
    """Cubic (order 3) B-spline free-form deformation."""

    kind = TRANSFORM_BSPLINE
    order = 3

    def __init__(self):
        self.fixed = np.zeros(18)
        self.fixed[:3] = 4
        self.fixed[6:9] = 1.0
        self.fixed[9:] = np.eye(3).reshape(9)
        self.params = np.zeros(3 * 64)

    # --- domain, as SetFixedParametersFromTransformDomainInformation (.hxx:285-330)
    def SetTransformDomain(self, origin, physical_dimensions, mesh_size, direction=None):
        origin = np.asarray(origin, np.float64).reshape(3)
        phys = np.asarray(physical_dimensions, np.float64).reshape(3)
        mesh = np.asarray(mesh_size, np.int64).reshape(3)
        d = np.eye(3) if direction is None else np.asarray(direction, np.float64).reshape(3, 3)
        spacing = phys / mesh
        go = d @ (-0.5 * spacing * (self.order - 1)) + origin
        self.fixed = np.concatenate([(mesh + self.order).astype(np.float64), go, spacing, d.reshape(9)])
        self.params = np.zeros(3 * int(np.prod(mesh + self.order)))

    def GetTransformDomainMeshSize(self):
        return (self.fixed[:3] - self.order).astype(np.int64)

    def grid_size(self):
        return self.fixed[:3].astype(np.int64)

    def GetNumberOfParametersPerDimension(self):
        return int(np.prod(self.grid_size()))

    def GetNumberOfParameters(self):
        return 3 * self.GetNumberOfParametersPerDimension()

    def GetParameters(self):
        return self.params.copy()

    def SetParameters(self, p):
        p = np.asarray(p, dtype=np.float64).reshape(-1)
        if p.size != self.GetNumberOfParameters():
            raise ValueError("B-spline parameter count must be 3 * grid nodes")
        self.params = p.copy()

    def GetFixedParameters(self):
        return self.fixed.copy()

    def SetFixedParameters(self, f):
        f = np.asarray(f, dtype=np.float64).reshape(18)
        self.fixed = f.copy()
        if self.params.size != self.GetNumberOfParameters():
            self.params = np.zeros(self.GetNumberOfParameters())

    def UpdateTransformParameters(self, update, factor=1.0):
        self.SetParameters(self.params + np.asarray(update, np.float64) * factor)

    def coefficient_images(self):
        g = self.grid_size()
        return self.params.reshape(3, g[2], g[1], g[0])

    def TransformPoint(self, x):
        """Vectorized BSplineTransform::TransformPoint (itkBSplineTransform.hxx:510-591)."""
        x = np.atleast_2d(np.asarray(x, dtype=np.float64))
        g = self.grid_size()
        go, gs, gd = self.fixed[3:6], self.fixed[6:9], self.fixed[9:18].reshape(3, 3)
        p2i = np.linalg.inv(gd @ np.diag(gs))
        ci = (x - go) @ p2i.T
        lo, hi = 1.0, g.astype(np.float64) - 2.0
        inside = np.all((ci >= lo) & (ci < hi), axis=1)
        start = np.floor(ci - 1.0).astype(np.int64)
        u = ci - start
        w1 = [np.stack([_bspline3(u[:, j] - k) for k in range(4)], axis=1) for j in range(3)]
        coeff = np.ascontiguousarray(self.params.reshape(3, -1).T)  # (nodes, 3)
        out = x.copy()
        disp = np.zeros_like(x)
        st = np.where(inside[:, None], start, 1)
        base = st[:, 0] + g[0] * (st[:, 1] + g[1] * st[:, 2])
        k4 = np.arange(4)
        for iz in range(4):
            for iy in range(4):
                # the 4 x-consecutive nodes of one (y, z) row in one gather: (n, 4, 3)
                row = coeff[(base + g[0] * (iy + g[1] * iz))[:, None] + k4]
                disp += (w1[1][:, iy] * w1[2][:, iz])[:, None] * np.einsum("nk,nkc->nc", w1[0], row)
        out[inside] += disp[inside]
        return out

    def flat(self):
        return self.kind, self.GetParameters(), self.GetFixedParameters()


def _bspline3(u):
    a = np.abs(u)
    s = a * a
    return np.where(a < 1.0, (4.0 - 6.0 * s + 3.0 * s * a) / 6.0,
                    np.where(a < 2.0, (8.0 - 12.0 * a + 6.0 * s - s * a) / 6.0, 0.0))


class DisplacementFieldTransform:
    """Dense displacement field; local support (3 parameters per voxel)."""

    kind = TRANSFORM_DISPLACEMENT_FIELD

    def __init__(self):
        self.field = None

    def SetDisplacementField(self, field: DisplacementFieldImage):
        """The transform keeps the field: its parameters are the field's buffer."""
        if not isinstance(field, DisplacementFieldImage):
            raise TypeError("SetDisplacementField expects a DisplacementFieldImage")
        self.field = field

    def GetDisplacementField(self) -> DisplacementFieldImage:
        return self.field

    def _need_field(self):
        if self.field is None:
            raise ValueError("No displacement field is specified.")

    def GetNumberOfLocalParameters(self):
        return 3

    def GetNumberOfParameters(self):
        return 0 if self.field is None else self.field.array.size

    def GetParameters(self):
        self._need_field()
        return self.field.array.reshape(-1).copy()

    def parameters_view(self):
        """The field's buffer as the flat parameter array, without a copy."""
        self._need_field()
        return self.field.array.reshape(-1)

    def SetParameters(self, p):
        self._need_field()
        p = np.asarray(p, dtype=np.float64).reshape(-1)
        if p.size != self.field.array.size:
            raise ValueError("displacement field parameter count must be 3 * field voxels")
        self.field.array[...] = p.reshape(self.field.array.shape)

    def GetFixedParameters(self):
        self._need_field()
        f = self.field
        return np.concatenate([np.asarray(f.GetSize(), np.float64), f.origin, f.spacing, f.direction.reshape(9)])

    def SetFixedParameters(self, fp):
        """A zero field of the described grid (SetDisplacementFieldFromFixedParameters)."""
        fp = np.asarray(fp, dtype=np.float64).reshape(18)
        nx, ny, nz = (int(v) for v in fp[:3])
        self.field = DisplacementFieldImage(np.zeros((nz, ny, nx, 3)), fp[6:9], fp[3:6], fp[9:18].reshape(3, 3))

    def UpdateTransformParameters(self, update, factor=1.0):
        self.SetParameters(self.GetParameters() + np.asarray(update, np.float64) * factor)

    def TransformPoint(self, x):
        """x + u(x) inside the field's buffer (VectorLinearInterpolateImageFunction:
        neighbours of floor(cindex) clamped to the buffer), x outside it."""
        self._need_field()
        x = np.atleast_2d(np.asarray(x, dtype=np.float64))
        f = self.field
        n = np.asarray(f.GetSize(), np.int64)
        ci = (x - f.origin) @ np.linalg.inv(f.direction @ np.diag(f.spacing)).T
        inside = np.all((ci >= -0.5) & (ci < n - 0.5), axis=1)
        base = np.floor(ci).astype(np.int64)
        dist = ci - base
        u = np.zeros_like(x)
        for corner in range(8):
            w = np.ones(len(x))
            idx = np.empty_like(base)
            for d in range(3):
                if (corner >> d) & 1:
                    idx[:, d] = np.minimum(base[:, d] + 1, n[d] - 1)
                    w = w * dist[:, d]
                else:
                    idx[:, d] = np.maximum(base[:, d], 0)
                    w = w * (1.0 - dist[:, d])
            idx = np.clip(idx, 0, n - 1)
            u += w[:, None] * f.array[idx[:, 2], idx[:, 1], idx[:, 0]]
        out = x.copy()
        out[inside] += u[inside]
        return out

    def flat(self):
        return self.kind, self.GetParameters(), self.GetFixedParameters()


class CompositeTransform:
    """Queue of transforms applied last-added first; the last one is optimized."""

    def __init__(self):
        self.queue = []

    def AddTransform(self, t):
        self.queue.append(t)

    def GetNumberOfTransforms(self):
        return len(self.queue)

    def GetNthTransform(self, n):
        return self.queue[n]

    @property
    def active(self):
        return self.queue[-1]

    @property
    def kind(self):
        if len(self.queue) == 1:
            return self.queue[0].kind
        if len(self.queue) == 2 and isinstance(self.queue[0], AffineTransform) and \
                isinstance(self.queue[1], BSplineTransform):
            return TRANSFORM_COMPOSITE
        if len(self.queue) == 2 and isinstance(self.queue[0], AffineTransform) and \
                isinstance(self.queue[1], DisplacementFieldTransform):
            return TRANSFORM_DISPLACEMENT_FIELD  # the field's flat form with the initial affine appended
        raise ValueError("supported composite queues: [T], [AffineTransform, BSplineTransform] or "
                         "[AffineTransform, DisplacementFieldTransform]")

    def GetNumberOfParameters(self):
        return self.active.GetNumberOfParameters()

    def GetParameters(self):
        return self.active.GetParameters()

    @property
    def parameters_view(self):
        return getattr(self.active, "parameters_view", None)

    def SetParameters(self, p):
        self.active.SetParameters(p)

    def UpdateTransformParameters(self, update, factor=1.0):
        self.active.UpdateTransformParameters(update, factor)

    def TransformPoint(self, x):
        y = np.asarray(x, dtype=np.float64)
        for t in reversed(self.queue):
            y = t.TransformPoint(y)
        return y

    def GetFixedParameters(self):
        if self.kind == TRANSFORM_COMPOSITE or len(self.queue) == 2:
            a, b = self.queue
            return np.concatenate([b.GetFixedParameters(), a.GetParameters(), a.GetFixedParameters()])
        return self.active.GetFixedParameters()

    def flat(self):
        return self.kind, self.GetParameters(), self.GetFixedParameters()
