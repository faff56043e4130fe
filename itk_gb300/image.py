"""``Image<float,3>``: a numpy volume plus the geometry ITK's ImageBase keeps.

Memory order is ITK's: the array has shape (nz, ny, nx), x fastest.  The
index-to-physical map is ``origin + direction @ diag(spacing) @ index``
(Core/Common/include/itkImageBase.h:594-604).
"""
from __future__ import annotations

import numpy as np


class Image:
    """Scalar 3-D image (``itk::Image<float,3>``) held on the host."""

    def __init__(self, array, spacing=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0), direction=None):
        a = np.asarray(array)
        if a.ndim != 3:
            raise ValueError("Image expects a (nz, ny, nx) array")
        self.array = np.ascontiguousarray(a, dtype=np.float32)
        self.spacing = np.asarray(spacing, dtype=np.float64).reshape(3)
        self.origin = np.asarray(origin, dtype=np.float64).reshape(3)
        self.direction = (np.eye(3) if direction is None else np.asarray(direction, dtype=np.float64)).reshape(3, 3)

    # ITK-style accessors
    def GetSpacing(self):
        return tuple(self.spacing)

    def GetOrigin(self):
        return tuple(self.origin)

    def GetDirection(self):
        return self.direction.copy()

    def GetSize(self):
        nz, ny, nx = self.array.shape
        return (nx, ny, nz)

    def GetBufferPointer(self):
        return self.array

    @property
    def size(self):
        return self.GetSize()

    def index_to_physical(self):
        return self.direction @ np.diag(self.spacing)

    def TransformIndexToPhysicalPoint(self, index):
        return self.origin + self.index_to_physical() @ np.asarray(index, dtype=np.float64)

    def TransformPhysicalPointToContinuousIndex(self, point):
        return np.linalg.solve(self.index_to_physical(), np.asarray(point, dtype=np.float64) - self.origin)

    def physical_center(self):
        return self.TransformIndexToPhysicalPoint((np.asarray(self.GetSize(), np.float64) - 1.0) / 2.0)

    def geometry_flat(self):
        """spacing(3) + origin(3) + direction(9), the oracle's flat geometry."""
        return np.concatenate([self.spacing, self.origin, self.direction.reshape(9)])


class GradientImage:
    """``Image<CovariantVector<double,3>,3>``: array of shape (nz, ny, nx, 3)."""

    def __init__(self, array):
        a = np.asarray(array, dtype=np.float64)
        if a.ndim != 4 or a.shape[3] != 3:
            raise ValueError("GradientImage expects a (nz, ny, nx, 3) array")
        self.array = np.ascontiguousarray(a)


class DisplacementFieldImage:
    """``Image<Vector<double,3>,3>``: a displacement per voxel, array of shape
    (nz, ny, nx, 3) with the geometry of a scalar image."""

    def __init__(self, array, spacing=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0), direction=None):
        a = np.asarray(array, dtype=np.float64)
        if a.ndim != 4 or a.shape[3] != 3:
            raise ValueError("DisplacementFieldImage expects a (nz, ny, nx, 3) array")
        self.array = np.ascontiguousarray(a)
        self.spacing = np.asarray(spacing, dtype=np.float64).reshape(3)
        self.origin = np.asarray(origin, dtype=np.float64).reshape(3)
        self.direction = (np.eye(3) if direction is None else np.asarray(direction, dtype=np.float64)).reshape(3, 3)

    @classmethod
    def like(cls, image, array=None):
        """A field on the grid of `image` (zero unless `array` is given)."""
        nx, ny, nz = image.GetSize()
        a = np.zeros((nz, ny, nx, 3)) if array is None else array
        return cls(a, image.spacing, image.origin, image.direction)

    def GetSize(self):
        nz, ny, nx, _ = self.array.shape
        return (nx, ny, nz)

    def GetSpacing(self):
        return tuple(self.spacing)

    def GetOrigin(self):
        return tuple(self.origin)

    def GetDirection(self):
        return self.direction.copy()
