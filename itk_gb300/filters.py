"""Host-side mirror of the per-level image filters over the GB300 C ABI.

``SmoothingRecursiveGaussianImageFilter``, ``GradientRecursiveGaussianImageFilter``
and ``ShrinkImageFilter`` on ``Image<float,3>`` (Filtering/Smoothing,
Filtering/ImageGradient, Filtering/ImageGrid in ITK's Modules/), with ITK's
SetInput / Set... / Update / GetOutput pattern.  The recursive-Gaussian filters
run on the GPU (gb_smooth_recursive_gaussian_host,
gb_gradient_recursive_gaussian_host); the shrink filter's geometry comes from
gb_shrink_geometry and its pixels are a strided copy.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import check, f64, i64, ptr
from .image import GradientImage, Image
from .metrics import context


def _size(img: Image):
    return i64(img.GetSize())


class SmoothingRecursiveGaussianImageFilter:
    """Zero-order recursive Gaussian along z, x, y; sigma in physical units."""

    def __init__(self, device: int = 0):
        self._device = device
        self._sigma = np.ones(3)
        self._input = None
        self._output = None

    def SetSigma(self, sigma):
        self._sigma = np.full(3, float(sigma))

    def SetSigmaArray(self, sigma):
        self._sigma = f64(sigma).reshape(3).copy()

    def GetSigmaArray(self):
        return self._sigma.copy()

    def SetInput(self, image: Image):
        self._input = image

    def Update(self):
        img = self._input
        out = np.empty_like(img.array)
        L = _capi.lib()
        check(L.gb_smooth_recursive_gaussian_host(context(self._device), ptr(img.array), ptr(out), ptr(_size(img)),
                                                  ptr(f64(img.spacing)), ptr(f64(self._sigma))))
        self._output = Image(out, spacing=img.spacing, origin=img.origin, direction=img.direction)

    def GetOutput(self) -> Image:
        return self._output


class GradientRecursiveGaussianImageFilter:
    """Gradient by first-order recursive Gaussian along each axis (zero order along the
    others), divided by spacing, mapped by the image direction when UseImageDirection."""

    def __init__(self, device: int = 0):
        self._device = device
        self._sigma = 1.0
        self._normalize = False
        self._use_direction = True
        self._input = None
        self._output = None

    def SetSigma(self, sigma):
        self._sigma = float(sigma)

    def SetNormalizeAcrossScale(self, on):
        self._normalize = bool(on)

    def SetUseImageDirection(self, on):
        self._use_direction = bool(on)

    def SetInput(self, image: Image):
        self._input = image

    def Update(self):
        img = self._input
        out = np.empty(img.array.shape + (3,), np.float32)
        L = _capi.lib()
        check(L.gb_gradient_recursive_gaussian_host(context(self._device), ptr(img.array), ptr(out), ptr(_size(img)),
                                                    ptr(f64(img.spacing)), ptr(f64(img.direction.reshape(9))),
                                                    self._sigma, int(self._normalize), int(self._use_direction)))
        self._output = GradientImage(out.astype(np.float64))

    def GetOutput(self) -> GradientImage:
        return self._output


def shrink_geometry(image: Image, factors):
    """ShrinkImageFilter output (size xyz, spacing, origin) for the image's geometry."""
    osz = np.zeros(3, np.int64)
    osp = np.zeros(3, np.float64)
    oorg = np.zeros(3, np.float64)
    check(_capi.lib().gb_shrink_geometry(ptr(_size(image)), ptr(f64(image.spacing)), ptr(f64(image.origin)),
                                         ptr(f64(image.direction.reshape(9))), ptr(i64(factors)), ptr(osz),
                                         ptr(osp), ptr(oorg)))
    return osz, osp, oorg


class ShrinkImageFilter:
    """Subsampling by integer factors with the image centre kept in place
    (Filtering/ImageGrid/include/itkShrinkImageFilter.hxx:100-290)."""

    def __init__(self):
        self._factors = np.ones(3, np.int64)
        self._input = None
        self._output = None

    def SetShrinkFactors(self, factors):
        f = np.broadcast_to(np.asarray(factors, np.int64), (3,)).copy()
        self._factors = np.maximum(f, 1)

    def SetInput(self, image: Image):
        self._input = image

    def Update(self):
        img = self._input
        osz, osp, oorg = shrink_geometry(img, self._factors)
        out = Image(np.zeros((osz[2], osz[1], osz[0]), np.float32), spacing=osp, origin=oorg,
                    direction=img.direction)
        # input index of output index 0 (TransformPhysicalPointToIndex rounds half up), then a stride
        p0 = out.TransformIndexToPhysicalPoint((0, 0, 0))
        ci = img.TransformPhysicalPointToContinuousIndex(p0)
        off = np.maximum(np.floor(ci + 0.5).astype(np.int64), 0)
        f = self._factors
        out.array[...] = img.array[off[2]::f[2], off[1]::f[1], off[0]::f[0]][:osz[2], :osz[1], :osz[0]]
        self._output = out

    def GetOutput(self) -> Image:
        return self._output
