"""The oracle's CorrelationImageToImageMetricv4, pinned by the properties the
reference's test and the metric's definition fix (no GPU needed): the toy images
of itkCorrelationImageToImageMetricv4Test.cxx, thread-count invariance to 1e-8
(the test's check), the non-overlapping case (value DBL_MAX, no valid point),
self-correlation -1 with a zero derivative, invariance under an increasing
affine intensity map, and the derivative against central finite differences
(the metric returns the descent direction, -dV/dp)."""
import sys

import numpy as np
import pytest

from cases import geom, oracle_transform
from itk_gb300 import AffineTransform, Image
from oracle import oracle as O


def toy(offset, n=20):
    idx = np.arange(n, dtype=np.float64)
    Z, Y, X = np.meshgrid(idx, idx, idx, indexing="ij")
    v = (X + offset[0]) ** 2 + (Y + offset[1]) ** 2 + (Z + offset[2]) ** 2
    return Image(np.exp(-v / 8.0).astype(np.float32))


def corr(fixed, moving, T, **kw):
    return O.correlation(fixed.array, geom(fixed), moving.array, geom(moving), oracle_transform(T), **kw)


@pytest.fixture(scope="module")
def toys():
    return toy((0.0, 0.0, 0.0)), toy((1.0, 0.5, 0.25))


def test_thread_invariance_and_finite(toys):
    f, m = toys
    T = AffineTransform()
    r1 = corr(f, m, T, nthreads=1)
    r8 = corr(f, m, T, nthreads=8)
    assert r1[0] == 0 and r1[3] == 20 ** 3
    assert abs(r1[1] - r8[1]) <= 1e-8 and np.linalg.norm(r1[2] - r8[2]) <= 1e-8
    assert -1.0 <= r1[1] < 0.0


def test_non_overlapping_images(toys):
    f, m = toys
    T = AffineTransform()
    T.SetTranslation([1000.0, 1000.0, 1000.0])
    rc, v, d, nv = corr(f, m, T)
    assert rc == 2 and nv == 0 and v == sys.float_info.max and np.all(d == 0)


def test_self_correlation(toys):
    f, _ = toys
    rc, v, d, nv = corr(f, f, AffineTransform())
    assert rc == 0 and v == -1.0 and np.all(d == 0)


def test_intensity_map_invariance(toys):
    f, m = toys
    T = AffineTransform()
    T.SetTranslation([0.3, -0.2, 0.1])
    m2 = Image(3.0 * m.array + 7.0)  # float32 voxels: the map itself rounds
    v1 = corr(f, m, T)[1]
    v2 = corr(f, m2, T)[1]
    assert abs(v1 - v2) <= 1e-5 * abs(v1)


def test_derivative_is_minus_finite_difference():
    # blobs inside the volume: the reference's gradient is zero on the buffer border,
    # where the toy images of the reference test keep their blob
    f, m = toy((-9.5, -9.5, -9.5)), toy((-8.5, -9.0, -9.25))
    T = AffineTransform()
    T.SetCenter([9.5, 9.5, 9.5])
    T.SetTranslation([0.3, -0.2, 0.1])
    p0 = T.GetParameters().copy()
    _, v0, d, _ = corr(f, m, T, pixel_double=True)
    h = 1e-5
    fd = np.zeros(12)
    for k in range(12):
        for sgn in (1, -1):
            p = p0.copy()
            p[k] += sgn * h
            T.SetParameters(p)
            fd[k] += sgn * corr(f, m, T, pixel_double=True)[1]
        fd[k] /= 2 * h
    T.SetParameters(p0)
    # translations: the central-difference gradient against the exact change of the
    # trilinear interpolant (matrix entries weight that gap by position; MeanSquares
    # shows the same)
    assert np.max(np.abs(d[9:] + fd[9:])) <= 0.02 * np.max(np.abs(fd[9:]))
