"""Pins of the oracle's per-level image filters (test infrastructure).

Restated from the reference's filter tests (paths relative to ITK's Modules/):
  Filtering/Smoothing/test/itkRecursiveGaussianImageFilterTest.cxx:160-380
    - 1-D impulse of 1000 at the centre of 21 samples: the zero-order response
      sums to 1000 within 1e-3 (sigma 2); normalizing across scale leaves the
      zero order unchanged (1e-4);
    - the first derivative at centre - 2 lies between the finite differences of
      the zero-order response, the second derivative between those of the first
      (sigma 3);
  Filtering/ImageGradient/test/itkGradientRecursiveGaussianFilterTest.cxx:36-185
    - an 8^3 image with a 4^3 box of 100: with direction -I the physical gradient
      is the mirrored, negated gradient of the identity-direction image;
  Filtering/ImageGrid/include/itkShrinkImageFilter.hxx:230-290
    - shrink geometry keeps the image centre fixed.
"""
import numpy as np
import pytest

from oracle import oracle as O


def impulse(n=21, value=1000.0):
    x = np.zeros(n)
    x[(n - 1) // 2] = value
    return x


def test_impulse_normalization():
    x = impulse()
    y = O.rg_filter_line(x, 2.0, order=0, normalize_across_scale=True)
    total = np.sum(np.sort(y.astype(np.float32).astype(np.float64)))
    assert abs(total - 1000.0) / 1000.0 <= 1e-3
    y2 = O.rg_filter_line(x, 2.0, order=0, normalize_across_scale=False)
    assert abs(np.float32(y2[10]) - np.float32(y[10])) <= 1e-4


def test_derivative_bounds():
    x = impulse()
    c = 10
    z = O.rg_filter_line(x, 3.0, order=0).astype(np.float32)
    a, b, cc = float(z[c]), float(z[c - 2]), float(z[c - 4])
    d1 = O.rg_filter_line(x, 3.0, order=1).astype(np.float32)
    assert (a - b) / 2.0 <= d1[c - 2] <= (b - cc) / 2.0
    a1, b1, c1 = float(d1[c]), float(d1[c - 2]), float(d1[c - 4])
    d2 = O.rg_filter_line(x, 3.0, order=2).astype(np.float32)
    assert (a1 - b1) / 2.0 <= d2[c - 2] <= (b1 - c1) / 2.0


def test_gradient_flipped_direction():
    img = np.zeros((8, 8, 8), np.float32)
    img[2:6, 2:6, 2:6] = 100.0
    sp = (1.0, 1.0, 1.0)
    g = O.gradient_recursive_gaussian(img, sp, np.eye(3), 2.5, normalize_across_scale=False,
                                      use_image_direction=False)
    # the second filter keeps the defaults: no normalization across scale, image direction used
    gf = O.gradient_recursive_gaussian(img, sp, -np.eye(3), 2.5, normalize_across_scale=False)
    mirrored = g[::-1, ::-1, ::-1]
    assert np.max(np.abs(gf - mirrored)) <= 1e-12 * np.max(np.abs(g))
    assert np.max(np.abs(g)) > 1.0


def test_smoothing_keeps_constants_and_mass():
    const = np.full((6, 7, 8), 3.5, np.float32)
    s = O.smooth_recursive_gaussian(const, (1.0, 1.5, 2.0), 2.0)
    assert np.max(np.abs(s - 3.5)) <= 1e-5
    rng = np.random.default_rng(1)
    img = rng.normal(size=(20, 24, 28)).astype(np.float32)
    s = O.smooth_recursive_gaussian(img, (1.0, 1.0, 1.0), 1.0)
    assert s.std() < 0.5 * img.std()


def test_gradient_of_linear_ramp():
    nz, ny, nx = 34, 30, 32
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    sp = np.array([1.0, 1.5, 0.75])  # sigma = 1.5 mm: 1, 1.5 and 2 voxels; 12 voxels of margin below
    img = (0.5 * x * sp[0] - 1.25 * y * sp[1] + 2.0 * z * sp[2]).astype(np.float32)
    slope = np.array([0.5, -1.25, 2.0])
    sigma = float(sp.max())
    # without normalization across scale: the physical slope (to the recursive
    # approximation's ~1e-3); with it (the metric's default gradient filter) the
    # first-order response is scaled by sigma, itkRecursiveGaussianImageFilter.hxx:104-108
    for normalize, scale in ((False, 1.0), (True, sigma)):
        g = O.gradient_recursive_gaussian(img, sp, np.eye(3), sigma, normalize_across_scale=normalize)
        inner = g[12:-12, 12:-12, 12:-12]
        for d in range(3):
            assert np.allclose(inner[..., d], slope[d] * scale, rtol=2e-3), (normalize, d)


def test_shrink_geometry_keeps_centre():
    size, osp, org = O.shrink_geometry((256, 256, 200), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), np.eye(3), (4, 4, 4))
    assert tuple(size) == (64, 64, 50)
    assert np.allclose(osp, 4.0)
    assert np.allclose(org, 1.5)
    size, osp, org = O.shrink_geometry((7, 9, 10), (0.5, 1.0, 2.0), (1.0, -2.0, 3.0), np.eye(3), (2, 2, 3))
    assert tuple(size) == (3, 4, 3)
    in_centre = np.array([1.0, -2.0, 3.0]) + np.array([0.5, 1.0, 2.0]) * (np.array([7, 9, 10]) - 1) / 2.0
    out_centre = org + osp * (size - 1) / 2.0
    assert np.allclose(in_centre, out_centre)


def test_filters_reject_short_axes():
    with pytest.raises(ValueError):
        O.smooth_recursive_gaussian(np.zeros((3, 8, 8), np.float32), (1, 1, 1), 1.0)
