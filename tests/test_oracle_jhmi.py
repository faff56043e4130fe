"""The oracle's JointHistogramMutualInformationImageToImageMetricv4 (no GPU).

Pinned by the reference test's own checks
(Registration/Metricsv4/test/itkJointHistogramMutualInformationImageToImageMetricv4Test.cxx:30-165)
on its images (a 20^3 blob plus ramps, moving = fixed^3, 20 bins, variance 1.5,
the default moving-gradient filter): GetValue equals GetValueAndDerivative's
value exactly; at a 1-voxel detune the analytic translation derivative points
downhill and lies within [0.7, 1.4] of the central difference (h = 0.5) of the
value; non-overlapping images give no valid point and the maximum value.  The
discrete Gaussian kernel is checked against scaled Bessel functions, the joint
PDF's mass and marginals against their definitions."""
import numpy as np
import pytest

from cases import geom, oracle_transform
from itk_gb300 import AffineTransform, Image
from oracle import oracle as O


def reference_images(n=20):
    k = np.arange(n, dtype=np.float64)
    Z, Y, X = np.meshgrid(k, k, k, indexing="ij")
    c = (n - 1) / 2.0
    r2 = sum(((a - c) / (n / 3.0)) ** 2 for a in (X, Y, Z))
    f = np.exp(-r2) + 0.3 * X / n + 0.15 * Y / n
    return Image(f.astype(np.float32)), Image((f ** 3).astype(np.float32))


def run(fixed, moving, T, grad, deriv=True, bins=20, variance=1.5, points=None):
    return O.joint_histogram_mi(fixed.array, geom(fixed), moving.array, geom(moving), oracle_transform(T), bins=bins,
                                variance=variance, moving_grad=grad, points=points, compute_derivative=deriv,
                                pixel_double=True)


@pytest.fixture(scope="module")
def case():
    fixed, moving = reference_images()
    grad = O.gradient_recursive_gaussian(moving.array, moving.spacing, moving.direction, 1.0)
    return fixed, moving, grad


def translation(dx):
    T = AffineTransform()
    T.SetTranslation([dx, 0.0, 0.0])
    return T


def test_value_paths_agree(case):
    fixed, moving, grad = case
    rc1, v1, _, n1, _ = run(fixed, moving, translation(0.0), grad, deriv=False)
    rc2, v2, _, n2, _ = run(fixed, moving, translation(0.0), grad, deriv=True)
    assert rc1 == rc2 == 0 and v1 == v2 and n1 == n2 == fixed.array.size
    assert v1 < 0  # metrics minimize: value = -MI (bits)


def test_derivative_matches_finite_difference(case):
    fixed, moving, grad = case
    _, _, d, _, _ = run(fixed, moving, translation(1.0), grad)
    vp = run(fixed, moving, translation(1.5), grad, deriv=False)[1]
    vm = run(fixed, moving, translation(0.5), grad, deriv=False)[1]
    fd = (vp - vm) / (2 * 0.5)
    analytic = d[9]
    assert abs(fd) > 1e-10 and analytic * fd < 0
    assert 0.7 * abs(fd) <= abs(analytic) <= 1.4 * abs(fd)
    # the reference test records the ratio it measures on these images: ~1.08 at h = 0.5
    assert 1.03 < abs(analytic) / abs(fd) < 1.13


def test_non_overlap(case):
    fixed, moving, grad = case
    T = translation(1000.0)
    T.SetTranslation([1000.0, 1000.0, 1000.0])
    rc, v, d, nv, _ = run(fixed, moving, T, grad)
    assert rc == 2 and nv == 0 and v == np.finfo(np.float64).max and not np.any(d)


def test_gaussian_kernel_is_the_discrete_gaussian():
    scipy_special = pytest.importorskip("scipy.special")
    for var in (0.5, 1.5, 4.0):
        c = O.gaussian_kernel(var)
        r = (len(c) - 1) // 2
        ex = np.array([scipy_special.ive(abs(k), var) for k in range(-r, r + 1)])
        np.testing.assert_allclose(c, ex / ex.sum(), rtol=1e-6)
        assert c.sum() == pytest.approx(1.0, abs=1e-14)
        # truncated where the two-sided mass first reaches 0.99
        full = ex / np.sum([scipy_special.ive(abs(k), var) for k in range(-60, 61)])
        assert full.sum() >= 0.99 - 1e-9 and full[1:-1].sum() < 0.99


def test_pdf_mass_and_smoothing(case):
    fixed, moving, grad = case
    _, _, _, _, raw = run(fixed, moving, translation(0.3), grad, deriv=False, variance=0.0)
    _, _, _, _, smooth = run(fixed, moving, translation(0.3), grad, deriv=False, variance=1.5)
    # the histogram is normalized; the zero-flux smoothing is not renormalized (mass
    # that reaches the border reads the edge bins again)
    assert raw.sum() == pytest.approx(1.0, abs=1e-12) and 0.95 < smooth.sum() <= 1.0 + 1e-12
    # counts only inside [2, bins - 3] on both axes (the padding); smoothing spreads them
    assert not raw[:2].any() and not raw[:, :2].any() and not raw[-2:].any() and not raw[:, -2:].any()
    assert smooth[1].any() and np.count_nonzero(smooth) > np.count_nonzero(raw)
