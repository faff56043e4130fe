"""GPU metric vs the FP64 oracle on identical inputs: BSplineTransform (order 3)
and the [affine, B-spline] CompositeTransform (B-spline optimized).

Same contract as the affine tests: value within 1e-5 relative, derivative
within 1e-4 of its largest-magnitude component (all 3 * nodes entries),
GetValue equal to GetValueAndDerivative's value.
"""
import numpy as np
import pytest

from cases import perturbed, run_oracle
from conftest import MATTES_VALUE_ATOL, assert_deriv_close, assert_value_close
from itk_gb300 import (BSplineTransform, CompositeTransform, MattesMutualInformationImageToImageMetricv4,
                       MeanSquaresImageToImageMetricv4, data)

pytestmark = pytest.mark.gpu


def make_metric(kind, fixed, moving, transform, gradient=None, points=None, bins=50):
    m = MeanSquaresImageToImageMetricv4() if kind == "msq" else MattesMutualInformationImageToImageMetricv4()
    m.SetFixedImage(fixed)
    m.SetMovingImage(moving)
    m.SetMovingTransform(transform)
    if gradient is not None:
        m.SetMovingImageGradientImage(gradient)
    else:
        m.SetUseMovingImageGradientFilter(False)
    if kind == "mattes":
        m.SetNumberOfHistogramBins(bins)
    if points is not None:
        m.SetVirtualSampledPointSet(points)
        m.SetUseSampledPointSet(True)
    m.Initialize()
    return m


def check(kind, fixed, moving, transform, gradient=None, points=None, bins=50, nvalid_slack=0):
    m = make_metric(kind, fixed, moving, transform, gradient, points, bins)
    v, d = m.GetValueAndDerivative()
    r = run_oracle(kind, fixed, moving, transform, gradient=gradient, points=points, bins=bins)
    assert r["status"] == 0
    assert abs(m.GetNumberOfValidPoints() - r["nvalid"]) <= nvalid_slack
    assert d.shape == r["derivative"].shape
    assert_value_close(v, r["value"], atol=MATTES_VALUE_ATOL if kind == "mattes" else 0.0)
    assert_deriv_close(d, r["derivative"])
    assert m.GetValue() == v
    return m, v, d, r


def composite(A, B):
    C = CompositeTransform()
    C.AddTransform(A)
    C.AddTransform(B)
    return C


@pytest.fixture(scope="module")
def bpair():
    fixed, moving, A, B = data.pair_bspline((40, 36, 32), (4, 4, 4), instance=0, multimodal_map=False)
    return fixed, moving, A, B, data.gradient_image(moving)


@pytest.fixture(scope="module")
def bpair_mm():
    fixed, moving, A, B = data.pair_bspline((44, 40, 36), (4, 4, 4), instance=1, multimodal_map=True)
    return fixed, moving, A, B, data.gradient_image(moving)


def bspline_with(fixed, mesh, seed, max_disp=2.0):
    return data.random_bspline_coefficients(data.bspline_over_image(fixed, mesh), seed, max_disp)


@pytest.mark.parametrize("gradient_image", [True, False])
@pytest.mark.parametrize("seed", [0, 1])
def test_mean_squares_bspline_dense(bpair, seed, gradient_image):
    fixed, moving, A, B, grad = bpair
    T = bspline_with(fixed, (4, 4, 4), 10 + seed)
    check("msq", fixed, moving, T, grad if gradient_image else None)


def test_mean_squares_bspline_sparse(bpair):
    fixed, moving, A, B, grad = bpair
    T = bspline_with(fixed, (5, 3, 4), 20)
    pts = data.random_points(fixed, 0.2, seed=21)
    check("msq", fixed, moving, T, grad, points=pts)


@pytest.mark.parametrize("gradient_image", [True, False])
def test_mean_squares_composite(bpair, gradient_image):
    fixed, moving, A, B, grad = bpair
    T = composite(perturbed(A, 30, scale=0.01, trans=0.5), bspline_with(fixed, (4, 4, 4), 31, 1.0))
    check("msq", fixed, moving, T, grad if gradient_image else None)


@pytest.mark.parametrize("gradient_image", [True, False])
def test_mattes_bspline_dense(bpair_mm, gradient_image):
    fixed, moving, A, B, grad = bpair_mm
    T = bspline_with(fixed, (4, 4, 4), 40)
    check("mattes", fixed, moving, T, grad if gradient_image else None)


@pytest.mark.parametrize("bins", [20, 50])
def test_mattes_composite_sparse(bpair_mm, bins):
    fixed, moving, A, B, grad = bpair_mm
    T = composite(A, bspline_with(fixed, (4, 4, 4), 41, 1.5))
    pts = data.random_points(fixed, 0.25, seed=42)
    check("mattes", fixed, moving, T, grad, points=pts, bins=bins)


def test_mattes_composite_generating_and_zero(bpair_mm):
    """The generating [affine, B-spline] and the same affine with a zero B-spline (the
    start of a B-spline stage initialised from an affine stage)."""
    fixed, moving, A, B, grad = bpair_mm
    Bc = BSplineTransform()
    Bc.SetFixedParameters(B.GetFixedParameters())
    Bc.SetParameters(B.GetParameters())
    check("mattes", fixed, moving, composite(A, Bc), grad)
    Bz = BSplineTransform()
    Bz.SetFixedParameters(B.GetFixedParameters())
    check("mattes", fixed, moving, composite(A, Bz), grad)


def test_partial_domain_and_rotated_grid(bpair):
    """B-spline domain covering part of the image with a rotated grid: samples outside
    the valid region map by the identity and carry no Jacobian."""
    fixed, moving, A, B, grad = bpair
    th = np.deg2rad(20.0)
    R = np.array([[np.cos(th), -np.sin(th), 0.0], [np.sin(th), np.cos(th), 0.0], [0.0, 0.0, 1.0]])
    T = BSplineTransform()
    T.SetTransformDomain(fixed.origin + np.array([6.0, 4.0, 3.0]), np.array([24.0, 22.0, 20.0]), (3, 4, 3), R)
    data.random_bspline_coefficients(T, 50, 2.0)
    check("msq", fixed, moving, T, grad)
    check("mattes", fixed, moving, T, grad, bins=30)


def test_large_grid_nodes_in_global_memory(bpair_mm):
    """A control grid too large for shared-memory staging (28^3 nodes) takes the global-memory path."""
    fixed, moving, A, B, grad = bpair_mm
    T = bspline_with(fixed, (25, 25, 25), 60, 1.0)
    assert T.GetNumberOfParameters() == 3 * 28 ** 3
    check("msq", fixed, moving, T, grad)
    check("mattes", fixed, moving, T, grad, bins=12)


def test_zero_bspline_matches_affine(bpair):
    """[A, zero B-spline] evaluates like A alone (B-spline kernels vs affine kernels)."""
    fixed, moving, A, B, grad = bpair
    # a domain 1 mm wider than the image on every side: every sample inside the valid region
    Bz = BSplineTransform()
    size = np.asarray(fixed.GetSize(), np.float64)
    Bz.SetTransformDomain(fixed.origin - 1.0, fixed.spacing * (size - 1.0) + 2.0, (4, 4, 4))
    for kind in ("msq", "mattes"):
        mc = make_metric(kind, fixed, moving, composite(A, Bz), grad)
        ma = make_metric(kind, fixed, moving, A, grad)
        vc, dc = mc.GetValueAndDerivative()
        va, da = ma.GetValueAndDerivative()
        assert mc.GetNumberOfValidPoints() == ma.GetNumberOfValidPoints()
        assert_value_close(vc, va, rtol=1e-6, atol=MATTES_VALUE_ATOL if kind == "mattes" else 0.0)
        # partition of unity: the node derivatives of one dimension sum to M^T (translation derivative)
        nper = Bz.GetNumberOfParametersPerDimension()
        sums = dc.reshape(3, nper).sum(axis=1)
        want = A.GetMatrix().T @ da[9:12]
        assert np.max(np.abs(sums - want)) <= 1e-4 * np.max(np.abs(want))


def test_repeatable_and_updates(bpair_mm):
    fixed, moving, A, B, grad = bpair_mm
    T = composite(A, bspline_with(fixed, (4, 4, 4), 70, 1.0))
    m = make_metric("mattes", fixed, moving, T, grad)
    v1, d1 = m.GetValueAndDerivative()
    v2, d2 = m.GetValueAndDerivative()
    assert v1 == v2 and np.array_equal(d1, d2)
    step = -0.5 * d1 / np.max(np.abs(d1))
    m.UpdateTransformParameters(step)  # updates T, the metric's moving transform
    v3, d3 = m.GetValueAndDerivative()
    assert v3 != v1
    r = run_oracle("mattes", fixed, moving, T, gradient=grad)
    assert_value_close(v3, r["value"], atol=MATTES_VALUE_ATOL)
    assert_deriv_close(d3, r["derivative"])
