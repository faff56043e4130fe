"""JointHistogramMutualInformationImageToImageMetricv4 on the GPU against the FP64
oracle (value within 1e-5 relative, derivative within 1e-4 of its largest
component; dense and sampled; gradient image, central difference and the
default gradient filter; smoothing on and off), the smoothed joint PDF, and the
reference test's own checks on its images (value paths identical, the analytic
derivative against a central difference of the value, non-overlap)."""
import sys
import warnings

import numpy as np
import pytest

from cases import geom, oracle_transform, perturbed, small_pair
from conftest import assert_deriv_close, assert_value_close
from itk_gb300 import (AffineTransform, Image, JointHistogramMutualInformationImageToImageMetricv4,
                       RegularStepGradientDescentOptimizerv4, data)
from oracle import oracle as O
from oracle import registration as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pair():
    return small_pair((40, 36, 32), config=1, multimodal=True)


def make(fixed, moving, T, gradient="image", points=None, bins=20, variance=1.5):
    m = JointHistogramMutualInformationImageToImageMetricv4()
    m.SetNumberOfHistogramBins(bins)
    m.SetVarianceForJointPDFSmoothing(variance)
    m.SetFixedImage(fixed)
    m.SetMovingImage(moving)
    m.SetMovingTransform(T)
    if gradient == "image":
        m.SetMovingImageGradientImage(data.gradient_image(moving))
    elif gradient == "cd":
        m.SetUseMovingImageGradientFilter(False)
    if points is not None:
        m.SetVirtualSampledPointSet(points)
        m.SetUseSampledPointSet(True)
    m.Initialize()
    return m


def oracle(fixed, moving, T, gradient="image", points=None, bins=20, variance=1.5, deriv=True, pixel_double=False):
    if gradient == "image":
        g = data.gradient_image(moving).array
    elif gradient == "filter":
        g = O.gradient_recursive_gaussian(moving.array, moving.spacing, moving.direction, float(max(moving.spacing)))
    else:
        g = None
    return O.joint_histogram_mi(fixed.array, geom(fixed), moving.array, geom(moving), oracle_transform(T), bins=bins,
                                variance=variance, moving_grad=g, points=points, compute_derivative=deriv,
                                pixel_double=pixel_double)


@pytest.mark.parametrize("gradient", ["image", "cd", "filter"])
@pytest.mark.parametrize("sampled", [False, True])
@pytest.mark.parametrize("bins,variance", [(20, 1.5), (32, 0.0), (48, 2.5)])
def test_matches_oracle(pair, gradient, sampled, bins, variance):
    fixed, moving, T = pair
    U = perturbed(T, bins)
    pts = data.random_points(fixed, 0.3, seed=bins) if sampled else None
    m = make(fixed, moving, U, gradient, pts, bins, variance)
    v, d = m.GetValueAndDerivative()
    rc, rv, rd, nv, pdf = oracle(fixed, moving, U, gradient, pts, bins, variance)
    assert rc == 0 and m.GetNumberOfValidPoints() == nv
    assert_value_close(v, rv)
    assert_deriv_close(d, rd)
    np.testing.assert_allclose(m.GetJointPDF(), pdf, rtol=0, atol=1e-12 * pdf.max())
    assert m.GetValue() == v


def reference_images(n=20):
    k = np.arange(n, dtype=np.float64)
    Z, Y, X = np.meshgrid(k, k, k, indexing="ij")
    c = (n - 1) / 2.0
    r2 = sum(((a - c) / (n / 3.0)) ** 2 for a in (X, Y, Z))
    f = np.exp(-r2) + 0.3 * X / n + 0.15 * Y / n
    return Image(f.astype(np.float32)), Image((f ** 3).astype(np.float32))


def translation(dx, dy=0.0, dz=0.0):
    T = AffineTransform()
    T.SetTranslation([dx, dy, dz])
    return T


def test_reference_checks():
    """itkJointHistogramMutualInformationImageToImageMetricv4Test.cxx:30-165, on the GPU
    with the default gradient filter."""
    fixed, moving = reference_images()
    T = translation(0.0)
    m = make(fixed, moving, T, gradient="filter")
    v1 = m.GetValue()
    v2, _ = m.GetValueAndDerivative()
    assert v1 == v2
    T.SetTranslation([1.0, 0.0, 0.0])
    _, d = m.GetValueAndDerivative()
    T.SetTranslation([1.5, 0.0, 0.0])
    vp = m.GetValue()
    T.SetTranslation([0.5, 0.0, 0.0])
    vm = m.GetValue()
    fd = (vp - vm) / (2 * 0.5)
    assert abs(fd) > 1e-10 and d[9] * fd < 0
    assert 0.7 * abs(fd) <= abs(d[9]) <= 1.4 * abs(fd)
    assert 1.03 < abs(d[9]) / abs(fd) < 1.13  # the reference test measures ~1.08
    T.SetTranslation([1000.0, 1000.0, 1000.0])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        v, d = m.GetValueAndDerivative()
    assert m.GetNumberOfValidPoints() == 0 and v == sys.float_info.max and not np.any(d)


def test_device_resident_equals_host_call(pair):
    import torch
    fixed, moving, T = pair
    U = perturbed(T, 3)
    m = make(fixed, moving, U)
    v, d = m.GetValueAndDerivative()
    dp = torch.tensor(U.GetParameters(), dtype=torch.float64, device="cuda")
    out = torch.zeros(14, dtype=torch.float64, device="cuda")
    m.evaluate_device(dp.data_ptr(), out.data_ptr(), True)
    assert m.synchronize() == 0
    o = out.cpu().numpy()
    assert o[0] == v and np.array_equal(o[2:], d)


def test_device_optimizer_matches_host_loop(pair):
    fixed, moving, T = pair
    U = perturbed(T, 6, scale=0.02, trans=1.5)
    p0 = U.GetParameters().copy()
    scales = np.array([1.0] * 9 + [1.0 / 50.0] * 3)
    m = make(fixed, moving, U)

    def evaluate(p):
        U.SetParameters(p)
        v, d = m.GetValueAndDerivative()
        return 0, v, d

    h = R.regular_step(evaluate, p0, learning_rate=0.5, minimum_step_length=1e-3, number_of_iterations=20,
                       scales=scales, mean_squares=True)
    U.SetParameters(p0)
    o = RegularStepGradientDescentOptimizerv4()
    o.SetMetric(m)
    o.SetLearningRate(0.5)
    o.SetMinimumStepLength(1e-3)
    o.SetNumberOfIterations(20)
    o.SetScales(scales)
    o.StartOptimization()
    assert o.GetStopCondition() == h["stop"] and o.GetCurrentIteration() == h["iterations"]
    assert np.max(np.abs(U.GetParameters() - h["params"])) <= 1e-9 * max(np.max(np.abs(h["params"])), 1.0)


def test_bins_and_transform_limits(pair):
    from itk_gb300 import ExceptionObject
    fixed, moving, T = pair
    with pytest.raises(ExceptionObject, match="6 to 64 bins"):
        make(fixed, moving, perturbed(T, 1), bins=65)
    from itk_gb300 import CorrelationImageToImageMetricv4, DisplacementFieldImage, DisplacementFieldTransform
    F = DisplacementFieldTransform()
    F.SetDisplacementField(DisplacementFieldImage.like(fixed))
    c = CorrelationImageToImageMetricv4()
    c.SetFixedImage(fixed)
    c.SetMovingImage(moving)
    c.SetMovingTransform(F)
    with pytest.raises(ExceptionObject, match="does not support displacement field"):
        c.Initialize()


@pytest.mark.parametrize("composite", [False, True])
@pytest.mark.parametrize("sampled", [False, True])
@pytest.mark.parametrize("gradient", ["image", "cd"])
def test_bspline_matches_oracle(pair, composite, sampled, gradient):
    """B-spline and [affine, B-spline] composite transforms: the B-spline pass 1, the
    per-sample derivative factors and the sparse Jacobian sums against the oracle."""
    from itk_gb300 import CompositeTransform
    fixed, moving, T = pair
    B = data.random_bspline_coefficients(data.bspline_over_image(fixed, (3, 3, 3)), seed=4, max_disp=2.0)
    if composite:
        U = CompositeTransform()
        U.AddTransform(perturbed(T, 5))
        U.AddTransform(B)
    else:
        U = B
    pts = data.random_points(fixed, 0.3, seed=9) if sampled else None
    m = make(fixed, moving, U, gradient, pts)
    v, d = m.GetValueAndDerivative()
    rc, rv, rd, nv, pdf = oracle(fixed, moving, U, gradient, pts)
    assert rc == 0 and m.GetNumberOfValidPoints() == nv
    assert_value_close(v, rv)
    assert_deriv_close(d, rd)
    assert m.GetValue() == v


def test_displacement_field_several_points_per_voxel(pair):
    """Three points in each sampled voxel: the local-support derivative sums their blocks
    into the voxel (Derivatives[offset + i] +=), against the oracle; the FP64 atomics make
    the last bits depend on the order, so the comparison is within the usual tolerance."""
    from cases import shared_voxel_points
    from itk_gb300 import DisplacementFieldImage, DisplacementFieldTransform
    fixed, moving, _ = pair
    F = DisplacementFieldTransform()
    F.SetDisplacementField(DisplacementFieldImage.like(fixed, data.smooth_displacement_field(fixed, 21, 2.0).array))
    pts = shared_voxel_points(fixed, 0.1, seed=8)
    m = make(fixed, moving, F, "image", pts)
    v, d = m.GetValueAndDerivative()
    rc, rv, rd, nv, pdf = oracle(fixed, moving, F, "image", pts)
    assert rc == 0 and m.GetNumberOfValidPoints() == nv
    assert_value_close(v, rv)
    assert_deriv_close(d, rd)


@pytest.mark.parametrize("sampled", [False, True])
@pytest.mark.parametrize("gradient", ["image", "cd"])
def test_displacement_field_matches_oracle(pair, sampled, gradient):
    """A displacement field (local support): the derivative field's blocks sf g at each
    point's voxel, not averaged, against the oracle."""
    from itk_gb300 import DisplacementFieldImage, DisplacementFieldTransform
    fixed, moving, _ = pair
    F = DisplacementFieldTransform()
    F.SetDisplacementField(DisplacementFieldImage.like(fixed, data.smooth_displacement_field(fixed, 21, 2.0).array))
    pts = data.unique_voxel_points(fixed, 0.25, seed=7) if sampled else None
    m = make(fixed, moving, F, gradient, pts)
    assert m.HasLocalSupport()
    v, d = m.GetValueAndDerivative()
    rc, rv, rd, nv, pdf = oracle(fixed, moving, F, gradient, pts)
    assert rc == 0 and m.GetNumberOfValidPoints() == nv
    assert_value_close(v, rv)
    assert_deriv_close(d, rd)
    assert m.GetValue() == v
