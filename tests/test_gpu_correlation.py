"""CorrelationImageToImageMetricv4 on the GPU against the FP64 oracle: value within
1e-5 relative, derivative within 1e-4 of its largest component, dense and
sampled, gradient image and central difference; the reference test's cases
(non-overlapping images: value DBL_MAX with no valid point), self-correlation,
GetValue / device-resident call agreement, and the device optimizer loop."""
import sys
import warnings

import numpy as np
import pytest

from cases import geom, oracle_transform, perturbed, small_pair
from conftest import assert_deriv_close, assert_value_close
from itk_gb300 import (AffineTransform, CorrelationImageToImageMetricv4, Image, RegularStepGradientDescentOptimizerv4,
                       data)
from oracle import oracle as O
from oracle import registration as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pair():
    return small_pair((40, 36, 32), config=1, multimodal=True)


def make(fixed, moving, T, gradient=None, points=None):
    m = CorrelationImageToImageMetricv4()
    m.SetFixedImage(fixed)
    m.SetMovingImage(moving)
    m.SetMovingTransform(T)
    if gradient is not None:
        m.SetMovingImageGradientImage(gradient)
    else:
        m.SetUseMovingImageGradientFilter(False)
    if points is not None:
        m.SetVirtualSampledPointSet(points)
        m.SetUseSampledPointSet(True)
    m.Initialize()
    return m


def oracle(fixed, moving, T, gradient=None, points=None, **kw):
    return O.correlation(fixed.array, geom(fixed), moving.array, geom(moving), oracle_transform(T),
                         moving_grad=None if gradient is None else gradient.array, points=points, **kw)


@pytest.mark.parametrize("gradient_image", [True, False])
@pytest.mark.parametrize("sampled", [False, True])
@pytest.mark.parametrize("seed", [1, 2])
def test_matches_oracle(pair, gradient_image, sampled, seed):
    fixed, moving, T = pair
    U = perturbed(T, seed)
    grad = data.gradient_image(moving) if gradient_image else None
    pts = data.random_points(fixed, 0.3, seed=seed) if sampled else None
    m = make(fixed, moving, U, grad, pts)
    v, d = m.GetValueAndDerivative()
    rc, rv, rd, nv = oracle(fixed, moving, U, grad, pts)
    assert rc == 0 and m.GetNumberOfValidPoints() == nv
    assert_value_close(v, rv)
    assert_deriv_close(d, rd)
    assert m.GetValue() == v


def test_toy_images_and_non_overlap():
    n = 20
    idx = np.arange(n, dtype=np.float64)
    Z, Y, X = np.meshgrid(idx, idx, idx, indexing="ij")

    def toy(o):
        return Image(np.exp(-((X + o[0]) ** 2 + (Y + o[1]) ** 2 + (Z + o[2]) ** 2) / 8.0).astype(np.float32))

    f, mv = toy((0, 0, 0)), toy((1, 0.5, 0.25))
    T = AffineTransform()
    m = make(f, mv, T)
    v, d = m.GetValueAndDerivative()
    rc, rv, rd, nv = oracle(f, mv, T)
    assert_value_close(v, rv)
    assert_deriv_close(d, rd)
    T.SetTranslation([1000.0, 1000.0, 1000.0])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        v, d = m.GetValueAndDerivative()
    assert v == sys.float_info.max and m.GetNumberOfValidPoints() == 0 and np.all(d == 0)


def test_self_correlation(pair):
    fixed, _, _ = pair
    T = AffineTransform()
    T.SetCenter(fixed.physical_center())
    m = make(fixed, fixed, T, data.gradient_image(fixed))
    v, d = m.GetValueAndDerivative()
    assert v == -1.0 and np.all(d == 0)


def test_device_resident_equals_host_call(pair):
    import torch
    fixed, moving, T = pair
    U = perturbed(T, 4)
    m = make(fixed, moving, U, data.gradient_image(moving))
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
    m = make(fixed, moving, U, data.gradient_image(moving))

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
    assert o.GetValue() < -0.5  # correlated


@pytest.mark.parametrize("composite", [False, True])
@pytest.mark.parametrize("sampled", [False, True])
@pytest.mark.parametrize("gradient_image", [True, False])
def test_bspline_matches_oracle(pair, composite, sampled, gradient_image):
    """B-spline and [affine, B-spline] composites: the derivative from per-sample factors
    2 fm / (f2 m2) (f1 - fm / m2 m1) M^T g through the B-spline chunk and parameter sums."""
    from itk_gb300 import CompositeTransform
    fixed, moving, T = pair
    B = data.random_bspline_coefficients(data.bspline_over_image(fixed, (3, 3, 3)), seed=6, max_disp=2.0)
    if composite:
        U = CompositeTransform()
        U.AddTransform(perturbed(T, 7))
        U.AddTransform(B)
    else:
        U = B
    grad = data.gradient_image(moving) if gradient_image else None
    pts = data.random_points(fixed, 0.3, seed=3) if sampled else None
    m = make(fixed, moving, U, grad, pts)
    v, d = m.GetValueAndDerivative()
    rc, rv, rd, nv = oracle(fixed, moving, U, grad, pts)
    assert rc == 0 and m.GetNumberOfValidPoints() == nv
    assert_value_close(v, rv)
    assert_deriv_close(d, rd)
    assert m.GetValue() == pytest.approx(v, rel=1e-12)
