"""GPU metric vs the FP64 oracle on identical inputs (affine transform).

Tolerances (the parity contract): metric value within 1e-5 relative; derivative
within 1e-4 of its largest-magnitude component; valid-point counts equal up to
samples whose moving position sits within FP32 rounding of a buffer edge.
"""
import json
import os

import numpy as np
import pytest

from cases import mattes_2d_case, mattes_2d_sample_points, perturbed, run_oracle, small_pair
from conftest import MATTES_VALUE_ATOL, assert_deriv_close, assert_value_close
from itk_gb300 import (AffineTransform, ExceptionObject, MattesMutualInformationImageToImageMetricv4,
                       MeanSquaresImageToImageMetricv4, data)
from itk_gb300 import _capi

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_known_values.json")))


def make_metric(kind, fixed, moving, transform, gradient=None, points=None, bins=50, points_virtual=True):
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
        if points_virtual:
            m.SetVirtualSampledPointSet(points)
        else:
            m.SetFixedSampledPointSet(points)
        m.SetUseSampledPointSet(True)
    m.Initialize()
    return m


def check_against_oracle(kind, fixed, moving, transform, gradient=None, points=None, bins=50, nvalid_slack=0):
    m = make_metric(kind, fixed, moving, transform, gradient, points, bins)
    v, d = m.GetValueAndDerivative()
    r = run_oracle(kind, fixed, moving, transform, gradient=gradient, points=points, bins=bins)
    assert r["status"] == 0
    assert abs(m.GetNumberOfValidPoints() - r["nvalid"]) <= nvalid_slack
    assert_value_close(v, r["value"], atol=MATTES_VALUE_ATOL if kind == "mattes" else 0.0)
    assert_deriv_close(d, r["derivative"])
    # GetValue == GetValueAndDerivative: the reference allows 8 ULP
    # (itkMattesMutualInformationImageToImageMetricv4Test.cxx:319); the device reductions are deterministic
    vo = m.GetValue()
    assert vo == v
    return m, r


@pytest.fixture(scope="module")
def pair():
    fixed, moving, T = small_pair((41, 37, 29), config=0)
    return fixed, moving, T, data.gradient_image(moving)


@pytest.fixture(scope="module")
def pair_mm():
    fixed, moving, T = small_pair((48, 44, 40), config=1, multimodal=True)
    return fixed, moving, T, data.gradient_image(moving)


@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("gradient_image", [True, False])
def test_mean_squares_dense(pair, seed, gradient_image):
    fixed, moving, T, grad = pair
    check_against_oracle("msq", fixed, moving, perturbed(T, seed), grad if gradient_image else None, nvalid_slack=2)


@pytest.mark.parametrize("seed", [0, 1])
def test_mean_squares_sparse(pair, seed):
    fixed, moving, T, grad = pair
    pts = data.random_points(fixed, 0.2, seed=100 + seed)
    check_against_oracle("msq", fixed, moving, perturbed(T, seed), grad, points=pts, nvalid_slack=2)


@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("gradient_image", [True, False])
def test_mattes_dense(pair_mm, seed, gradient_image):
    fixed, moving, T, grad = pair_mm
    m, r = check_against_oracle("mattes", fixed, moving, perturbed(T, seed), grad if gradient_image else None,
                                nvalid_slack=2)
    np.testing.assert_allclose(m.GetJointPDF(), r["pdf"], atol=2e-6)
    np.testing.assert_allclose(m.GetHistogramState(), r["state"], rtol=1e-12)


@pytest.mark.parametrize("bins", [5, 20, 50, 100])
def test_mattes_sparse_bins(pair_mm, bins):
    fixed, moving, T, grad = pair_mm
    pts = data.random_points(fixed, 0.2, seed=7)
    check_against_oracle("mattes", fixed, moving, perturbed(T, 4), grad, points=pts, bins=bins, nvalid_slack=2)


def test_mattes_at_true_transform(pair_mm):
    """Near the optimum the derivative is small: parity must hold relative to its own size."""
    fixed, moving, T, grad = pair_mm
    pts = data.random_points(fixed, 0.3, seed=9)
    check_against_oracle("mattes", fixed, moving, T, grad, points=pts, nvalid_slack=2)


def test_mattes_reference_known_values_on_gpu():
    """The reference's 2-D known-answer case (Image<float> semantics), dense and sampled."""
    g = GOLDEN["mattes_2d_known_values"]
    fixed, moving = mattes_2d_case()
    t = AffineTransform()
    for pts in (None, mattes_2d_sample_points(fixed)):
        m = make_metric("mattes", fixed, moving, t, None, pts, points_virtual=False)
        v, d = m.GetValueAndDerivative()
        assert abs(abs(v / g["values"][0]) - 1.0) <= g["value_tolerance"]
        r = run_oracle("mattes", fixed, moving, t, points=pts)
        assert_value_close(v, r["value"])
        assert_deriv_close(d, r["derivative"])
        assert m.GetNumberOfValidPoints() == r["nvalid"]
    m = make_metric("mattes", fixed, moving, t)
    v, _ = m.GetValueAndDerivative()
    assert abs(v / g["values"][0] - 1.0) < 2e-5


def test_fixed_sampled_points_outside_domain_are_dropped(pair):
    fixed, moving, T, grad = pair
    pts = data.random_points(fixed, 0.1, seed=3)
    pts = np.concatenate([pts, np.array([[-50.0, 0, 0], [0, 1e4, 0]], np.float32)])
    m = make_metric("msq", fixed, moving, T, grad, pts, points_virtual=False)
    assert m.GetNumberOfDomainPoints() == len(pts)
    v, d = m.GetValueAndDerivative()
    r = run_oracle("msq", fixed, moving, T, gradient=grad, points=pts[:-2])
    assert_value_close(v, r["value"])


def test_no_overlap(pair):
    fixed, moving, T, grad = pair
    t = AffineTransform()
    t.SetTranslation([1e4, 0, 0])
    m = make_metric("msq", fixed, moving, t, grad)
    with pytest.warns(UserWarning):
        v, d = m.GetValueAndDerivative()
    assert v == np.finfo(np.float64).max and not np.any(d) and m.GetNumberOfValidPoints() == 0
    m = make_metric("mattes", fixed, moving, t, grad)
    with pytest.raises(ExceptionObject) as ei:
        m.GetValueAndDerivative()
    assert ei.value.code == _capi.GB_ERR_NO_VALID_POINTS
    assert "All samples map outside moving image buffer" in str(ei.value)


def test_constant_images_raise():
    n = 20
    varying = data.Image(np.arange(n * n, dtype=np.float32).reshape(1, n, n))
    const = data.Image(np.zeros((1, n, n), np.float32))
    for fx, mv, code, text in ((const, varying, _capi.GB_ERR_FIXED_CONSTANT, "All fixed-image samples"),
                               (varying, const, _capi.GB_ERR_MOVING_CONSTANT, "All moving-image samples")):
        with pytest.raises(ExceptionObject) as ei:
            make_metric("mattes", fx, mv, AffineTransform())
        assert ei.value.code == code and text in str(ei.value)


def test_ragged_and_thin_volumes():
    for size in ((1, 1, 9), (7, 1, 1), (3, 5, 2), (65, 3, 17)):
        fixed = data.blob_volume(size, seed=11)
        moving = data.blob_volume(size, seed=12)
        t = AffineTransform()
        t.SetTranslation([0.3, -0.2, 0.1])
        for kind in ("msq", "mattes"):
            if kind == "mattes" and fixed.array.size < 2:
                continue
            m = make_metric(kind, fixed, moving, t)
            r = run_oracle(kind, fixed, moving, t)
            if r["status"] != 0:
                with pytest.raises(ExceptionObject):
                    m.GetValueAndDerivative()
                continue
            v, d = m.GetValueAndDerivative()
            assert m.GetNumberOfValidPoints() == r["nvalid"]
            assert_value_close(v, r["value"])
            assert_deriv_close(d, r["derivative"])


def test_repeated_calls_are_stable(pair_mm):
    fixed, moving, T, grad = pair_mm
    m = make_metric("mattes", fixed, moving, perturbed(T, 5), grad)
    v0, d0 = m.GetValueAndDerivative()
    for _ in range(5):
        v, d = m.GetValueAndDerivative()
        assert v == v0 and np.array_equal(d, d0), "evaluations must be bitwise reproducible"
    m2 = make_metric("msq", fixed, moving, perturbed(T, 5), grad)
    a = m2.GetValueAndDerivative()
    b = m2.GetValueAndDerivative()
    assert a[0] == b[0] and np.array_equal(a[1], b[1])


def test_parameter_updates_follow_transform(pair):
    fixed, moving, T, grad = pair
    U = perturbed(T, 8)
    m = make_metric("msq", fixed, moving, U, grad)
    m.GetValueAndDerivative()
    U.SetTranslation(U.GetTranslation() + np.array([0.5, -0.25, 0.125]))
    v, d = m.GetValueAndDerivative()
    r = run_oracle("msq", fixed, moving, U, gradient=grad)
    assert_value_close(v, r["value"])
    assert_deriv_close(d, r["derivative"])


def test_full_size_mattes_config(pair_mm):
    """Mattes, 50 bins, 20 % random samples of a 256x256x200 multimodal pair: GPU vs oracle."""
    fixed, moving, T = small_pair((256, 256, 200), config=1, multimodal=True)
    grad = data.gradient_image(moving)
    pts = data.random_points(fixed, 0.2, seed=1001)
    check_against_oracle("mattes", fixed, moving, perturbed(T, 11, scale=0.01, trans=2.0), grad, points=pts,
                         nvalid_slack=8)


@pytest.mark.parametrize("resolution", [10.0, 1e6])
def test_floating_point_correction(resolution):
    """SetUseFloatingPointCorrection on the GPU (MeanSquares, affine) against the oracle's
    truncated sums; the correction is seen at a coarse resolution."""
    from cases import geom, oracle_transform
    from oracle import oracle as O
    fixed, moving, T = small_pair((40, 36, 32), config=0)
    U = perturbed(T, 8)
    grad = data.gradient_image(moving)
    out = []
    for on in (False, True):
        m = MeanSquaresImageToImageMetricv4()
        m.SetFixedImage(fixed)
        m.SetMovingImage(moving)
        m.SetMovingTransform(U)
        m.SetMovingImageGradientImage(grad)
        m.SetUseFloatingPointCorrection(on)
        m.SetFloatingPointCorrectionResolution(resolution)
        m.Initialize()
        out.append(m.GetValueAndDerivative())
    rc, rv, rd, nv = O.mean_squares_fpc(fixed.array, geom(fixed), moving.array, geom(moving), oracle_transform(U),
                                        resolution, moving_grad=grad.array)
    assert rc == 0
    assert out[0][0] == out[1][0]
    assert_deriv_close(out[1][1], rd)
    if resolution == 10.0:
        assert np.max(np.abs(out[1][1] - out[0][1])) > 1e-3 / nv
