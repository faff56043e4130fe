"""Metrics under a displacement-field transform (local support) on the GPU
against the FP64 oracle: value within 1e-5 relative, the derivative field
within 1e-4 of its largest component; MeanSquares and Mattes, dense and
sampled (one point per voxel), gradient image and central difference.  Plus the
identity-field truth of the reference's ImageToImageMetricv4Test, a constant
field against the equivalent affine translation, the grid check, GetValue /
device-resident agreement, no valid points, and the device optimizer loop."""
import warnings

import numpy as np
import pytest

from cases import geom, oracle_transform
from conftest import assert_deriv_close, assert_value_close
from itk_gb300 import (AffineTransform, DisplacementFieldImage, DisplacementFieldTransform, ExceptionObject, Image,
                       MattesMutualInformationImageToImageMetricv4, MeanSquaresImageToImageMetricv4,
                       RegularStepGradientDescentOptimizerv4, data)
from oracle import oracle as O
from oracle import registration as R

pytestmark = pytest.mark.gpu

BINS = 32


@pytest.fixture(scope="module")
def pair():
    fixed, moving, _ = data.pair_affine((36, 33, 30), config=1, instance=2, multimodal_map=True)
    return fixed, moving


def field_transform(image, array):
    t = DisplacementFieldTransform()
    t.SetDisplacementField(DisplacementFieldImage.like(image, np.array(array, np.float64)))
    return t


def make(kind, fixed, moving, T, gradient=None, points=None):
    m = MeanSquaresImageToImageMetricv4() if kind == "msq" else MattesMutualInformationImageToImageMetricv4()
    if kind != "msq":
        m.SetNumberOfHistogramBins(BINS)
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


def oracle(kind, fixed, moving, T, gradient=None, points=None):
    g = None if gradient is None else gradient.array
    if kind == "msq":
        rc, v, d, nv = O.mean_squares(fixed.array, geom(fixed), moving.array, geom(moving), oracle_transform(T),
                                      moving_grad=g, points=points)
    else:
        rc, v, d, nv, _, _ = O.mattes(fixed.array, geom(fixed), moving.array, geom(moving), oracle_transform(T),
                                      bins=BINS, moving_grad=g, points=points)
    return rc, v, np.asarray(d), nv


@pytest.mark.parametrize("kind", ["msq", "mattes"])
@pytest.mark.parametrize("sampled", [False, True])
@pytest.mark.parametrize("gradient_image", [True, False])
def test_matches_oracle(pair, kind, sampled, gradient_image):
    fixed, moving = pair
    T = field_transform(fixed, data.smooth_displacement_field(fixed, seed=7, max_disp=2.5).array)
    grad = data.gradient_image(moving) if gradient_image else None
    pts = data.unique_voxel_points(fixed, 0.25, seed=3) if sampled else None
    m = make(kind, fixed, moving, T, grad, pts)
    assert m.HasLocalSupport() and m.GetNumberOfLocalParameters() == 3
    v, d = m.GetValueAndDerivative()
    rc, rv, rd, nv = oracle(kind, fixed, moving, T, grad, pts)
    assert rc == 0 and m.GetNumberOfValidPoints() == nv
    assert len(d) == 3 * fixed.array.size
    assert_value_close(v, rv)
    assert_deriv_close(d, rd)
    assert m.GetValue() == v


def test_meansquares_several_points_per_voxel(pair):
    """Three points in each sampled voxel: MeanSquares sums their blocks into the voxel as
    the reference's local-support branch does, against the oracle (the FP64 atomics make
    the last bits order-dependent).  Mattes is left out: the reference keeps one joint-PDF
    index per voxel there, whichever point's thread wrote last."""
    from cases import shared_voxel_points
    fixed, moving = pair
    T = field_transform(fixed, data.smooth_displacement_field(fixed, seed=7, max_disp=2.5).array)
    grad = data.gradient_image(moving)
    pts = shared_voxel_points(fixed, 0.1, seed=4)
    m = make("msq", fixed, moving, T, grad, pts)
    v, d = m.GetValueAndDerivative()
    rc, rv, rd, nv = oracle("msq", fixed, moving, T, grad, pts)
    assert rc == 0 and m.GetNumberOfValidPoints() == nv
    assert_value_close(v, rv)
    assert_deriv_close(d, rd)


def test_identity_field_meansquares_truth(pair):
    fixed, moving = pair
    grad = data.gradient_image(moving)
    m = make("msq", fixed, moving, field_transform(fixed, np.zeros(fixed.array.shape + (3,))), grad)
    v, d = m.GetValueAndDerivative()
    diff = (fixed.array - moving.array).astype(np.float64)
    truth = (2.0 * diff[..., None] * grad.array).reshape(-1)
    assert_value_close(v, np.mean(diff ** 2))
    assert_deriv_close(d, truth)


@pytest.mark.parametrize("kind", ["msq", "mattes"])
def test_constant_field_is_a_translation(pair, kind):
    fixed, moving = pair
    c = np.array([0.75, -0.5, 0.25])
    grad = data.gradient_image(moving)
    mf = make(kind, fixed, moving, field_transform(fixed, np.broadcast_to(c, fixed.array.shape + (3,))), grad)
    A = AffineTransform()
    A.SetTranslation(c)
    ma = make(kind, fixed, moving, A, grad)
    vf, df = mf.GetValueAndDerivative()
    va, da = ma.GetValueAndDerivative()
    assert mf.GetNumberOfValidPoints() == ma.GetNumberOfValidPoints()
    assert_value_close(vf, va)
    s = np.asarray(df).reshape(-1, 3).sum(axis=0)
    want = np.asarray(da)[9:12] * (ma.GetNumberOfValidPoints() if kind == "msq" else 1.0)
    assert_deriv_close(s, want)


def test_field_must_share_the_virtual_grid(pair):
    fixed, moving = pair
    shifted = Image(fixed.array, fixed.spacing, fixed.origin + 0.5)
    with pytest.raises(ExceptionObject, match="same physical space"):
        make("msq", fixed, moving, field_transform(shifted, np.zeros(fixed.array.shape + (3,))))
    small = Image(fixed.array[:, :, :-1])
    with pytest.raises(ExceptionObject, match="same size"):
        make("mattes", fixed, moving, field_transform(small, np.zeros(small.array.shape + (3,))))


@pytest.mark.parametrize("kind", ["msq", "mattes"])
def test_device_resident_equals_host_call(pair, kind):
    import torch
    fixed, moving = pair
    T = field_transform(fixed, data.smooth_displacement_field(fixed, seed=9, max_disp=2.0).array)
    m = make(kind, fixed, moving, T, data.gradient_image(moving))
    v, d = m.GetValueAndDerivative()
    dp = torch.tensor(T.GetParameters(), dtype=torch.float64, device="cuda")
    out = torch.zeros(2 + dp.numel(), dtype=torch.float64, device="cuda")
    m.evaluate_device(dp.data_ptr(), out.data_ptr(), True)
    assert m.synchronize() == 0
    o = out.cpu().numpy()
    assert o[0] == v and np.array_equal(o[2:], d)


def test_no_valid_points(pair):
    fixed, moving = pair
    m = make("msq", fixed, moving, field_transform(fixed, np.full(fixed.array.shape + (3,), 1000.0)))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        v, d = m.GetValueAndDerivative()
    assert v == np.finfo(np.float64).max and m.GetNumberOfValidPoints() == 0 and not np.any(d)


def test_device_optimizer_matches_host_loop():
    fixed, moving, _ = data.pair_affine((12, 12, 12), config=1, instance=5, multimodal_map=False)
    T = field_transform(fixed, np.zeros(fixed.array.shape + (3,)))
    p0 = T.GetParameters().copy()
    scales = np.array([1.0, 2.0, 0.5])
    m = make("msq", fixed, moving, T, data.gradient_image(moving))

    def evaluate(p):
        T.SetParameters(p)
        v, d = m.GetValueAndDerivative()
        return 0, v, d

    h = R.regular_step(evaluate, p0, learning_rate=1.0, minimum_step_length=1e-3, number_of_iterations=15,
                       scales=np.tile(scales, p0.size // 3), mean_squares=True)
    T.SetParameters(p0)
    o = RegularStepGradientDescentOptimizerv4()
    o.SetMetric(m)
    o.SetLearningRate(1.0)
    o.SetMinimumStepLength(1e-3)
    o.SetNumberOfIterations(15)
    o.SetScales(scales)  # one scale per local parameter
    o.StartOptimization()
    assert o.GetStopCondition() == h["stop"] and o.GetCurrentIteration() == h["iterations"]
    assert np.max(np.abs(T.GetParameters() - h["params"])) <= 1e-9 * max(np.max(np.abs(h["params"])), 1.0)


@pytest.mark.parametrize("kind", ["msq", "mattes"])
def test_oblique_grids_match_oracle(pair, kind):
    """A rotated image direction: the positions take the general double-float map
    (the axis-aligned grids above take the diagonal one)."""
    fixed0, moving0 = pair
    t = np.deg2rad(20.0)
    rot = np.array([[np.cos(t), -np.sin(t), 0.0], [np.sin(t), np.cos(t), 0.0], [0.0, 0.0, 1.0]])
    fixed = Image(fixed0.array, spacing=(1.0, 1.2, 0.9), origin=(3.0, -2.0, 1.0), direction=rot)
    moving = Image(moving0.array, spacing=(1.0, 1.2, 0.9), origin=(3.0, -2.0, 1.0), direction=rot)
    T = field_transform(fixed, data.smooth_displacement_field(fixed, seed=11, max_disp=2.0).array)
    grad = data.gradient_image(moving)
    m = make(kind, fixed, moving, T, grad)
    v, d = m.GetValueAndDerivative()
    rc, rv, rd, nv = oracle(kind, fixed, moving, T, grad)
    assert rc == 0 and m.GetNumberOfValidPoints() == nv
    assert_value_close(v, rv)
    assert_deriv_close(d, rd)


def test_device_optimizer_many_parameters(pair):
    """The device RegularStep loop on a field of 138,240 parameters (grid-stride step
    kernels) against the oracle's RegularStep restatement driven by the same metric."""
    fixed, moving = pair
    T = field_transform(fixed, np.zeros(fixed.array.shape + (3,)))
    p0 = T.GetParameters().copy()
    assert p0.size > 65536
    m = make("mattes", fixed, moving, T, data.gradient_image(moving))

    def evaluate(p):
        T.SetParameters(p)
        v, d = m.GetValueAndDerivative()
        return 0, v, d

    h = R.regular_step(evaluate, p0, learning_rate=1.0, minimum_step_length=1e-3, number_of_iterations=8)
    T.SetParameters(p0)
    o = RegularStepGradientDescentOptimizerv4()
    o.SetMetric(m)
    o.SetLearningRate(1.0)
    o.SetMinimumStepLength(1e-3)
    o.SetNumberOfIterations(8)
    o.StartOptimization()
    assert o.GetStopCondition() == h["stop"] and o.GetCurrentIteration() == h["iterations"]
    assert np.max(np.abs(T.GetParameters() - h["params"])) <= 1e-9 * max(np.max(np.abs(h["params"])), 1.0)


@pytest.mark.parametrize("kind", ["msq", "mattes"])
def test_virtual_domain_with_dropped_voxels(pair, kind):
    """A virtual domain shifted by half a voxel: its last plane falls outside the fixed
    image, those voxels hold no sample, and the derivative field is cleared before the
    blocks are stored (the other voxels' blocks as the oracle's)."""
    fixed, moving = pair
    virt = Image(np.zeros(fixed.array.shape, np.float32), spacing=fixed.spacing, origin=fixed.origin + 0.5,
                 direction=fixed.direction)
    T = field_transform(virt, data.smooth_displacement_field(virt, seed=13, max_disp=1.5).array)
    grad = data.gradient_image(moving)
    m = MeanSquaresImageToImageMetricv4() if kind == "msq" else MattesMutualInformationImageToImageMetricv4()
    if kind != "msq":
        m.SetNumberOfHistogramBins(BINS)
    m.SetFixedImage(fixed)
    m.SetMovingImage(moving)
    m.SetVirtualDomainFromImage(virt)
    m.SetMovingTransform(T)
    m.SetMovingImageGradientImage(grad)
    m.Initialize()
    v, d = m.GetValueAndDerivative()
    assert m.GetNumberOfDomainPoints() == virt.array.size
    g = grad.array
    if kind == "msq":
        rc, rv, rd, nv = O.mean_squares(fixed.array, geom(fixed), moving.array, geom(moving), oracle_transform(T),
                                        moving_grad=g, virtual_geom=geom(virt))
    else:
        rc, rv, rd, nv, _, _ = O.mattes(fixed.array, geom(fixed), moving.array, geom(moving), oracle_transform(T),
                                        bins=BINS, moving_grad=g, virtual_geom=geom(virt))
    assert rc == 0 and m.GetNumberOfValidPoints() == nv < virt.array.size
    assert_value_close(v, rv)
    assert_deriv_close(d, rd)
    blocks = np.asarray(d).reshape(virt.array.shape + (3,))
    assert not np.any(blocks[:, :, -1])  # the last x plane maps outside the fixed image


@pytest.mark.parametrize("kind", ["msq", "mattes"])
@pytest.mark.parametrize("sampled", [False, True])
def test_affine_then_field_composite(pair, kind, sampled):
    """CompositeTransform [affine, displacement field] (the field applied first and
    optimized, as behind a registration's moving initial transform): positions
    A(x + u(x)), local blocks from M^T g, against the oracle."""
    from itk_gb300 import CompositeTransform
    fixed, moving = pair
    A = AffineTransform()
    A.SetCenter(fixed.physical_center())
    t = np.deg2rad(6.0)
    A.SetMatrix([[np.cos(t), -np.sin(t), 0.0], [np.sin(t), np.cos(t), 0.0], [0.0, 0.0, 1.0]])
    A.SetTranslation([0.8, -0.5, 0.3])
    F = field_transform(fixed, data.smooth_displacement_field(fixed, seed=17, max_disp=1.5).array)
    C = CompositeTransform()
    C.AddTransform(A)
    C.AddTransform(F)
    grad = data.gradient_image(moving)
    pts = data.unique_voxel_points(fixed, 0.25, seed=5) if sampled else None
    m = make(kind, fixed, moving, C, grad, pts)
    assert m.HasLocalSupport() and m.GetNumberOfParameters() == 3 * fixed.array.size
    v, d = m.GetValueAndDerivative()
    rc, rv, rd, nv = oracle(kind, fixed, moving, C, grad, pts)
    assert rc == 0 and m.GetNumberOfValidPoints() == nv
    assert_value_close(v, rv)
    assert_deriv_close(d, rd)
