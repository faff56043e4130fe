"""Parity at the benchmark configurations' full sizes, against the FP64 oracle.

* B-spline configuration, one evaluation: 192x192x160 volumes whose moving
  image carries a seeded smooth displacement, 10 % RANDOM samples drawn as
  ImageRegistrationMethodv4 draws them, 50 bins, [affine, BSplineTransform
  order 3] with the B-spline optimized, over a 4^3 mesh (7^3 nodes, 1029
  parameters) and a 5^3 mesh (8^3 nodes, 1536 parameters), Mattes MI and
  MeanSquares.  At these sizes the kernels take their large-grid forms (nodes
  and chunk lists of full-size sample sets, the block-per-node parameter
  gather), which the small parity tests do not reach.
* Mattes affine registration: 256x256x200, 3 levels (shrink 4/2/1, sigmas
  2/1/0 mm), 20 % RANDOM, RegularStep, through ImageRegistrationMethodv4 and
  the device optimizer, against the oracle's restatement of the same levels
  and optimizer with the same points: final displacement within 0.05 voxel RMS.
* B-spline registration: the 192x192x160 pair, 2 levels (shrink 2/1, sigmas
  1/0 mm), 10 % RANDOM, [affine initial, B-spline mesh 4 optimized], the same
  check.

Value within 1e-5 relative, derivative within 1e-4 of its largest component.
"""
import numpy as np
import pytest

from cases import run_oracle
from conftest import MATTES_VALUE_ATOL, assert_deriv_close, assert_value_close
from itk_gb300 import (AffineTransform, BSplineTransform, CompositeTransform, ImageRegistrationMethodv4,
                       MattesMutualInformationImageToImageMetricv4, MeanSquaresImageToImageMetricv4,
                       RegularStepGradientDescentOptimizerv4, data, sample_points)
from itk_gb300.registration import RANDOM

pytestmark = pytest.mark.gpu

BSPLINE_SIZE = (192, 192, 160)
AFFINE_SIZE = (256, 256, 200)


@pytest.fixture(scope="module")
def bspline_pair():
    fixed, moving, A, B = data.pair_bspline(BSPLINE_SIZE, (4, 4, 4), instance=0, multimodal_map=True)
    pts, _ = sample_points(RANDOM, fixed.GetSize(), fixed.spacing, fixed.origin, fixed.direction, 0.1, 2001)
    return fixed, moving, A, B, data.gradient_image(moving), pts


def composite(A, B):
    C = CompositeTransform()
    C.AddTransform(A)
    C.AddTransform(B)
    return C


def bspline_under_test(fixed, B, mesh):
    """Mid-optimization B-spline parameters: half the generating coefficients on the
    generating mesh, seeded coefficients of at most 2 mm on another mesh."""
    if mesh == 4:
        T = BSplineTransform()
        T.SetFixedParameters(B.GetFixedParameters())
        T.SetParameters(0.5 * B.GetParameters())
        return T
    return data.random_bspline_coefficients(data.bspline_over_image(fixed, (mesh,) * 3), 500 + mesh, 2.0)


@pytest.mark.parametrize("kind", ["mattes", "msq"])
@pytest.mark.parametrize("mesh", [4, 5])
def test_bspline_config_single_evaluation(bspline_pair, mesh, kind):
    fixed, moving, A, B, grad, pts = bspline_pair
    T = composite(A, bspline_under_test(fixed, B, mesh))
    assert T.GetNumberOfParameters() == 3 * (mesh + 3) ** 3
    m = MeanSquaresImageToImageMetricv4() if kind == "msq" else MattesMutualInformationImageToImageMetricv4()
    m.SetFixedImage(fixed)
    m.SetMovingImage(moving)
    m.SetMovingTransform(T)
    m.SetMovingImageGradientImage(grad)
    if kind == "mattes":
        m.SetNumberOfHistogramBins(50)
    m.SetVirtualSampledPointSet(pts)
    m.SetUseSampledPointSet(True)
    m.Initialize()
    v, d = m.GetValueAndDerivative()
    r = run_oracle(kind, fixed, moving, T, gradient=grad, points=pts, bins=50)
    assert r["status"] == 0
    assert m.GetNumberOfValidPoints() == r["nvalid"]
    assert_value_close(v, r["value"], atol=MATTES_VALUE_ATOL if kind == "mattes" else 0.0)
    assert_deriv_close(d, r["derivative"])
    assert m.GetValue() == v


def displacement_rms(fixed, T1, T2, step=4):
    nx, ny, nz = fixed.GetSize()
    iz, iy, ix = np.meshgrid(np.arange(0, nz, step), np.arange(0, ny, step), np.arange(0, nx, step), indexing="ij")
    idx = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], 1).astype(np.float64)
    x = idx @ fixed.index_to_physical().T + fixed.origin
    d = (T1.TransformPoint(x) - T2.TransformPoint(x)) / fixed.spacing
    return float(np.sqrt(np.mean(np.sum(d * d, axis=1))))


def gpu_registration(fixed, moving, transform, levels, pct, opt, seed, moving_initial=None):
    m = MattesMutualInformationImageToImageMetricv4()
    m.SetNumberOfHistogramBins(50)
    o = RegularStepGradientDescentOptimizerv4()
    o.SetLearningRate(opt["learning_rate"])
    o.SetNumberOfIterations(opt["number_of_iterations"])
    o.SetMinimumStepLength(opt["minimum_step_length"])
    o.SetScales(opt.get("scales"))
    reg = ImageRegistrationMethodv4()
    reg.SetFixedImage(fixed)
    reg.SetMovingImage(moving)
    reg.SetMetric(m)
    reg.SetOptimizer(o)
    reg.SetInitialTransform(transform)
    if moving_initial is not None:
        reg.SetMovingInitialTransform(moving_initial)
    reg.SetNumberOfLevels(len(levels))
    reg.SetShrinkFactorsPerLevel([lv[0] for lv in levels])
    reg.SetSmoothingSigmasPerLevel([lv[1] for lv in levels])
    reg.SetSmoothingSigmasAreSpecifiedInPhysicalUnits(True)
    reg.SetMetricSamplingStrategy(RANDOM)
    reg.SetMetricSamplingPercentage(pct)
    reg.MetricSamplingReinitializeSeed(seed)
    reg.Update()
    return reg, o


def oracle_registration(fixed, moving, T0, levels, points, opt):
    from cases import geom
    from oracle import registration as R
    kindcode, params0, tfixed = T0.flat()
    lv = [dict(shrink=(s,) * 3, sigma=sg, sigma_physical=True, points=p) for (s, sg), p in zip(levels, points)]
    return R.register("mattes", fixed.array, geom(fixed), moving.array, geom(moving), kindcode, params0, tfixed, lv,
                      opt, bins=50)


def test_affine_config_registration_three_levels():
    """Each level runs to convergence (RegularStep's minimum step length), as a
    registration that is used ends, so the comparison is of end points rather than of
    positions part-way along two FP32 / FP64 trajectories."""
    fixed, moving, _ = data.pair_affine(AFFINE_SIZE, config=1, multimodal_map=True)
    R = 0.5 * float(max(np.asarray(fixed.GetSize()) * fixed.spacing))
    opt = dict(learning_rate=1.0, number_of_iterations=150, minimum_step_length=1e-3,
               scales=np.array([R * R] * 9 + [1.0] * 3))
    levels = [(4, 2.0), (2, 1.0), (1, 0.0)]
    U = AffineTransform()
    U.SetCenter(fixed.physical_center())
    U0 = AffineTransform()
    U0.SetCenter(fixed.physical_center())
    reg, o = gpu_registration(fixed, moving, U, levels, 0.2, opt, seed=1001)
    pts = [reg.GetMetricSamplePoints(k) for k in range(3)]
    assert len(pts[2]) == 2621440
    p, res = oracle_registration(fixed, moving, U0, levels, pts, opt)
    U0.SetParameters(p)
    trail = [(r["stop"], r["iterations"]) for r in res]
    assert o.GetStopCondition() == res[-1]["stop"], trail
    rms = displacement_rms(fixed, U, U0)
    assert rms <= 0.05, f"displacement RMS {rms:.4f} voxel; oracle levels (stop, iterations) {trail}, " \
                        f"device final level {o.GetStopCondition()}, {o.GetCurrentIteration()}"
    assert np.max(np.abs(U.GetParameters() - AffineTransform().GetParameters())) > 1e-3  # it moved


def test_bspline_config_registration_two_levels(bspline_pair):
    fixed, moving, A, B, _, _ = bspline_pair
    Bs = data.bspline_over_image(fixed, (4, 4, 4))
    Bo = data.bspline_over_image(fixed, (4, 4, 4))
    opt = dict(learning_rate=1.0, number_of_iterations=10, minimum_step_length=1e-3)
    levels = [(2, 1.0), (1, 0.0)]
    reg, o = gpu_registration(fixed, moving, Bs, levels, 0.1, opt, seed=2001, moving_initial=A)
    pts = [reg.GetMetricSamplePoints(k) for k in range(2)]
    p, res = oracle_registration(fixed, moving, composite(A, Bo), levels, pts, opt)
    Bo.SetParameters(p)
    assert o.GetStopCondition() == res[-1]["stop"]
    rms = displacement_rms(fixed, composite(A, Bs), composite(A, Bo))
    assert rms <= 0.05, f"displacement RMS {rms:.4f} voxel"
    assert np.max(np.abs(Bs.GetParameters())) > 0.1  # it moved
