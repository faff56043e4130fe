"""End-to-end registrations (ImageRegistrationMethodv4 + device optimizer) against
the oracle's restatement of the same levels and optimizer on the FP64 oracle
metric, with the same sample points.  The contract: the final transforms'
displacement fields over the fixed image differ by at most 0.05 voxel RMS."""
import numpy as np
import pytest

from cases import geom, perturbed, small_pair
from itk_gb300 import (CompositeTransform, ImageRegistrationMethodv4, MattesMutualInformationImageToImageMetricv4,
                       MeanSquaresImageToImageMetricv4, RegularStepGradientDescentOptimizerv4, data)
from itk_gb300.registration import NONE, RANDOM
from oracle import registration as R

pytestmark = pytest.mark.gpu

AFFINE_SCALES = np.array([1.0] * 9 + [1.0 / 50.0] * 3)


def displacement_rms(fixed, T1, T2, step=3):
    nx, ny, nz = fixed.GetSize()
    iz, iy, ix = np.meshgrid(np.arange(0, nz, step), np.arange(0, ny, step), np.arange(0, nx, step), indexing="ij")
    idx = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], 1).astype(np.float64)
    x = idx @ (fixed.direction @ np.diag(fixed.spacing)).T + np.asarray(fixed.origin)
    d = (T1.TransformPoint(x) - T2.TransformPoint(x)) / np.asarray(fixed.spacing)
    return float(np.sqrt(np.mean(np.sum(d * d, axis=1))))


def run_gpu(kind, fixed, moving, transform, levels, strategy, pct, opt_kw, moving_initial=None, bins=32, seed=7):
    m = MeanSquaresImageToImageMetricv4() if kind == "msq" else MattesMutualInformationImageToImageMetricv4()
    if kind == "mattes":
        m.SetNumberOfHistogramBins(bins)
    o = RegularStepGradientDescentOptimizerv4()
    o.SetLearningRate(opt_kw["learning_rate"])
    o.SetNumberOfIterations(opt_kw["number_of_iterations"])
    o.SetMinimumStepLength(opt_kw["minimum_step_length"])
    o.SetRelaxationFactor(opt_kw.get("relaxation_factor", 0.5))
    o.SetGradientMagnitudeTolerance(opt_kw.get("gradient_magnitude_tolerance", 1e-4))
    o.SetScales(opt_kw.get("scales"))
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
    reg.SetMetricSamplingStrategy(strategy)
    reg.SetMetricSamplingPercentage(pct)
    reg.MetricSamplingReinitializeSeed(seed)
    reg.Update()
    return reg, o


def run_oracle(kind, fixed, moving, T0, levels, points, opt_kw, bins=32):
    kindcode, params0, tfixed = T0.flat()
    lv = [dict(shrink=(s,) * 3, sigma=sg, sigma_physical=True, points=p) for (s, sg), p in zip(levels, points)]
    return R.register(kind, fixed.array, geom(fixed), moving.array, geom(moving), kindcode, params0, tfixed, lv,
                      opt_kw, bins=bins)


@pytest.fixture(scope="module")
def pair_mono():
    return small_pair((48, 44, 40), config=0, multimodal=False)


@pytest.fixture(scope="module")
def pair_mm():
    return small_pair((48, 44, 40), config=1, multimodal=True)


OPT = dict(learning_rate=0.5, number_of_iterations=30, minimum_step_length=1e-3, scales=AFFINE_SCALES)


def test_affine_mean_squares_dense_two_levels(pair_mono):
    fixed, moving, T = pair_mono
    U = perturbed(T, 21, scale=0.02, trans=1.5)
    U0 = perturbed(T, 21, scale=0.02, trans=1.5)
    levels = [(2, 1.0), (1, 0.0)]
    reg, o = run_gpu("msq", fixed, moving, U, levels, NONE, 1.0, OPT)
    p, res = run_oracle("msq", fixed, moving, U0, levels, [None, None], OPT)
    U0.SetParameters(p)
    assert o.GetStopCondition() == res[-1]["stop"]
    rms = displacement_rms(fixed, U, U0)
    assert rms <= 0.05, f"displacement RMS {rms:.4f} voxel"


def test_affine_mattes_random_two_levels(pair_mm):
    fixed, moving, T = pair_mm
    U = perturbed(T, 22, scale=0.02, trans=1.5)
    U0 = perturbed(T, 22, scale=0.02, trans=1.5)
    levels = [(2, 1.0), (1, 0.0)]
    reg, o = run_gpu("mattes", fixed, moving, U, levels, RANDOM, 0.2, OPT)
    pts = [reg.GetMetricSamplePoints(0), reg.GetMetricSamplePoints(1)]
    p, res = run_oracle("mattes", fixed, moving, U0, levels, pts, OPT)
    U0.SetParameters(p)
    rms = displacement_rms(fixed, U, U0)
    assert rms <= 0.05, f"displacement RMS {rms:.4f} voxel"


def test_bspline_composite_mattes_random():
    fixed, moving, A, B = data.pair_bspline((44, 40, 36), (4, 4, 4), instance=3, multimodal_map=True)
    Bs = data.bspline_over_image(fixed, (4, 4, 4))
    Bo = data.bspline_over_image(fixed, (4, 4, 4))
    opt = dict(learning_rate=1.0, number_of_iterations=10, minimum_step_length=1e-3)
    levels = [(1, 0.0)]
    reg, o = run_gpu("mattes", fixed, moving, Bs, levels, RANDOM, 0.2, opt, moving_initial=A)
    C0 = CompositeTransform()
    C0.AddTransform(A)
    C0.AddTransform(Bo)
    p, res = run_oracle("mattes", fixed, moving, C0, levels, [reg.GetMetricSamplePoints(0)], opt)
    Bo.SetParameters(p)
    C = CompositeTransform()
    C.AddTransform(A)
    C.AddTransform(Bs)
    rms = displacement_rms(fixed, C, C0)
    assert rms <= 0.05, f"displacement RMS {rms:.4f} voxel"
    assert np.max(np.abs(Bs.GetParameters())) > 0.1  # it moved


def other_metric_registration(m, fixed, moving, U, levels, pct, iterations, seed=5):
    o = RegularStepGradientDescentOptimizerv4()
    o.SetLearningRate(0.5)
    o.SetNumberOfIterations(iterations)
    o.SetMinimumStepLength(1e-3)
    o.SetScales(AFFINE_SCALES)
    reg = ImageRegistrationMethodv4()
    reg.SetFixedImage(fixed)
    reg.SetMovingImage(moving)
    reg.SetMetric(m)
    reg.SetOptimizer(o)
    reg.SetInitialTransform(U)
    reg.SetNumberOfLevels(len(levels))
    reg.SetShrinkFactorsPerLevel([lv[0] for lv in levels])
    reg.SetSmoothingSigmasPerLevel([lv[1] for lv in levels])
    reg.SetMetricSamplingStrategy(RANDOM)
    reg.SetMetricSamplingPercentage(pct)
    reg.MetricSamplingReinitializeSeed(seed)
    reg.Update()
    return reg, o


def test_correlation_registration_recovers_the_transform(pair_mono):
    """CorrelationImageToImageMetricv4 drives ImageRegistrationMethodv4 and the device
    optimizer from the identity to the generating transform's inverse (moving(y) =
    fixed(T(y)))."""
    from itk_gb300 import AffineTransform, CorrelationImageToImageMetricv4
    fixed, moving, T = pair_mono
    truth = AffineTransform()
    truth.SetCenter(T.GetCenter())
    Minv = np.linalg.inv(T.GetMatrix())
    truth.SetMatrix(Minv)
    truth.SetTranslation(-Minv @ T.GetTranslation())
    U = perturbed(T, 23, scale=0.01, trans=1.5)
    start = displacement_rms(fixed, U, truth)
    other_metric_registration(CorrelationImageToImageMetricv4(), fixed, moving, U, [(2, 1.0), (1, 0.0)], 0.3, 100)
    end = displacement_rms(fixed, U, truth)
    assert end < 0.5 * start and end < 0.6, f"displacement RMS to the truth {start:.3f} -> {end:.3f} voxel"


def test_jhmi_registration_matches_oracle_loop(pair_mono):
    """JointHistogram MI through ImageRegistrationMethodv4 and the device optimizer against
    the oracle's RegularStep restatement on the oracle metric with the same points."""
    from itk_gb300 import JointHistogramMutualInformationImageToImageMetricv4
    from cases import oracle_transform
    from oracle import oracle as O
    fixed, moving, T = pair_mono
    U = perturbed(T, 24, scale=0.01, trans=1.0)
    U0 = perturbed(T, 24, scale=0.01, trans=1.0)
    reg, o = other_metric_registration(JointHistogramMutualInformationImageToImageMetricv4(), fixed, moving, U,
                                       [(1, 0.0)], 0.3, 30)
    pts = reg.GetMetricSamplePoints(0)
    g = O.gradient_recursive_gaussian(moving.array, moving.spacing, moving.direction, float(max(moving.spacing)))

    def evaluate(p):
        U0.SetParameters(p)
        rc, v, d, _, _ = O.joint_histogram_mi(fixed.array, geom(fixed), moving.array, geom(moving),
                                              oracle_transform(U0), moving_grad=g, points=pts)
        return rc, v, d

    h = R.regular_step(evaluate, U0.GetParameters().copy(), learning_rate=0.5, minimum_step_length=1e-3,
                       number_of_iterations=30, scales=AFFINE_SCALES)
    U0.SetParameters(h["params"])
    rms = displacement_rms(fixed, U, U0)
    assert rms <= 0.05, f"displacement RMS {rms:.4f} voxel"


def test_scales_estimator_in_the_registration_method(pair_mono):
    """A RegistrationParameterScalesFromPhysicalShift on the optimizer sets its scales at
    every level (the level's shrunk virtual grid); the run equals one with those scales
    given by hand."""
    from itk_gb300 import RegistrationParameterScalesFromPhysicalShift
    fixed, moving, T = pair_mono
    U1 = perturbed(T, 25, scale=0.01, trans=1.0)
    U2 = perturbed(T, 25, scale=0.01, trans=1.0)
    m1 = MeanSquaresImageToImageMetricv4()
    est = RegistrationParameterScalesFromPhysicalShift()
    est.SetMetric(m1)
    opt = dict(learning_rate=0.5, number_of_iterations=20, minimum_step_length=1e-3, scales=None)
    o1 = RegularStepGradientDescentOptimizerv4()
    o1.SetScalesEstimator(est)
    reg1 = ImageRegistrationMethodv4()
    reg1.SetFixedImage(fixed)
    reg1.SetMovingImage(moving)
    reg1.SetMetric(m1)
    reg1.SetOptimizer(o1)
    reg1.SetInitialTransform(U1)
    o1.SetLearningRate(0.5)
    o1.SetNumberOfIterations(20)
    o1.SetMinimumStepLength(1e-3)
    reg1.Update()
    scales = o1.GetScales()
    assert scales is not None and scales[9] == pytest.approx(1.0) and scales[0] > 1.0
    opt["scales"] = scales
    reg2, o2 = run_gpu("msq", fixed, moving, U2, [(1, 0.0)], NONE, 1.0, opt)
    assert np.array_equal(U1.GetParameters(), U2.GetParameters())
