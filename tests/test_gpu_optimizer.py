"""The device RegularStepGradientDescentOptimizerv4 loop.

(1) Against the same loop driven from the host: every iteration one
    GetValueAndDerivative through the C ABI and the oracle's restatement of
    AdvanceOneStep (sequential Kahan sums, FP64).  Both see bitwise-equal
    metric evaluations at equal parameters, so they agree to the last bits of
    ||g|| and g . g_prev (a fixed two-sum tree on the device, a sequential Kahan
    loop on the host): same stop condition and iteration count, parameters
    within 1e-9 of their scale.
(2) The stop conditions and return-best semantics of the reference
    (itkRegularStepGradientDescentOptimizerv4.hxx:78-171,
    itkGradientDescentOptimizerv4.hxx:59-169), with the loop run well past the
    stop so the halted iterations enqueued ahead are shown to be no-ops.
(3) CUDA-graph and direct launches give bitwise-equal results.
"""
import sys

import numpy as np
import pytest

from cases import perturbed, small_pair
from itk_gb300 import (AffineTransform, CompositeTransform, ExceptionObject,
                       MattesMutualInformationImageToImageMetricv4, MeanSquaresImageToImageMetricv4,
                       RegularStepGradientDescentOptimizerv4, data)
from itk_gb300 import _capi
from oracle import registration as R

pytestmark = pytest.mark.gpu

AFFINE_SCALES = np.array([1.0] * 9 + [1.0 / 50.0] * 3)


@pytest.fixture(scope="module")
def pair():
    return small_pair((40, 36, 32), config=1, multimodal=True)


def start_transform(T, seed=3):
    U = perturbed(T, seed, scale=0.03, trans=2.0)
    return U


def make_metric(kind, fixed, moving, transform, points=None, bins=32):
    m = MeanSquaresImageToImageMetricv4() if kind == "msq" else MattesMutualInformationImageToImageMetricv4()
    m.SetFixedImage(fixed)
    m.SetMovingImage(moving)
    m.SetMovingTransform(transform)
    if kind == "mattes":
        m.SetNumberOfHistogramBins(bins)
    if points is not None:
        m.SetVirtualSampledPointSet(points)
        m.SetUseSampledPointSet(True)
    m.Initialize()
    return m


def make_optimizer(m, lr=0.5, iters=30, min_step=1e-3, tol=1e-8, relax=0.5, scales=None, best=False, graphs=True):
    o = RegularStepGradientDescentOptimizerv4()
    o.SetMetric(m)
    o.SetLearningRate(lr)
    o.SetNumberOfIterations(iters)
    o.SetMinimumStepLength(min_step)
    o.SetGradientMagnitudeTolerance(tol)
    o.SetRelaxationFactor(relax)
    o.SetScales(scales)
    o.SetReturnBestParametersAndValue(best)
    o.SetUseCudaGraphs(graphs)
    return o


def host_loop(m, kind, p0, lr=0.5, iters=30, min_step=1e-3, tol=1e-8, relax=0.5, scales=None, best=False):
    """The reference's loop with the GPU metric as the cost function, stepped on the host."""
    T = m.GetMovingTransform()

    def evaluate(p):
        T.SetParameters(p)
        try:
            v, d = m.GetValueAndDerivative()
            return 0, v, d
        except ExceptionObject as e:
            return e.code, 0.0, np.zeros(len(p))

    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        r = R.regular_step(evaluate, p0, learning_rate=lr, relaxation_factor=relax, minimum_step_length=min_step,
                           gradient_magnitude_tolerance=tol, number_of_iterations=iters, return_best=best,
                           scales=scales, mean_squares=(kind == "msq"))
    T.SetParameters(p0)
    return r


def run_both(kind, fixed, moving, U, points=None, **kw):
    p0 = U.GetParameters().copy()
    m = make_metric(kind, fixed, moving, U, points)
    h = host_loop(m, kind, p0, **kw)
    U.SetParameters(p0)
    o = make_optimizer(m, **kw)
    o.StartOptimization()
    return o, U.GetParameters().copy(), h


def assert_params_close(got, want, rtol=1e-9):
    scale = max(np.max(np.abs(want)), 1.0)
    err = np.max(np.abs(got - want)) / scale
    assert err <= rtol, f"params differ by {err:.3e} of their scale\n got {got}\n want {want}"


@pytest.mark.parametrize("kind,sampled", [("msq", False), ("mattes", True), ("mattes", False)])
def test_device_loop_matches_host_loop_affine(pair, kind, sampled):
    fixed, moving, T = pair
    pts = data.random_points(fixed, 0.3, seed=11) if sampled else None
    U = start_transform(T)
    o, p, h = run_both(kind, fixed, moving, U, pts, scales=AFFINE_SCALES, iters=25)
    assert o.GetStopCondition() == h["stop"]
    assert o.GetCurrentIteration() == h["iterations"]
    assert_params_close(p, h["params"])
    assert o.GetValue() == pytest.approx(h["value"], rel=1e-12)
    assert o.GetCurrentLearningRateRelaxation() == h["relaxation"]
    assert o.GetCurrentStepLength() == h["step_length"]


def test_device_loop_relaxes_and_stops_on_small_step(pair):
    """Long enough for direction changes to halve the step until STEP_TOO_SMALL."""
    fixed, moving, T = pair
    U = start_transform(T, seed=5)
    o, p, h = run_both("msq", fixed, moving, U, scales=AFFINE_SCALES, lr=1.0, iters=200, min_step=0.05)
    assert h["stop"] == R.STOP_STEP_TOO_SMALL
    assert o.GetStopCondition() == _capi.GB_STOP_STEP_TOO_SMALL
    assert o.GetCurrentIteration() == h["iterations"] < 200
    assert o.GetCurrentLearningRateRelaxation() == h["relaxation"] < 0.1
    assert_params_close(p, h["params"], rtol=1e-7)
    assert "Step too small after" in o.GetStopConditionDescription()


def test_device_loop_matches_host_loop_bspline():
    fixed, moving, A, B = data.pair_bspline((40, 36, 32), (4, 4, 4), instance=2, multimodal_map=True)
    Bs = data.bspline_over_image(fixed, (4, 4, 4))
    C = CompositeTransform()
    C.AddTransform(A)
    C.AddTransform(Bs)
    pts = data.random_points(fixed, 0.25, seed=4)
    o, p, h = run_both("mattes", fixed, moving, C, pts, lr=1.0, iters=12, min_step=1e-3)
    assert o.GetStopCondition() == h["stop"]
    assert o.GetCurrentIteration() == h["iterations"]
    assert_params_close(p, h["params"], rtol=1e-8)


@pytest.mark.parametrize("best", [False, True])
def test_gradient_tolerance_stop(pair, best):
    fixed, moving, T = pair
    U = start_transform(T)
    p0 = U.GetParameters().copy()
    m = make_metric("msq", fixed, moving, U)
    o = make_optimizer(m, tol=1e30, iters=50, best=best)
    o.StartOptimization()
    assert o.GetStopCondition() == _capi.GB_STOP_GRADIENT_MAGNITUDE_TOLERANCE
    assert o.GetCurrentIteration() == 1  # counted, as the reference increments after AdvanceOneStep returns
    assert np.array_equal(U.GetParameters(), p0)
    v0 = m.GetValue()
    assert o.GetValue() == (sys.float_info.max if best else v0)
    assert "Gradient magnitude tolerance met after 0 iterations" in o.GetStopConditionDescription()


def test_step_too_small_at_first_iteration(pair):
    fixed, moving, T = pair
    U = start_transform(T)
    p0 = U.GetParameters().copy()
    m = make_metric("mattes", fixed, moving, U)
    o = make_optimizer(m, lr=1e-3, min_step=1e-2, iters=40)
    o.StartOptimization()
    assert o.GetStopCondition() == _capi.GB_STOP_STEP_TOO_SMALL
    assert o.GetCurrentIteration() == 1
    assert np.array_equal(U.GetParameters(), p0)


def test_zero_iterations(pair):
    fixed, moving, T = pair
    U = start_transform(T)
    p0 = U.GetParameters().copy()
    m = make_metric("msq", fixed, moving, U)
    for best in (False, True):
        o = make_optimizer(m, iters=0, best=best)
        o.StartOptimization()
        assert o.GetStopCondition() == _capi.GB_STOP_MAXIMUM_NUMBER_OF_ITERATIONS
        assert o.GetCurrentIteration() == 0
        assert np.array_equal(U.GetParameters(), p0)
        if best:
            assert o.GetValue() == sys.float_info.max


@pytest.mark.parametrize("kind", ["msq", "mattes"])
def test_return_best_matches_host_loop(pair, kind):
    """A large learning rate overshoots, so the best position is not the last one."""
    fixed, moving, T = pair
    U = start_transform(T, seed=8)
    o, p, h = run_both(kind, fixed, moving, U, scales=AFFINE_SCALES, lr=4.0, iters=15, min_step=1e-6, best=True)
    assert o.GetStopCondition() == h["stop"] == R.STOP_MAXIMUM_NUMBER_OF_ITERATIONS
    assert_params_close(p, h["params"], rtol=1e-7)
    assert o.GetValue() == pytest.approx(h["value"], rel=1e-9)


def test_no_overlap(pair):
    """Moving image far away: Mattes throws (COSTFUNCTION_ERROR, exception passed on);
    MeanSquares warns, returns DBL_MAX and a zero derivative, and the zero gradient
    stops the loop on the gradient tolerance."""
    fixed, moving, T = pair
    far = AffineTransform()
    far.SetCenter(T.GetCenter())
    far.SetTranslation([1e4, 0.0, 0.0])
    p0 = far.GetParameters().copy()
    m = make_metric("mattes", fixed, moving, far)
    o = make_optimizer(m, iters=20, best=True)
    with pytest.raises(ExceptionObject) as e:
        o.StartOptimization()
    assert e.value.code == _capi.GB_ERR_NO_VALID_POINTS
    assert o.GetStopCondition() == _capi.GB_STOP_COSTFUNCTION_ERROR
    assert o.GetCurrentIteration() == 0
    assert np.array_equal(far.GetParameters(), p0)
    far.SetParameters(p0)
    m = make_metric("msq", fixed, moving, far)
    o = make_optimizer(m, iters=20, tol=1e-4)
    o.StartOptimization()
    assert o.GetStopCondition() == _capi.GB_STOP_GRADIENT_MAGNITUDE_TOLERANCE
    assert o.GetValue() == sys.float_info.max
    assert np.array_equal(far.GetParameters(), p0)


@pytest.mark.parametrize("kind", ["msq", "mattes"])
def test_graphs_and_direct_launches_agree(pair, kind):
    fixed, moving, T = pair
    res = []
    for graphs in (True, False):
        U = start_transform(T)
        m = make_metric(kind, fixed, moving, U)
        o = make_optimizer(m, scales=AFFINE_SCALES, iters=20, graphs=graphs)
        o.StartOptimization()
        res.append((U.GetParameters().copy(), o.GetValue(), o.GetCurrentIteration(), o.GetStopCondition()))
    assert np.array_equal(res[0][0], res[1][0])
    assert res[0][1:] == res[1][1:]


def test_metric_evaluations_after_the_loop(pair):
    """After StartOptimization the handle evaluates normally (no stale stop flag) at the final position."""
    fixed, moving, T = pair
    U = start_transform(T)
    m = make_metric("mattes", fixed, moving, U)
    o = make_optimizer(m, iters=3, tol=1e30)
    o.StartOptimization()
    v, d = m.GetValueAndDerivative()
    m2 = make_metric("mattes", fixed, moving, U)
    v2, d2 = m2.GetValueAndDerivative()
    assert v == v2 and np.array_equal(d, d2)
    assert np.all(np.isfinite(d)) and np.any(d != 0)


def test_bad_settings(pair):
    fixed, moving, T = pair
    U = start_transform(T)
    m = make_metric("msq", fixed, moving, U)
    for kw in (dict(relax=1.0), dict(relax=-0.1), dict(tol=-1.0)):
        with pytest.raises(ExceptionObject):
            make_optimizer(m, **kw).StartOptimization()
    o = make_optimizer(m, scales=np.ones(5))
    with pytest.raises(ExceptionObject):
        o.StartOptimization()
    o = make_optimizer(m, scales=np.r_[np.ones(11), 0.0])
    with pytest.raises(ExceptionObject):
        o.StartOptimization()
