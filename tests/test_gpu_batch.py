"""The batched engine: many affine registrations, one launch per phase per iteration.

(1) A registration's result is bitwise the same alone and in a mix (its blocks
    and reduction orders depend only on its own sample count), with graphs or
    direct launches, and when the run is split into several calls.
(2) Against the single-registration device loop, which partitions the samples
    differently (metric sums equal to FP32 rounding): same stop condition and
    iteration count, parameters within 1e-5 of their scale.
(3) Registrations stop independently: an early stop, a metric error in one of
    them, zero iterations.
"""
import numpy as np
import pytest

from cases import perturbed, small_pair
from itk_gb300 import (AffineTransform, ExceptionObject, MattesMutualInformationImageToImageMetricv4,
                       MeanSquaresImageToImageMetricv4, RegistrationBatch, RegularStepGradientDescentOptimizerv4,
                       data)
from itk_gb300 import _capi

pytestmark = pytest.mark.gpu

SCALES = np.array([1.0] * 9 + [1.0 / 50.0] * 3)
SIZES = [(40, 36, 32), (33, 29, 41), (48, 44, 40), (28, 30, 26)]


@pytest.fixture(scope="module")
def pairs():
    out = []
    for i, size in enumerate(SIZES):
        out.append(small_pair(size, config=1, multimodal=(i % 2 == 1), seed_shift=i))
    return out


def make(pairs, i, kind, sampled=False, iters=15, tol=1e-8, min_step=1e-6, lr=0.5, best=False):
    k = i % len(pairs)
    if kind == "msq" and k % 2 == 1:  # MeanSquares on the single-modality pairs (even indices)
        k -= 1
    fixed, moving, T = pairs[k]
    U = perturbed(T, 100 + i, scale=0.02, trans=1.5)
    m = MeanSquaresImageToImageMetricv4() if kind == "msq" else MattesMutualInformationImageToImageMetricv4()
    m.SetFixedImage(fixed)
    m.SetMovingImage(moving)
    m.SetMovingTransform(U)
    if kind == "mattes":
        m.SetNumberOfHistogramBins(32)
    if sampled:
        m.SetVirtualSampledPointSet(data.random_points(fixed, 0.3, seed=7 + i))
        m.SetUseSampledPointSet(True)
    m.Initialize()
    o = RegularStepGradientDescentOptimizerv4()
    o.SetMetric(m)
    o.SetLearningRate(lr)
    o.SetNumberOfIterations(iters)
    o.SetMinimumStepLength(min_step)
    o.SetGradientMagnitudeTolerance(tol)
    o.SetScales(SCALES)
    o.SetReturnBestParametersAndValue(best)
    return U, o


SPECS = [("msq", False), ("mattes", True), ("mattes", False), ("msq", True), ("mattes", True), ("msq", False)]


def result(U, o):
    return U.GetParameters().copy(), o.GetValue(), o.GetCurrentIteration(), o.GetStopCondition()


def run_batch(pairs, idx, spb=(4096, 4096, 4096), graphs=True, chunk=0, persistent=True, **kw):
    b = RegistrationBatch()
    b.SetSamplesPerBlock(*spb)
    b.SetUseCudaGraphs(graphs)
    b.SetPersistent(persistent)
    regs = [make(pairs, i, *SPECS[i], **kw) for i in idx]
    for U, o in regs:
        b.Add(o)
    if chunk:
        while b.Run(chunk):
            pass
    else:
        assert b.Run() == 0
    return [result(U, o) for U, o in regs]


def same(r1, r2):
    assert np.array_equal(r1[0], r2[0]), f"{r1[0]} vs {r2[0]}"
    assert r1[1:] == r2[1:]


def test_alone_equals_in_mix(pairs):
    mix = run_batch(pairs, range(6))
    for i in range(6):
        alone = run_batch(pairs, [i])[0]
        same(alone, mix[i])


def test_graphs_direct_and_split_runs_agree(pairs):
    a = run_batch(pairs, range(4))
    b = run_batch(pairs, range(4), graphs=False)
    c = run_batch(pairs, range(4), chunk=3)
    for x, y, z in zip(a, b, c):
        same(x, y)
        same(x, z)


def test_persistent_and_per_phase_forms_agree(pairs):
    """The persistent kernel (several iterations per launch, items ordered by
    dependency) and the per-phase launches (graph and direct) give the same bits, for
    the whole mix and with runs split into chunks of iterations."""
    a = run_batch(pairs, range(6), persistent=True)
    b = run_batch(pairs, range(6), persistent=False)
    c = run_batch(pairs, range(6), persistent=False, graphs=False)
    d = run_batch(pairs, range(6), persistent=True, chunk=5)
    for w, x, y, z in zip(a, b, c, d):
        same(w, x)
        same(w, y)
        same(w, z)


@pytest.mark.parametrize("i", range(6))
def test_batch_matches_single_loop(pairs, i):
    got = run_batch(pairs, range(6))[i]
    U, o = make(pairs, i, *SPECS[i])
    o.StartOptimization()
    want = result(U, o)
    assert got[2:] == want[2:]
    scale = max(np.max(np.abs(want[0])), 1.0)
    assert np.max(np.abs(got[0] - want[0])) <= 1e-5 * scale
    assert got[1] == pytest.approx(want[1], rel=1e-5)


def test_independent_stops(pairs):
    """One stops at once on the gradient tolerance, one on a small step, the rest run out
    of iterations; each equals its alone run."""
    b = RegistrationBatch()
    b.SetSamplesPerBlock(4096, 4096, 4096)
    regs = [make(pairs, 0, "msq", iters=12, tol=1e30), make(pairs, 1, "mattes", True, iters=40, min_step=0.3, lr=1.0),
            make(pairs, 2, "mattes", False, iters=9), make(pairs, 3, "msq", True, iters=20, best=True)]
    for U, o in regs:
        b.Add(o)
    assert b.Run() == 0
    got = [result(U, o) for U, o in regs]
    assert got[0][3] == _capi.GB_STOP_GRADIENT_MAGNITUDE_TOLERANCE and got[0][2] == 1
    assert got[1][3] == _capi.GB_STOP_STEP_TOO_SMALL
    assert got[2][3] == _capi.GB_STOP_MAXIMUM_NUMBER_OF_ITERATIONS and got[2][2] == 9
    assert got[3][3] == _capi.GB_STOP_MAXIMUM_NUMBER_OF_ITERATIONS and got[3][2] == 20
    specs = [dict(i=0, kind="msq", iters=12, tol=1e30), dict(i=1, kind="mattes", sampled=True, iters=40, min_step=0.3,
                                                            lr=1.0),
             dict(i=2, kind="mattes", sampled=False, iters=9), dict(i=3, kind="msq", sampled=True, iters=20, best=True)]
    for r, kw in zip(got, specs):
        b1 = RegistrationBatch()
        b1.SetSamplesPerBlock(4096, 4096, 4096)
        i = kw.pop("i")
        U, o = make(pairs, i, **kw)
        b1.Add(o)
        b1.Run()
        same(result(U, o), r)


def test_metric_error_stops_only_that_registration(pairs):
    fixed, moving, T = pairs[0]
    far = AffineTransform()
    far.SetCenter(T.GetCenter())
    far.SetTranslation([1e4, 0.0, 0.0])
    m = MattesMutualInformationImageToImageMetricv4()
    m.SetFixedImage(fixed)
    m.SetMovingImage(moving)
    m.SetMovingTransform(far)
    m.Initialize()
    bad = RegularStepGradientDescentOptimizerv4()
    bad.SetMetric(m)
    bad.SetNumberOfIterations(10)
    b = RegistrationBatch()
    b.SetSamplesPerBlock(4096, 4096, 4096)
    good = [make(pairs, i, *SPECS[i]) for i in range(3)]
    b.Add(good[0][1])
    b.Add(bad)
    for U, o in good[1:]:
        b.Add(o)
    assert b.Run() == 0
    assert bad.GetStopCondition() == _capi.GB_STOP_COSTFUNCTION_ERROR
    assert bad._batch_status == _capi.GB_ERR_NO_VALID_POINTS
    alone = run_batch(pairs, range(3))
    for (U, o), want in zip(good, alone):
        same(result(U, o), want)


def test_zero_iterations_and_reuse(pairs):
    b = RegistrationBatch()
    U, o = make(pairs, 0, "mattes", iters=0)
    p0 = U.GetParameters().copy()
    b.Add(o)
    assert b.Run() == 0
    assert o.GetStopCondition() == _capi.GB_STOP_MAXIMUM_NUMBER_OF_ITERATIONS and o.GetCurrentIteration() == 0
    assert np.array_equal(U.GetParameters(), p0)
    # the same metric again, now with iterations
    o.SetNumberOfIterations(5)
    b.Add(o)
    assert b.Run() == 0
    assert o.GetCurrentIteration() == 5


def test_autotune_keeps_results_deterministic(pairs):
    b = RegistrationBatch()
    regs = [make(pairs, i, *SPECS[i]) for i in range(4)]
    for U, o in regs:
        b.Add(o)
    spb = b.Autotune(iterations=2)
    assert all(s >= 2048 for s in spb) and b.GetSamplesPerBlock() == spb
    assert b.Run() == 0
    got = [result(U, o) for U, o in regs]
    again = run_batch(pairs, range(4), spb=spb)
    for x, y in zip(got, again):
        same(x, y)


def test_rejects_non_affine(pairs):
    fixed, moving, A, B = data.pair_bspline((32, 30, 28), (4, 4, 4), instance=0, multimodal_map=False)
    m = MeanSquaresImageToImageMetricv4()
    m.SetFixedImage(fixed)
    m.SetMovingImage(moving)
    m.SetMovingTransform(data.bspline_over_image(fixed, (4, 4, 4)))
    m.Initialize()
    o = RegularStepGradientDescentOptimizerv4()
    o.SetMetric(m)
    b = RegistrationBatch()
    with pytest.raises(ExceptionObject):
        b.Add(o)


def test_first_iteration_matches_oracle(pairs):
    """One iteration of every registration in a mixed batch (MeanSquares and Mattes MI,
    dense and sampled, four volume sizes) against the FP64 oracle at the start
    parameters: the value the batch reports, and the derivative recovered from its
    step p1 = p0 + lr (d / s) / ||d / s|| (with ||d / s|| the reported gradient
    magnitude), within 1e-5 and 1e-4."""
    from cases import geom, oracle_transform
    from conftest import MATTES_VALUE_ATOL, assert_deriv_close, assert_value_close
    from oracle import oracle as O

    lr = 0.5
    b = RegistrationBatch()
    b.SetSamplesPerBlock(4096, 4096, 4096)
    regs = []
    for i in range(len(SPECS)):
        U, o = make(pairs, i, *SPECS[i], iters=1, lr=lr)
        regs.append((i, U, o, U.GetParameters().copy()))
        b.Add(o)
    assert b.Run() == 0
    for i, U, o, p0 in regs:
        kind, sampled = SPECS[i]
        m = o.GetMetric()
        fixed, moving = m.GetFixedImage(), m.GetMovingImage()
        pts = data.random_points(fixed, 0.3, seed=7 + i) if sampled else None
        grad = O.gradient_recursive_gaussian(moving.array, moving.spacing, moving.direction,
                                             float(max(moving.spacing)))
        T0 = AffineTransform()
        T0.SetCenter(U.GetCenter())
        T0.SetParameters(p0)
        Tk = oracle_transform(T0)
        if kind == "msq":
            rc, v, d, nv = O.mean_squares(fixed.array, geom(fixed), moving.array, geom(moving), Tk,
                                          moving_grad=grad, points=pts)
        else:
            rc, v, d, nv, _, _ = O.mattes(fixed.array, geom(fixed), moving.array, geom(moving), Tk, bins=32,
                                          moving_grad=grad, points=pts)
        assert rc == 0
        assert o.GetCurrentIteration() == 1
        assert_value_close(o.GetValue(), v, atol=MATTES_VALUE_ATOL if kind == "mattes" else 0.0)
        d_batch = (U.GetParameters() - p0) * SCALES * (o.GetGradientMagnitude() / lr)
        assert_deriv_close(d_batch, d)
