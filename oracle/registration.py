"""Oracle (test infrastructure): RegularStepGradientDescentOptimizerv4 and the
per-level loop of ImageRegistrationMethodv4, restated in plain Python on top of
the FP64 oracle metrics.  Used by the tests as the checker of the device
optimizer; never by the library.

Reference semantics (paths relative to ITK's Modules/):
  RegularStep StartOptimization / AdvanceOneStep
      Numerics/Optimizersv4/include/itkRegularStepGradientDescentOptimizerv4.hxx:39-229
  ResumeOptimization loop, StopOptimization with return-best
      Numerics/Optimizersv4/include/itkGradientDescentOptimizerv4.hxx:59-169
  scales check and identity test
      Numerics/Optimizersv4/src/itkObjectToObjectOptimizerBase.cxx:102-142
  CompensatedSummation (Kahan; GetSum returns the running sum)
      Core/Common/include/itkCompensatedSummation.hxx:38-48
  Transform::UpdateTransformParameters
      Core/Transform/include/itkTransform.hxx:69-121
  per-level set-up: smoothing, virtual-domain shrink, the metric's gradient filter
      Registration/RegistrationMethodsv4/include/itkImageRegistrationMethodv4.hxx:262-717
"""
from __future__ import annotations

import math
import sys

import numpy as np

from . import oracle as O

STOP_MAXIMUM_NUMBER_OF_ITERATIONS = 0
STOP_COSTFUNCTION_ERROR = 1
STOP_STEP_TOO_SMALL = 3
STOP_GRADIENT_MAGNITUDE_TOLERANCE = 5

DBL_MAX = sys.float_info.max
NO_VALID_POINTS = 2


class Kahan:
    """CompensatedSummation<double>: AddElement as itkCompensatedSummation.hxx:38-48."""

    def __init__(self):
        self.sum = 0.0
        self.comp = 0.0

    def add(self, x):
        y = x - self.comp
        t = self.sum + y
        self.comp = (t - self.sum) - y
        self.sum = t


def regular_step(evaluate, params0, learning_rate=1.0, relaxation_factor=0.5, minimum_step_length=1e-4,
                 gradient_magnitude_tolerance=1e-4, number_of_iterations=100, return_best=False, scales=None,
                 mean_squares=False, trace=None):
    """StartOptimization + ResumeOptimization of RegularStepGradientDescentOptimizerv4.

    evaluate(params) -> (status, value, derivative) is GetValueAndDerivative at params;
    a nonzero status is the metric throwing, except MeanSquares' no-valid-points,
    which is a warning with value DBL_MAX and a zero derivative.  trace: a list that
    receives (value, params before the step) per evaluated iteration.
    Returns dict(params, stop, iterations, value, step_length, grad_mag, relaxation, status)."""
    P = len(params0)
    params = np.array(params0, dtype=np.float64)
    inv = [1.0] * P
    if scales is not None:
        if len(scales) != P:
            raise ValueError("scales size must equal the number of parameters")
        if any(not (s > np.finfo(np.float64).eps) for s in scales):
            raise ValueError("m_Scales values must be > epsilon.")
        if any(abs(1.0 - s) > 0.01 for s in scales):
            inv = [1.0 / float(s) for s in scales]
    relax = 1.0
    it = 0
    grad = [0.0] * P
    best = params.copy()
    best_value = DBL_MAX
    value = 0.0
    out = dict(stop=None, step_length=0.0, grad_mag=0.0, status=0)

    def stop_opt(cond):
        nonlocal params, value
        out["stop"] = cond
        if return_best:
            params = best.copy()
            value = best_value

    while True:
        if it >= number_of_iterations:
            stop_opt(STOP_MAXIMUM_NUMBER_OF_ITERATIONS)
            break
        prev = grad
        status, value, d = evaluate(params.copy())
        if trace is not None:
            trace.append((value, params.copy()))
        if status != 0 and not (mean_squares and status == NO_VALID_POINTS):
            out["status"] = status
            stop_opt(STOP_COSTFUNCTION_ERROR)
            break
        # AdvanceOneStep
        g = [float(d[j]) * inv[j] for j in range(P)]
        prev = [prev[j] * inv[j] for j in range(P)]
        k = Kahan()
        for x in g:
            k.add(x * x)
        mag = math.sqrt(k.sum)
        out["grad_mag"] = mag
        stopped = False
        if mag < gradient_magnitude_tolerance:
            stop_opt(STOP_GRADIENT_MAGNITUDE_TOLERANCE)
            stopped = True
        else:
            k = Kahan()
            for j in range(P):
                k.add(g[j] * prev[j])
            if k.sum < 0:
                relax *= relaxation_factor
            step = relax * learning_rate
            out["step_length"] = step
            if step < minimum_step_length:
                stop_opt(STOP_STEP_TOO_SMALL)
                stopped = True
            else:
                g = [(x * relax) * learning_rate for x in g]
                factor = 1.0 / mag
                if factor == 1.0:
                    params = np.array([params[j] + g[j] for j in range(P)])
                else:
                    params = np.array([params[j] + g[j] * factor for j in range(P)])
        grad = g
        if return_best and value < best_value:
            best_value = value
            best = params.copy()
        it += 1
        if stopped:
            break
    out.update(params=params, iterations=it, value=value, relaxation=relax)
    return out


def level_inputs(fixed, fgeom, moving, mgeom, shrink=(1, 1, 1), sigma=0.0, sigma_physical=True):
    """One level of ImageRegistrationMethodv4 (itkImageRegistrationMethodv4.hxx:444-632):
    both images smoothed at full resolution (sigma in physical units or voxels,
    none when sigma is 0), the virtual domain the fixed geometry shrunk by the
    level's factors, and the metric's default moving-gradient filter on the
    smoothed moving image (sigma = its largest spacing).
    Returns (fixed_s, moving_s, moving_gradient, virtual_geometry)."""
    if sigma > 0:
        sf = sigma * (np.ones(3) if sigma_physical else np.asarray(fgeom.spacing))
        sm = sigma * (np.ones(3) if sigma_physical else np.asarray(mgeom.spacing))
        fs = O.smooth_recursive_gaussian(fixed, fgeom.spacing, sf)
        ms = O.smooth_recursive_gaussian(moving, mgeom.spacing, sm)
    else:
        fs, ms = fixed, moving
    g = O.gradient_recursive_gaussian(ms, mgeom.spacing, np.asarray(mgeom.direction).reshape(3, 3),
                                      float(max(mgeom.spacing)))
    size, sp, org = O.shrink_geometry(fgeom.size, fgeom.spacing, fgeom.origin,
                                      np.asarray(fgeom.direction).reshape(3, 3), shrink)
    vgeom = O.Geometry(tuple(int(s) for s in size), tuple(sp), tuple(org), tuple(fgeom.direction))
    return fs, ms, g, vgeom


def metric_evaluator(kind, fixed, fgeom, moving, mgeom, transform_kind, transform_fixed, moving_grad, vgeom,
                     points=None, bins=50):
    """evaluate(params) -> (status, value, derivative) of the oracle metric for one level."""
    tf = np.asarray(transform_fixed, np.float64)

    def evaluate(params):
        T = O.Transform(transform_kind, np.asarray(params, np.float64), tf)
        if kind == "msq":
            rc, v, d, _ = O.mean_squares(fixed, fgeom, moving, mgeom, T, moving_grad=moving_grad, points=points,
                                         virtual_geom=vgeom)
        else:
            rc, v, d, _, _, _ = O.mattes(fixed, fgeom, moving, mgeom, T, bins=bins, moving_grad=moving_grad,
                                         points=points, virtual_geom=vgeom)
        return rc, v, d

    return evaluate


def register(kind, fixed, fgeom, moving, mgeom, transform_kind, params0, transform_fixed, levels, optimizer,
             bins=50):
    """ImageRegistrationMethodv4::GenerateData over `levels`, each a dict with
    shrink, sigma, sigma_physical and points (virtual-space samples, or None for
    the dense shrunk domain); `optimizer` holds regular_step's keyword settings.
    Returns (final params, per-level optimizer results)."""
    params = np.array(params0, np.float64)
    results = []
    for lv in levels:
        fs, ms, g, vgeom = level_inputs(fixed, fgeom, moving, mgeom, lv.get("shrink", (1, 1, 1)),
                                        lv.get("sigma", 0.0), lv.get("sigma_physical", True))
        ev = metric_evaluator(kind, fs, fgeom, ms, mgeom, transform_kind, transform_fixed, g, vgeom,
                              points=lv.get("points"), bins=bins)
        r = regular_step(ev, params, mean_squares=(kind == "msq"), **optimizer)
        params = r["params"]
        results.append(r)
    return params, results
