"""The FP64 oracle pinned against the reference's own known answers (CPU only)."""
import json
import os

import numpy as np
import pytest

from cases import mattes_2d_case, mattes_2d_sample_points, run_oracle
from itk_gb300.image import GradientImage, Image
from itk_gb300.transforms import AffineTransform
from oracle import oracle as O

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_known_values.json")))


def _identity():
    t = AffineTransform()
    t.SetIdentity()
    return t


@pytest.mark.parametrize("sampled", [False, True])
def test_mattes_known_values_and_fd_ratio(sampled):
    """itkMattesMutualInformationImageToImageMetricv4Test.cxx:316-422 restated on the oracle with the
    test's Image<double,2> pixel semantics."""
    g = GOLDEN["mattes_2d_known_values"]
    fixed, moving = mattes_2d_case()
    pts = mattes_2d_sample_points(fixed) if sampled else None
    base = run_oracle("mattes", fixed, moving, _identity(), points=pts, pixel_double=True)
    assert base["status"] == 0
    vo = run_oracle("mattes", fixed, moving, _identity(), points=pts, pixel_double=True, compute_derivative=False)
    # GetValue equals GetValueAndDerivative to 8 ULP (.cxx:319)
    assert abs(vo["value"] - base["value"]) <= 8 * np.spacing(abs(base["value"]))
    delta = 1e-5
    tol = g["fd_ratio_tolerance_sampled"] if sampled else g["fd_ratio_tolerance_dense"]
    # the 2-D affine parameters inside the 3-D layout: m00 m01 m10 m11 t0 t1
    for k3 in (0, 1, 3, 4, 9, 10):
        vals = []
        for h in (delta, -delta, 2 * delta, -2 * delta):
            t = _identity()
            p = t.GetParameters()
            p[k3] += h
            t.SetParameters(p)
            vals.append(run_oracle("mattes", fixed, moving, t, points=pts, pixel_double=True,
                                   compute_derivative=False)["value"])
        for v, known in zip(vals, g["values"]):
            assert abs(abs(v / known) - 1.0) <= g["value_tolerance"]
        m1p, m1m, m2p, m2m = vals
        fd = -1.0 * ((-1 / 12) * m2p + (1 / 12) * m2m + (2 / 3) * m1p - (2 / 3) * m1m) / delta
        ratio = base["derivative"][k3] / fd
        assert abs(ratio - 1.0) <= tol, (k3, ratio)
    if not sampled:
        # dense: the oracle reproduces the known value far inside the 5 % window
        assert abs(base["value"] / g["values"][0] - 1.0) < 1e-5


def test_mattes_known_values_float_pixels():
    """Same images as Image<float,3> one voxel thick (the GPU's pixel type): value still matches."""
    g = GOLDEN["mattes_2d_known_values"]
    fixed, moving = mattes_2d_case()
    r = run_oracle("mattes", fixed, moving, _identity())
    assert r["status"] == 0 and r["nvalid"] == 10000
    assert abs(r["value"] / g["values"][0] - 1.0) < 1e-5


def test_mean_squares_closed_form():
    g = GOLDEN["mean_squares_5cube"]
    n = np.arange(1, 126, dtype=np.float64)
    fixed = Image((n * n).astype(np.float32).reshape(5, 5, 5))
    moving = Image((1.0 / (n * n)).astype(np.float32).reshape(5, 5, 5))
    grad = np.zeros((5, 5, 5, 3))
    r = run_oracle("msq", fixed, moving, _identity(), gradient=GradientImage(grad))
    assert r["status"] == 0 and r["nvalid"] == g["nvalid"]
    assert abs(r["value"] - g["value_float_pixels"]) <= 1e-13 * g["value_float_pixels"]
    rd = run_oracle("msq", fixed, moving, _identity(), gradient=GradientImage(grad), pixel_double=True)
    # double pixels: differences of float-stored 1/n^2, so only float-level agreement with exact rationals
    assert abs(rd["value"] - g["value_double_pixels"]) <= 1e-7 * g["value_double_pixels"]


def test_linear_interpolation_of_linear_function():
    """itkLinearInterpolateImageFunctionTest.cxx:100-205: 3x + y + z is reproduced exactly inside."""
    nx, ny, nz = 6, 5, 4
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    img = (3 * x + y + z).astype(np.float32)
    geo = O.Geometry((nx, ny, nz))
    rng = np.random.default_rng(0)
    pts = rng.uniform([0, 0, 0], [nx - 1, ny - 1, nz - 1], size=(500, 3))
    vals, inside = O.interpolate(img, geo, pts)
    assert inside.all()
    want = 3 * pts[:, 0] + pts[:, 1] + pts[:, 2]
    assert np.max(np.abs(vals - want)) <= GOLDEN["linear_interpolation"]["tolerance"]
    # buffer bounds are [-0.5, n - 0.5)
    _, ins = O.interpolate(img, geo, [[-0.5, 0, 0], [-0.5000001, 0, 0], [nx - 0.5, 0, 0], [nx - 0.5000001, 0, 0]])
    assert list(ins) == [True, False, False, True]
    # beyond the last voxel the value is clamped to the edge voxel
    v, _ = O.interpolate(img, geo, [[nx - 0.75, 0, 0]])
    assert v[0] == pytest.approx(3 * (nx - 1))


def test_bspline_kernels():
    g = GOLDEN["bspline_kernel"]
    for u, want in g["values"].items():
        assert O.bspline3(float(u)) == pytest.approx(want, abs=1e-15)
        assert O.bspline3(-float(u)) == pytest.approx(want, abs=1e-15)
    for u, want in g["derivative"].items():
        assert O.bspline3_derivative(float(u)) == pytest.approx(want, abs=1e-15)
    # partition of unity of the 64 tensor weights (BSplineInterpolationWeightFunction)
    w, start = O.bspline_weights([3.3, 4.7, 2.01])
    assert list(start) == [2, 3, 1]
    assert w.sum() == pytest.approx(1.0, abs=1e-14)


def test_oracle_work_unit_invariance():
    """itkImageToImageMetricv4Test.cxx:313-380 checks results across work-unit counts to 1e-10."""
    from cases import small_pair, perturbed
    from itk_gb300 import data
    fixed, moving, T = small_pair()
    grad = data.gradient_image(moving)
    U = perturbed(T, 3)
    for kind in ("msq", "mattes"):
        a = run_oracle(kind, fixed, moving, U, gradient=grad, nthreads=1)
        b = run_oracle(kind, fixed, moving, U, gradient=grad, nthreads=7)
        assert a["status"] == b["status"] == 0
        assert a["nvalid"] == b["nvalid"]
        assert abs(a["value"] - b["value"]) <= 1e-10 * abs(a["value"])
        assert np.max(np.abs(a["derivative"] - b["derivative"])) <= 1e-10 * np.max(np.abs(a["derivative"]))


def test_mattes_constant_images_raise():
    """itkMattesMutualInformationImageToImageMetricv4Test.cxx:452-544 (constant fixed / moving)."""
    n = 20
    varying = Image(np.arange(n * n, dtype=np.float32).reshape(1, n, n))
    const = Image(np.zeros((1, n, n), np.float32))
    r = run_oracle("mattes", const, varying, _identity())
    assert r["status"] == 4  # FIXED_CONSTANT
    r = run_oracle("mattes", varying, const, _identity())
    assert r["status"] == 5  # MOVING_CONSTANT


def test_no_overlap():
    fixed, moving = mattes_2d_case(30)
    t = _identity()
    t.SetTranslation([1e4, 0, 0])
    r = run_oracle("msq", fixed, moving, t, gradient=GradientImage(np.zeros((1, 30, 30, 3))))
    assert r["status"] == 2 and r["nvalid"] == 0 and r["value"] == np.finfo(np.float64).max
    assert not np.any(r["derivative"])
    r = run_oracle("mattes", fixed, moving, t)
    assert r["status"] == 2
