"""CPU checks of the oracle's B-spline and composite paths (test infrastructure).

* TransformPoint: the oracle's C restatement against the independent numpy
  BSplineTransform / CompositeTransform mirror, inside the valid region.
* Jacobian: the 64 cubic B-spline weights are a partition of unity, so for
  every sample in the valid region sum_n J(d, n + d * nper) = 1 and, through
  the composite's chain rule, the node derivatives of one dimension sum to
  M^T times the affine translation derivative.  The oracle must reproduce
  this identity for both metrics.
"""
import numpy as np
import pytest

from cases import geom, oracle_transform, run_oracle
from itk_gb300 import BSplineTransform, CompositeTransform, data
from oracle import oracle as O


@pytest.fixture(scope="module")
def bpair():
    fixed, moving, A, B = data.pair_bspline((30, 28, 24), (3, 3, 3), instance=5, multimodal_map=True)
    return fixed, moving, A, B, data.gradient_image(moving)


def test_transform_point_matches_numpy_mirror(bpair):
    fixed, moving, A, B, grad = bpair
    C = CompositeTransform()
    C.AddTransform(A)
    C.AddTransform(B)
    pts = data.random_points(fixed, 0.05, seed=3).astype(np.float64)
    for T in (B, C):
        got = O.transform_points(oracle_transform(T), pts)
        want = T.TransformPoint(pts)
        assert np.max(np.abs(got - want)) < 1e-9


@pytest.mark.parametrize("kind", ["msq", "mattes"])
def test_partition_of_unity_derivative(bpair, kind):
    fixed, moving, A, B, grad = bpair
    # a domain 1 mm wider than the image on every side: every sample inside the valid region
    Bz = BSplineTransform()
    size = np.asarray(fixed.GetSize(), np.float64)
    Bz.SetTransformDomain(fixed.origin - 1.0, fixed.spacing * (size - 1.0) + 2.0, (3, 3, 3))
    C = CompositeTransform()
    C.AddTransform(A)
    C.AddTransform(Bz)
    rc = run_oracle(kind, fixed, moving, C, gradient=grad, bins=32)
    ra = run_oracle(kind, fixed, moving, A, gradient=grad, bins=32)
    assert rc["status"] == 0 and ra["status"] == 0
    assert rc["nvalid"] == ra["nvalid"]
    assert rc["value"] == pytest.approx(ra["value"], rel=1e-12)
    nper = Bz.GetNumberOfParametersPerDimension()
    sums = rc["derivative"].reshape(3, nper).sum(axis=1)
    want = A.GetMatrix().T @ ra["derivative"][9:12]
    assert np.max(np.abs(sums - want)) <= 1e-10 * np.max(np.abs(want))


def test_outside_valid_region_is_identity():
    """Points outside the B-spline valid region map by the identity (itkBSplineTransform.hxx:519-523)."""
    T = BSplineTransform()
    T.SetTransformDomain((10.0, 10.0, 10.0), (8.0, 8.0, 8.0), (2, 2, 2))
    T.SetParameters(np.full(T.GetNumberOfParameters(), 3.0))
    pts = np.array([[0.0, 0.0, 0.0], [14.0, 14.0, 14.0], [30.0, 12.0, 12.0]])
    got = O.transform_points(oracle_transform(T), pts)
    assert np.array_equal(got[0], pts[0]) and np.array_equal(got[2], pts[2])
    assert np.allclose(got[1], pts[1] + 3.0)  # constant coefficients: constant displacement


def test_geometry_roundtrip(bpair):
    fixed = bpair[0]
    g = geom(fixed)
    assert g.size == tuple(int(s) for s in fixed.GetSize())
