"""RegistrationParameterScalesFromPhysicalShift (host code, no GPU), on the reference
test's expectations (Numerics/Optimizersv4/test/itkRegistrationParameterScalesFromPhysicalShiftTest.cxx:160-340):
affine scales upper[c]^2 for the matrix entries of column c and 1 for the
translation, non-uniform; the step scale of an identity-sized step |upper|; a
displacement field's local scales 1; and the optimizer taking the estimate."""
import numpy as np
import pytest

from itk_gb300 import (AffineTransform, DisplacementFieldImage, DisplacementFieldTransform, Image,
                       RegistrationParameterScalesFromPhysicalShift, data)


class _Metric:
    """The metric state the estimator reads: the virtual domain and the moving transform."""

    def __init__(self, fixed, T, shrink=(1, 1, 1)):
        self._fixed, self._virtual, self._level_shrink, self._T = fixed, None, shrink, T

    def GetMovingTransform(self):
        return self._T


@pytest.fixture
def image():
    return Image(np.zeros((30, 40, 50), np.float32), spacing=(1.0, 1.0, 1.0))


def test_affine_scales(image):
    T = AffineTransform()
    est = RegistrationParameterScalesFromPhysicalShift()
    est.SetMetric(_Metric(image, T))
    s = est.EstimateScales()
    upper = np.asarray(image.GetSize(), np.float64) - 1.0
    want = np.concatenate([np.tile(upper ** 2, 3), np.ones(3)])
    np.testing.assert_allclose(s, want, rtol=0.01)
    assert not np.all(s == s[0])
    assert np.array_equal(T.GetParameters(), AffineTransform().GetParameters())  # parameters restored


def test_step_scale(image):
    T = AffineTransform()
    est = RegistrationParameterScalesFromPhysicalShift()
    est.SetMetric(_Metric(image, T))
    step = T.GetParameters()  # an identity-sized step
    upper = np.asarray(image.GetSize(), np.float64) - 1.0
    assert est.EstimateStepScale(step) == pytest.approx(np.sqrt(np.sum(upper ** 2)), rel=0.01)


def test_displacement_field_local_scales():
    img = Image(np.zeros((12, 11, 10), np.float32))
    T = DisplacementFieldTransform()
    T.SetDisplacementField(DisplacementFieldImage.like(img))
    est = RegistrationParameterScalesFromPhysicalShift()
    est.SetMetric(_Metric(img, T))
    np.testing.assert_allclose(est.EstimateScales(), np.ones(3), rtol=0.01)


def test_bspline_scales_are_uniform(image):
    B = data.bspline_over_image(image, (1, 1, 1))
    est = RegistrationParameterScalesFromPhysicalShift()
    est.SetMetric(_Metric(image, B))
    s = est.EstimateScales()
    assert s.size == B.GetNumberOfParameters() and np.all(s == s[0]) and s[0] > 0


def test_shrunk_level_uses_the_shrunk_grid(image):
    T = AffineTransform()
    est = RegistrationParameterScalesFromPhysicalShift()
    est.SetMetric(_Metric(image, T, shrink=(2, 2, 2)))
    s = est.EstimateScales()
    from itk_gb300 import shrink_geometry
    size, spacing, origin = shrink_geometry(image, (2, 2, 2))
    upper = origin + (np.asarray(size) - 1) * spacing
    np.testing.assert_allclose(s[:3], upper ** 2, rtol=1e-9)
