"""UseFloatingPointCorrection in the oracle's MeanSquares (no GPU): each point's local
derivative truncated toward zero to 1 / resolution before it is summed
(Registration/Metricsv4/include/itkImageToImageMetricv4GetValueAndDerivativeThreaderBase.hxx:284-294).
So N * resolution * derivative is a sum of integers, and the corrected derivative
lies within 1 / resolution of the uncorrected one; the value is unchanged."""
import numpy as np
import pytest

from cases import geom, oracle_transform, perturbed, small_pair
from itk_gb300 import data
from oracle import oracle as O


@pytest.mark.parametrize("resolution", [10.0, 1e3, 1e6])
def test_truncated_sums(resolution):
    fixed, moving, T = small_pair((24, 22, 20), config=0)
    U = perturbed(T, 4)
    g = data.gradient_image(moving).array
    rc0, v0, d0, n0 = O.mean_squares(fixed.array, geom(fixed), moving.array, geom(moving), oracle_transform(U),
                                     moving_grad=g)
    rc1, v1, d1, n1 = O.mean_squares_fpc(fixed.array, geom(fixed), moving.array, geom(moving), oracle_transform(U),
                                         resolution, moving_grad=g)
    assert rc0 == rc1 == 0 and n0 == n1 and v0 == v1
    k = d1 * n1 * resolution
    np.testing.assert_allclose(k, np.round(k), rtol=0, atol=1e-6 * max(1.0, np.max(np.abs(k))))
    assert np.all(np.abs(d1 - d0) <= 1.0 / resolution + 1e-12 * np.abs(d0))
    if resolution == 10.0:
        assert np.any(d1 != d0)
