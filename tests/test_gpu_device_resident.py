"""The device-resident evaluation (gb_metric_evaluate_device: parameters and results
in device memory, transform constants computed on the device) gives the same bits as
the host call GetValueAndDerivative / GetValue: both compute the constants with the
same non-contracting FP64 operations and run the same kernels."""
import numpy as np
import pytest

from cases import perturbed, small_pair
from itk_gb300 import (CompositeTransform, MattesMutualInformationImageToImageMetricv4,
                       MeanSquaresImageToImageMetricv4, data)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pair():
    fixed, moving, T = small_pair((48, 44, 40), config=1, multimodal=True)
    return fixed, moving, T, data.gradient_image(moving)


def transform_of(kind, fixed, T):
    if kind == "affine":
        return perturbed(T, 12)
    B = data.random_bspline_coefficients(data.bspline_over_image(fixed, (4, 4, 4)), 13, 1.0)
    C = CompositeTransform()
    C.AddTransform(T)
    C.AddTransform(B)
    return C


@pytest.mark.parametrize("metric", ["msq", "mattes"])
@pytest.mark.parametrize("transform", ["affine", "composite"])
@pytest.mark.parametrize("sampled", [False, True])
def test_device_resident_matches_host_call(pair, metric, transform, sampled):
    torch = pytest.importorskip("torch")
    fixed, moving, T, grad = pair
    U = transform_of(transform, fixed, T)
    m = MeanSquaresImageToImageMetricv4() if metric == "msq" else MattesMutualInformationImageToImageMetricv4()
    m.SetFixedImage(fixed)
    m.SetMovingImage(moving)
    m.SetMovingTransform(U)
    m.SetMovingImageGradientImage(grad)
    if sampled:
        m.SetVirtualSampledPointSet(data.random_points(fixed, 0.3, seed=14))
        m.SetUseSampledPointSet(True)
    m.Initialize()
    v, d = m.GetValueAndDerivative()
    v_only = m.GetValue()
    P = d.size
    dp = torch.tensor(U.GetParameters(), dtype=torch.float64, device="cuda")
    out = torch.full((2 + P,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    m.evaluate_device(dp.data_ptr(), out.data_ptr(), True)
    assert m.synchronize() == 0
    o = out.cpu().numpy()
    assert o[0] == v
    assert o[1] == m.GetNumberOfValidPoints()
    assert np.array_equal(o[2:], d)
    out.fill_(float("nan"))
    torch.cuda.synchronize()
    m.evaluate_device(dp.data_ptr(), out.data_ptr(), False)
    assert m.synchronize() == 0
    assert out[0].item() == v_only == v
