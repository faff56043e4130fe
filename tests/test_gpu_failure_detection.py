"""Failure detection on the device without a GPU fault.

Every wait of the kernels on an asynchronous copy is bounded.  With the
stalled-copy injection the affine Mattes derivative pass issues none of its
streamed record copies, so each of its mbarrier waits runs out after a short
limit: the kernel records GB_ERR_TIMEOUT and returns (nothing is in flight),
GetValueAndDerivative raises with that status, and the handle stays usable --
the next evaluation without the injection gives the same bits as before.
"""
import numpy as np
import pytest

from cases import perturbed, small_pair
from itk_gb300 import ExceptionObject, MattesMutualInformationImageToImageMetricv4, _capi, data

pytestmark = pytest.mark.gpu


def test_stalled_copy_times_out_and_handle_recovers():
    fixed, moving, T = small_pair((40, 36, 32), config=1, multimodal=True)
    m = MattesMutualInformationImageToImageMetricv4()
    m.SetFixedImage(fixed)
    m.SetMovingImage(moving)
    m.SetMovingTransform(perturbed(T, 3))
    m.SetMovingImageGradientImage(data.gradient_image(moving))
    m.SetVirtualSampledPointSet(data.random_points(fixed, 0.2, seed=4))
    m.SetUseSampledPointSet(True)
    m.Initialize()
    v0, d0 = m.GetValueAndDerivative()
    m.set_fault_injection(_capi.GB_FAULT_STALLED_COPY)
    for _ in range(2):
        with pytest.raises(ExceptionObject) as e:
            m.GetValueAndDerivative()
        assert e.value.code == _capi.GB_ERR_TIMEOUT
        assert "timed out" in str(e.value)
    # the value alone does not stream records: unaffected
    assert m.GetValue() == v0
    m.set_fault_injection(_capi.GB_FAULT_NONE)
    v1, d1 = m.GetValueAndDerivative()
    assert v1 == v0 and np.array_equal(d1, d0)


def test_errors_are_kept_per_handle():
    """Two handles driven from one thread: each keeps the text of its own last error
    (gb_metric_last_error), while gb_last_error holds the thread's latest."""
    from itk_gb300 import Image, MeanSquaresImageToImageMetricv4
    fixed, moving, T = small_pair((24, 22, 20), config=0)
    a = MeanSquaresImageToImageMetricv4()
    b = MattesMutualInformationImageToImageMetricv4()
    assert _capi.metric_last_error(a.handle) == ""
    a.SetFixedImage(fixed)
    a.SetMovingImage(moving)
    a.SetMovingTransform(perturbed(T, 1))
    L = _capi.lib()
    assert L.gb_metric_get_value(a.handle, None) == _capi.GB_ERR_BAD_ARG  # a null output
    err_a = _capi.metric_last_error(a.handle)
    assert err_a and _capi.last_error() == err_a
    b.SetFixedImage(Image(np.zeros((20, 22, 24), np.float32)))  # a constant fixed image
    b.SetMovingImage(moving)
    b.SetMovingTransform(perturbed(T, 2))
    with pytest.raises(ExceptionObject):
        b.Initialize()
    err_b = _capi.metric_last_error(b.handle)
    assert err_b and err_b != err_a and _capi.last_error() == err_b
    assert _capi.metric_last_error(a.handle) == err_a
