"""The allocation-free MeanSquares entry point, gb_msq_affine_noalloc.

Some callers of this library cannot allocate device memory: code running
inside another framework's memory pool or arena, real-time loops that forbid
allocation once started, hosts that account for every device allocation.
gb_msq_affine_noalloc serves them: inputs and output live in caller-owned
device memory and the per-call scratch sits in a static device array.  This
test gives it the same images, samples and transform as the allocating metric
handle and checks that both agree, on two calls in a row (the shared scratch
keeps the previous call's contents and must be cleared by each call).
"""
import ctypes

import numpy as np
import pytest

from cases import perturbed
from conftest import assert_deriv_close, assert_value_close

pytestmark = pytest.mark.gpu


def test_noalloc_matches_metric_handle():
    import torch

    from itk_gb300 import MeanSquaresImageToImageMetricv4, _capi, data

    fixed, moving, T = data.pair_affine((40, 36, 32), config=0)
    grad = data.gradient_image(moving)
    U = perturbed(T, 21)
    # samples at fixed-image voxel centres (spacing 1, origin 0): the fixed value there is the voxel
    nx, ny, nz = fixed.GetSize()
    rng = np.random.default_rng(5)
    idx = rng.choice(nx * ny * nz, size=9000, replace=False)
    ix, iy, iz = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    pts = np.stack([ix, iy, iz], 1).astype(np.float32)
    fvals = fixed.array[iz, iy, ix]

    # the allocating path: a metric handle
    m = MeanSquaresImageToImageMetricv4()
    m.SetFixedImage(fixed)
    m.SetMovingImage(moving)
    m.SetMovingTransform(U)
    m.SetMovingImageGradientImage(grad)
    m.SetVirtualSampledPointSet(pts)
    m.SetUseSampledPointSet(True)
    m.Initialize()
    v_ref, d_ref = m.GetValueAndDerivative()
    n_ref = m.GetNumberOfValidPoints()
    assert n_ref > 0

    # the allocation-free path: every device buffer belongs to the caller
    dev = torch.device("cuda:0")
    samples = torch.tensor(np.concatenate([pts, fvals[:, None]], 1), dtype=torch.float32, device=dev)
    packed = np.concatenate([moving.array[..., None], grad.array.astype(np.float32)], axis=-1)
    mov = torch.tensor(packed.reshape(-1, 4), dtype=torch.float32, device=dev)
    out = torch.empty(14, dtype=torch.float64, device=dev)
    L = _capi.lib()
    size = np.asarray(moving.GetSize(), np.int64)
    spacing, origin = moving.spacing.copy(), moving.origin.copy()
    direction = moving.direction.reshape(9).copy()
    params, center = U.GetParameters(), U.GetCenter()
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        out.fill_(float("nan"))
        rc = L.gb_msq_affine_noalloc(ctypes.c_void_p(samples.data_ptr()), samples.shape[0],
                                     ctypes.c_void_p(mov.data_ptr()), _capi.ptr(size), _capi.ptr(spacing),
                                     _capi.ptr(origin), _capi.ptr(direction), _capi.ptr(params), _capi.ptr(center),
                                     ctypes.c_void_p(out.data_ptr()), stream)
        assert rc == _capi.GB_OK, _capi.last_error()
        torch.cuda.synchronize()
        res = out.cpu().numpy()
        assert int(res[1]) == n_ref
        assert_value_close(res[0], v_ref)
        assert_deriv_close(res[2:], d_ref)

    # sizes beyond the stated maximum are rejected before anything runs
    rc = L.gb_msq_affine_noalloc(ctypes.c_void_p(samples.data_ptr()), 1 << 31, ctypes.c_void_p(mov.data_ptr()),
                                 _capi.ptr(size), _capi.ptr(spacing), _capi.ptr(origin), _capi.ptr(direction),
                                 _capi.ptr(params), _capi.ptr(center), ctypes.c_void_p(out.data_ptr()), stream)
    assert rc == _capi.GB_ERR_BAD_ARG and "2^31-1 samples" in _capi.last_error()
