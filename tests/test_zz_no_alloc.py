"""The allocation-free MeanSquares entry point, gb_msq_affine_noalloc.

Some callers of this library cannot allocate device memory: code running
inside another framework's memory pool or arena, real-time loops that forbid
allocation once started, hosts that account for every device allocation.
gb_msq_affine_noalloc serves them: inputs and output live in caller-owned
device memory and the per-call scratch sits in a static device array.  This
test gives it the same images, samples and transform as the allocating metric
handle and the FP64 oracle, on an oblique grid with non-unit spacing and an
offset origin (so physical points and indices differ), and checks that all
three agree on two calls in a row (the shared scratch keeps the previous
call's contents and must be cleared by each call).  A transform that maps
every sample outside the moving image leaves out = [DBL_MAX, 0, 0...].
"""
import ctypes

import numpy as np
import pytest

from cases import perturbed, run_oracle
from conftest import assert_deriv_close, assert_value_close

pytestmark = pytest.mark.gpu


def _rotation(ax, ay, az):
    cx, sx, cy, sy, cz, sz = np.cos(ax), np.sin(ax), np.cos(ay), np.sin(ay), np.cos(az), np.sin(az)
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    return Rz @ Ry @ Rx


def _oblique_case():
    """A blob pair on an oblique grid (spacing 1.2 / 0.9 / 1.1 mm, origin off zero, rotated
    direction); the moving image on the same grid shifted by a few millimetres."""
    from itk_gb300 import Image, data

    f0, m0, T0 = data.pair_affine((40, 36, 32), config=0)
    spacing = np.array([1.2, 0.9, 1.1])
    direction = _rotation(0.2, -0.15, 0.3)
    fixed = Image(f0.array, spacing=spacing, origin=(-12.5, 7.25, 3.0), direction=direction)
    moving = Image(m0.array, spacing=spacing, origin=(-11.0, 6.0, 4.5), direction=direction)
    grad = data.gradient_image(moving)
    U = perturbed(T0, 21)
    U.SetCenter(fixed.physical_center())
    return fixed, moving, grad, U


def _call(L, samples, mov, moving, U, out, stream):
    from itk_gb300 import _capi
    size = np.asarray(moving.GetSize(), np.int64)
    spacing, origin = moving.spacing.copy(), moving.origin.copy()
    direction = moving.direction.reshape(9).copy()
    params, center = np.ascontiguousarray(U.GetParameters()), np.ascontiguousarray(U.GetCenter())
    return L.gb_msq_affine_noalloc(ctypes.c_void_p(samples.data_ptr()), samples.shape[0],
                                   ctypes.c_void_p(mov.data_ptr()), _capi.ptr(size), _capi.ptr(spacing),
                                   _capi.ptr(origin), _capi.ptr(direction), _capi.ptr(params), _capi.ptr(center),
                                   ctypes.c_void_p(out.data_ptr()), stream)


def test_noalloc_matches_metric_handle_and_oracle():
    import torch

    from itk_gb300 import AffineTransform, MeanSquaresImageToImageMetricv4, _capi

    fixed, moving, grad, U = _oblique_case()
    # physical points at fixed-image voxel centres: the fixed value there is the voxel itself
    nx, ny, nz = fixed.GetSize()
    rng = np.random.default_rng(5)
    idx = rng.choice(nx * ny * nz, size=9000, replace=False)
    ix, iy, iz = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    phys = np.stack([ix, iy, iz], 1).astype(np.float64) @ fixed.index_to_physical().T + fixed.origin
    pts = phys.astype(np.float32)
    # the fixed value as the metric stores it: the fixed image at the (float) point, FP64
    # trilinear interpolation rounded to float
    from itk_gb300 import data
    ci = np.linalg.solve(fixed.index_to_physical(), (pts.astype(np.float64) - fixed.origin).T).T
    fvals = data.trilinear(fixed.array.astype(np.float64), ci).astype(np.float32)

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
    assert 0 < n_ref < len(pts)  # some samples leave the shifted moving image

    # the FP64 oracle on the same inputs
    r = run_oracle("msq", fixed, moving, U, gradient=grad, points=pts)
    assert r["nvalid"] == n_ref

    # the allocation-free path: every device buffer belongs to the caller
    dev = torch.device("cuda:0")
    samples = torch.tensor(np.concatenate([pts, fvals[:, None]], 1), dtype=torch.float32, device=dev)
    packed = np.concatenate([moving.array[..., None], grad.array.astype(np.float32)], axis=-1)
    mov = torch.tensor(packed.reshape(-1, 4), dtype=torch.float32, device=dev)
    out = torch.empty(14, dtype=torch.float64, device=dev)
    L = _capi.lib()
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        out.fill_(float("nan"))
        rc = _call(L, samples, mov, moving, U, out, stream)
        assert rc == _capi.GB_OK, _capi.last_error()
        torch.cuda.synchronize()
        res = out.cpu().numpy()
        assert int(res[1]) == n_ref
        assert_value_close(res[0], v_ref)
        assert_deriv_close(res[2:], d_ref)
        assert_value_close(res[0], r["value"])
        assert_deriv_close(res[2:], r["derivative"])

    # no sample inside the moving image: the call succeeds, out = [DBL_MAX, 0, 0...]
    far = AffineTransform()
    far.SetCenter(U.GetCenter())
    far.SetTranslation([1.0e4, 0.0, 0.0])
    out.fill_(float("nan"))
    rc = _call(L, samples, mov, moving, far, out, stream)
    assert rc == _capi.GB_OK, _capi.last_error()
    torch.cuda.synchronize()
    res = out.cpu().numpy()
    assert res[0] == np.finfo(np.float64).max and res[1] == 0.0 and np.all(res[2:] == 0.0)

    # and the next call is again the metric's (the scratch is cleared per call)
    out.fill_(float("nan"))
    assert _call(L, samples, mov, moving, U, out, stream) == _capi.GB_OK
    torch.cuda.synchronize()
    res = out.cpu().numpy()
    assert int(res[1]) == n_ref
    assert_value_close(res[0], v_ref)

    # sizes beyond the stated maximum are rejected before anything runs
    params, center = np.ascontiguousarray(U.GetParameters()), np.ascontiguousarray(U.GetCenter())
    size = np.asarray(moving.GetSize(), np.int64)
    rc = L.gb_msq_affine_noalloc(ctypes.c_void_p(samples.data_ptr()), 1 << 31, ctypes.c_void_p(mov.data_ptr()),
                                 _capi.ptr(size), _capi.ptr(moving.spacing.copy()), _capi.ptr(moving.origin.copy()),
                                 _capi.ptr(moving.direction.reshape(9).copy()), _capi.ptr(params), _capi.ptr(center),
                                 ctypes.c_void_p(out.data_ptr()), stream)
    assert rc == _capi.GB_ERR_BAD_ARG and "2^31-1 samples" in _capi.last_error()
