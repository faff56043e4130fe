"""Device recursive-Gaussian filters and the per-level set-up vs the FP64 oracle.

The device recursions run in FP32 against the reference's double: smoothed
values within 2e-6 of the image's largest magnitude, gradients within 2e-5 of
the largest gradient component.  Metrics built on the device filters (the
metric's default gradient filter, level smoothing and shrink) are held to the
usual contract against the oracle metric run on the oracle's filtered images.
"""
import numpy as np
import pytest

from cases import geom, oracle_transform, run_oracle, small_pair
from conftest import MATTES_VALUE_ATOL, assert_deriv_close, assert_value_close
from itk_gb300 import (AffineTransform, GradientRecursiveGaussianImageFilter, Image, MattesMutualInformationImageToImageMetricv4,
                       MeanSquaresImageToImageMetricv4, ShrinkImageFilter, SmoothingRecursiveGaussianImageFilter,
                       data, shrink_geometry)
from itk_gb300.image import GradientImage
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rotation(deg):
    t = np.deg2rad(deg)
    return np.array([[np.cos(t), -np.sin(t), 0.0], [np.sin(t), np.cos(t), 0.0], [0.0, 0.0, 1.0]])


@pytest.fixture(scope="module")
def vol():
    img = data.blob_volume((37, 33, 29), seed=5)
    return Image(img.array, spacing=(1.0, 1.5, 0.8), origin=(2.0, -3.0, 1.0), direction=rotation(15))


@pytest.mark.parametrize("sigma", [0.7, 2.0, (1.0, 3.0, 0.5)])
def test_smoothing_matches_oracle(vol, sigma):
    f = SmoothingRecursiveGaussianImageFilter()
    if np.ndim(sigma):
        f.SetSigmaArray(sigma)
    else:
        f.SetSigma(sigma)
    f.SetInput(vol)
    f.Update()
    got = f.GetOutput().array
    want = O.smooth_recursive_gaussian(vol.array, vol.spacing, np.broadcast_to(np.asarray(sigma, float), (3,)))
    assert np.max(np.abs(got - want)) <= 2e-6 * np.max(np.abs(want))


@pytest.mark.parametrize("normalize,use_direction", [(True, True), (False, False), (True, False)])
def test_gradient_matches_oracle(vol, normalize, use_direction):
    f = GradientRecursiveGaussianImageFilter()
    f.SetSigma(1.5)
    f.SetNormalizeAcrossScale(normalize)
    f.SetUseImageDirection(use_direction)
    f.SetInput(vol)
    f.Update()
    got = f.GetOutput().array
    want = O.gradient_recursive_gaussian(vol.array, vol.spacing, vol.direction, 1.5, normalize, use_direction)
    assert np.max(np.abs(got - want)) <= 2e-5 * np.max(np.abs(want))


def test_shrink_filter_pixels(vol):
    f = ShrinkImageFilter()
    f.SetShrinkFactors((2, 3, 2))
    f.SetInput(vol)
    f.Update()
    out = f.GetOutput()
    size, sp, org = O.shrink_geometry(vol.GetSize(), vol.spacing, vol.origin, vol.direction, (2, 3, 2))
    assert tuple(out.GetSize()) == tuple(size)
    assert np.allclose(out.spacing, sp) and np.allclose(out.origin, org, rtol=0, atol=1e-12)
    # every output pixel is the input pixel at its own physical point
    for idx in [(0, 0, 0), (3, 2, 5), tuple(np.asarray(out.GetSize()) - 1)]:
        p = out.TransformIndexToPhysicalPoint(idx)
        ci = np.floor(vol.TransformPhysicalPointToContinuousIndex(p) + 0.5).astype(int)
        assert out.array[idx[2], idx[1], idx[0]] == vol.array[ci[2], ci[1], ci[0]]


@pytest.fixture(scope="module")
def pair_mm():
    fixed, moving, T = small_pair((48, 44, 40), config=1, multimodal=True)
    return fixed, moving, T


def metric(kind, fixed, moving, T, bins=40):
    m = MeanSquaresImageToImageMetricv4() if kind == "msq" else MattesMutualInformationImageToImageMetricv4()
    m.SetFixedImage(fixed)
    m.SetMovingImage(moving)
    m.SetMovingTransform(T)
    if kind == "mattes":
        m.SetNumberOfHistogramBins(bins)
    return m


@pytest.mark.parametrize("kind", ["msq", "mattes"])
def test_metric_default_gradient_filter(pair_mm, kind):
    """SetUseMovingImageGradientFilter(True) with no gradient image given: the moving
    gradient comes from the device GradientRecursiveGaussianImageFilter
    (sigma = max spacing, normalized across scale, image direction)."""
    fixed, moving, T = pair_mm
    m = metric(kind, fixed, moving, T)
    m.SetUseMovingImageGradientFilter(True)
    m.Initialize()
    v, d = m.GetValueAndDerivative()
    g = O.gradient_recursive_gaussian(moving.array, moving.spacing, moving.direction, float(max(moving.spacing)))
    r = run_oracle(kind, fixed, moving, T, gradient=GradientImage(g), bins=40)
    assert_value_close(v, r["value"], atol=MATTES_VALUE_ATOL if kind == "mattes" else 0.0)
    assert_deriv_close(d, r["derivative"])


@pytest.mark.parametrize("kind", ["msq", "mattes"])
@pytest.mark.parametrize("sigma,physical,shrink", [(2.0, True, (4, 4, 4)), (1.0, False, (2, 2, 2)),
                                                   (0.0, True, (2, 3, 1))])
def test_level_setup_matches_oracle(pair_mm, kind, sigma, physical, shrink):
    """A pyramid level as ImageRegistrationMethodv4 builds it: both images smoothed
    (sigma in physical units or voxels), the virtual domain the shrunk fixed geometry,
    the gradient from the default gradient filter on the smoothed moving image."""
    fixed, moving, T = pair_mm
    m = metric(kind, fixed, moving, T)
    m.SetUseMovingImageGradientFilter(True)
    m.SetLevelSmoothingSigma(sigma, physical)
    m.SetLevelShrinkFactors(shrink)
    m.Initialize()
    v, d = m.GetValueAndDerivative()
    if sigma > 0:
        sf = sigma * (np.ones(3) if physical else fixed.spacing)
        sm = sigma * (np.ones(3) if physical else moving.spacing)
        fs = Image(O.smooth_recursive_gaussian(fixed.array, fixed.spacing, sf), fixed.spacing, fixed.origin,
                   fixed.direction)
        ms = Image(O.smooth_recursive_gaussian(moving.array, moving.spacing, sm), moving.spacing, moving.origin,
                   moving.direction)
    else:
        fs, ms = fixed, moving
    g = O.gradient_recursive_gaussian(ms.array, ms.spacing, ms.direction, float(max(ms.spacing)))
    size, sp, org = O.shrink_geometry(fixed.GetSize(), fixed.spacing, fixed.origin, fixed.direction, shrink)
    vgeom = O.Geometry(tuple(int(s) for s in size), tuple(sp), tuple(org), tuple(fixed.direction.reshape(9)))
    T_o = oracle_transform(T)
    if kind == "msq":
        rc, rv, rd, nv = O.mean_squares(fs.array, geom(fs), ms.array, geom(ms), T_o, moving_grad=g,
                                        virtual_geom=vgeom)
    else:
        rc, rv, rd, nv, _, _ = O.mattes(fs.array, geom(fs), ms.array, geom(ms), T_o, bins=40, moving_grad=g,
                                        virtual_geom=vgeom)
    assert rc == 0
    assert m.GetNumberOfValidPoints() == nv
    assert m.GetNumberOfDomainPoints() == int(np.prod(size))
    assert_value_close(v, rv, atol=MATTES_VALUE_ATOL if kind == "mattes" else 0.0)
    assert_deriv_close(d, rd)


@pytest.mark.parametrize("degrees", range(0, 360, 15))
def test_gradient_filter_agrees_with_central_difference(degrees):
    """itkMetricImageGradientTest (3-D arm): a 60^3 box image with a 20-voxel zero
    border, the moving image resampled through a rotation about x, scale 1.2 and
    shear; at the virtual index (20, 20, 20) the moving gradient the metric uses --
    the default recursive-Gaussian gradient filter, and the central difference at
    the mapped point -- is compared with the oracle's CentralDifferenceImageFunction
    on the (double) resampled image; the mean of the two cosines must reach 0.96.  The metric
    is MeanSquares on the one point against an all-zero fixed image, so the
    translation entries of its derivative are -2 m(T(x)) times that gradient."""
    n, border = 60, 20
    k = np.arange(n)
    inside = (k >= border) & (np.abs(k - n) >= border)
    box = (inside[:, None, None] & inside[None, :, None] & inside[None, None, :]).astype(np.float64)
    t = np.deg2rad(degrees)
    rot = np.array([[1.0, 0.0, 0.0], [0.0, np.cos(t), -np.sin(t)], [0.0, np.sin(t), np.cos(t)]])
    shear = np.eye(3)
    shear[0, 1] = 0.05
    M = shear @ (1.2 * np.eye(3)) @ rot
    c = np.full(3, (n - 1) / 2.0)
    # moving(x) = box(M (x - c) + c), resampled on the same grid
    zz, yy, xx = np.meshgrid(k, k, k, indexing="ij")
    q = (np.stack([xx, yy, zz], -1).reshape(-1, 3) - c) @ M.T + c
    i0 = np.floor(q).astype(np.int64)
    fr = q - i0
    moving = np.zeros(n ** 3)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                x, y, z = i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz
                ok = (x >= 0) & (x < n) & (y >= 0) & (y < n) & (z >= 0) & (z < n)
                w = ((fr[:, 0] if dx else 1 - fr[:, 0]) * (fr[:, 1] if dy else 1 - fr[:, 1])
                     * (fr[:, 2] if dz else 1 - fr[:, 2]))
                moving[ok] += w[ok] * box[z[ok], y[ok], x[ok]]
    moving = moving.reshape(n, n, n)
    # the moving transform is the inverse: x -> M^-1 (x - c) + c
    Minv = np.linalg.inv(M)
    T = AffineTransform()
    T.SetCenter(c)
    T.SetMatrix(Minv)
    v = np.full(3, float(border))
    mapped = Minv @ (v - c) + c

    fixed = Image(np.zeros((n, n, n), np.float32))
    mov = Image(moving.astype(np.float32))
    truth = O.central_difference(moving, geom(mov), mapped[None, :])[0]
    total = 0.0
    for use_filter in (False, True):
        m = MeanSquaresImageToImageMetricv4()
        m.SetFixedImage(fixed)
        m.SetMovingImage(mov)
        m.SetMovingTransform(T)
        m.SetUseMovingImageGradientFilter(use_filter)
        m.SetVirtualSampledPointSet(v[None, :].astype(np.float32))
        m.SetUseSampledPointSet(True)
        m.Initialize()
        _, d = m.GetValueAndDerivative()
        g = -np.asarray(d)[9:12]
        n1, n2 = np.linalg.norm(truth), np.linalg.norm(g)
        if n1 > 0 and n2 > 0:
            total += (g @ truth) / (n1 * n2)
    assert total / 2.0 >= 0.96
