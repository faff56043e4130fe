"""The oracle's displacement-field transform and local-support derivative (no GPU).

Pinned by the reference's own constructions:
  * ImageToImageMetricv4Test's identity-field truth (Registration/Metricsv4/test/
    itkImageToImageMetricv4Test.cxx:200-300): under an identity displacement field
    the derivative at voxel v is that voxel's own point derivative, stored at
    v * NumberOfLocalParameters and not averaged -- here for MeanSquares,
    2 (f - m) grad m with the gradient image read at the voxel;
  * a constant field is a translation: value equal to the affine translation's
    and, by linearity, the derivative field summed over the voxels equal to the
    translation entries of the affine derivative (times N for MeanSquares, whose
    local derivative is not averaged);
  * TransformPoint against the package's own numpy restatement."""
import numpy as np
import pytest

from cases import geom, oracle_transform
from itk_gb300 import AffineTransform, DisplacementFieldImage, DisplacementFieldTransform, Image, data
from oracle import oracle as O


@pytest.fixture(scope="module")
def pair():
    fixed, moving, _ = data.pair_affine((23, 19, 17), config=1, instance=3, multimodal_map=True)
    return fixed, moving


def field_transform(image, array):
    t = DisplacementFieldTransform()
    t.SetDisplacementField(DisplacementFieldImage.like(image, array))
    return t


def run(kind, fixed, moving, T, gradient=None, points=None, bins=20):
    g = None if gradient is None else gradient.array
    if kind == "msq":
        rc, v, d, nv = O.mean_squares(fixed.array, geom(fixed), moving.array, geom(moving), oracle_transform(T),
                                      moving_grad=g, points=points)
    else:
        rc, v, d, nv, _, _ = O.mattes(fixed.array, geom(fixed), moving.array, geom(moving), oracle_transform(T),
                                      bins=bins, moving_grad=g, points=points)
    return rc, v, np.asarray(d), nv


def test_transform_point_matches_numpy():
    rng = np.random.default_rng(0)
    img = Image(np.zeros((7, 8, 9), np.float32), spacing=(1.2, 0.9, 1.1), origin=(1.0, -2.0, 0.5))
    t = field_transform(img, rng.normal(size=(7, 8, 9, 3)))
    x = rng.uniform(-2.0, 12.0, size=(3000, 3))
    y = O.transform_points(oracle_transform(t), x)
    np.testing.assert_allclose(y, t.TransformPoint(x), rtol=0, atol=1e-12)
    outside = np.all(y == x, axis=1)
    assert 0.05 < outside.mean() < 0.95  # both branches exercised
    # at the voxel centres the field value itself
    nx, ny, nz = img.GetSize()
    k = np.arange(nx * ny * nz)
    pts = np.stack([k % nx, (k // nx) % ny, k // (nx * ny)], axis=1) @ img.index_to_physical().T + img.origin
    np.testing.assert_allclose(O.transform_points(oracle_transform(t), pts) - pts,
                               t.GetDisplacementField().array.reshape(-1, 3), rtol=0, atol=1e-12)


def test_identity_field_meansquares_truth(pair):
    fixed, moving = pair
    T = field_transform(fixed, np.zeros(fixed.array.shape + (3,)))
    grad = data.gradient_image(moving)
    rc, v, d, nv = run("msq", fixed, moving, T, gradient=grad)
    assert rc == 0 and nv == fixed.array.size
    diff = (fixed.array - moving.array).astype(np.float32).astype(np.float64)  # FixedImagePixelType diff
    assert v == pytest.approx(np.mean(diff ** 2), rel=1e-12)
    truth = (2.0 * diff[..., None] * grad.array).reshape(-1)
    np.testing.assert_allclose(d, truth, rtol=1e-12, atol=1e-12 * np.max(np.abs(truth)))


@pytest.mark.parametrize("kind", ["msq", "mattes"])
@pytest.mark.parametrize("gradient", [True, False])
def test_constant_field_is_a_translation(pair, kind, gradient):
    fixed, moving = pair
    c = np.array([0.75, -0.5, 0.25])
    T = field_transform(fixed, np.broadcast_to(c, fixed.array.shape + (3,)).copy())
    A = AffineTransform()
    A.SetTranslation(c)
    grad = data.gradient_image(moving) if gradient else None
    rc1, v1, d1, n1 = run(kind, fixed, moving, T, gradient=grad)
    rc2, v2, d2, n2 = run(kind, fixed, moving, A, gradient=grad)
    assert rc1 == rc2 == 0 and n1 == n2
    assert v1 == pytest.approx(v2, rel=1e-13, abs=1e-15)
    s = d1.reshape(-1, 3).sum(axis=0)
    want = d2[9:12] * (n2 if kind == "msq" else 1.0)
    np.testing.assert_allclose(s, want, rtol=1e-9, atol=1e-12 * np.max(np.abs(want)))


def test_sampled_points_feed_their_nearest_voxel(pair):
    fixed, moving = pair
    T = field_transform(fixed, data.smooth_displacement_field(fixed, seed=5, max_disp=1.5).array)
    pts = data.unique_voxel_points(fixed, 0.2, seed=2)
    grad = data.gradient_image(moving)
    rc, v, d, nv = run("msq", fixed, moving, T, gradient=grad, points=pts)
    assert rc == 0 and nv > 0
    blocks = np.abs(d.reshape(-1, 3)).sum(axis=1)
    # only voxels holding a point carry a block
    idx = np.rint((pts.astype(np.float64) - fixed.origin) / fixed.spacing).astype(np.int64)
    nx, ny, _ = fixed.GetSize()
    holders = np.zeros(blocks.size, bool)
    holders[idx[:, 0] + nx * (idx[:, 1] + ny * idx[:, 2])] = True
    assert np.all(blocks[~holders] == 0) and np.count_nonzero(blocks[holders]) > 0.5 * holders.sum()


def test_field_must_share_the_virtual_grid(pair):
    fixed, moving = pair
    img = Image(np.zeros((fixed.array.shape[0], fixed.array.shape[1], fixed.array.shape[2] + 1), np.float32))
    T = field_transform(img, np.zeros(img.array.shape + (3,)))
    assert run("msq", fixed, moving, T)[0] == 1  # BAD_ARG
    shifted = Image(fixed.array, fixed.spacing, fixed.origin + 0.5)
    T = field_transform(shifted, np.zeros(fixed.array.shape + (3,)))
    assert run("mattes", fixed, moving, T)[0] == 1  # BAD_ARG
