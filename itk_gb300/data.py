"""Seeded synthetic registration inputs with the shapes of the benchmark configs.

* blob volume: 12 Gaussian blobs (centres uniform in the volume, sigma
  U[3, 10] voxels, amplitude U[50, 200]) plus N(0, 2) noise, float32, 1 mm
  spacing, origin 0, identity direction;
* moving image: the fixed image resampled (trilinear, 0 outside) under a seeded
  affine about the image centre (Euler angles U(+-8 deg), translations
  U(+-5 mm), scales U(0.95, 1.05)) plus fresh N(0, 2) noise;
* multimodal variant: v' = 1000 (max(v, 0) / max)^1.7 + N(0, 5);
* random_points: uniform voxel picks with replacement plus N(0, spacing/3)
  jitter per coordinate, stored as float32 points -- the shape of
  ImageRegistrationMethodv4's RANDOM strategy
  (Registration/RegistrationMethodsv4/include/itkImageRegistrationMethodv4.hxx:965-1003)
  from numpy's generator, for tests; itk_gb300.sample_points draws the
  reference's own points (its Mersenne Twister, bit for bit).

The seed of an instance is 1000 * config + instance.
"""
from __future__ import annotations

import numpy as np

from .image import DisplacementFieldImage, GradientImage, Image
from .transforms import AffineTransform, BSplineTransform, CompositeTransform


def blob_volume(size_xyz, seed, n_blobs=12, noise_sigma=2.0, spacing=(1.0, 1.0, 1.0)):
    nx, ny, nz = (int(s) for s in size_xyz)
    rng = np.random.default_rng(seed)
    centres = rng.uniform([0, 0, 0], [nx - 1, ny - 1, nz - 1], size=(n_blobs, 3))
    sigmas = rng.uniform(3.0, 10.0, size=n_blobs)
    amps = rng.uniform(50.0, 200.0, size=n_blobs)
    x = np.arange(nx, dtype=np.float32)
    y = np.arange(ny, dtype=np.float32)
    z = np.arange(nz, dtype=np.float32)
    vol = np.zeros((nz, ny, nx), dtype=np.float32)
    for c, s, a in zip(centres, sigmas, amps):
        gx = np.exp(-((x - c[0]) ** 2) / (2 * s * s)).astype(np.float32)
        gy = np.exp(-((y - c[1]) ** 2) / (2 * s * s)).astype(np.float32)
        gz = (a * np.exp(-((z - c[2]) ** 2) / (2 * s * s))).astype(np.float32)
        vol += gz[:, None, None] * (gy[:, None] * gx[None, :])[None, :, :]
    vol += rng.normal(0.0, noise_sigma, size=vol.shape).astype(np.float32)
    return Image(vol, spacing=spacing)


def random_affine(seed, center, max_rot_deg=8.0, max_trans=5.0, scale_range=(0.95, 1.05)):
    rng = np.random.default_rng(seed)
    ax, ay, az = np.deg2rad(rng.uniform(-max_rot_deg, max_rot_deg, size=3))
    t = rng.uniform(-max_trans, max_trans, size=3)
    s = rng.uniform(scale_range[0], scale_range[1], size=3)
    cx, sx, cy, sy, cz, sz = np.cos(ax), np.sin(ax), np.cos(ay), np.sin(ay), np.cos(az), np.sin(az)
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    T = AffineTransform()
    T.SetCenter(center)
    T.SetMatrix(Rz @ Ry @ Rx @ np.diag(s))
    T.SetTranslation(t)
    return T


def trilinear(array, ci, default=0.0):
    """Trilinear samples of a (nz, ny, nx) array at continuous indices ci (n, 3) in xyz order;
    points outside [-0.5, n-0.5) get `default` (ResampleImageFilter's default value)."""
    nz, ny, nx = array.shape
    n = np.array([nx, ny, nz])
    inside = np.all((ci >= -0.5) & (ci < n - 0.5), axis=1)
    b = np.floor(ci).astype(np.int64)
    d = ci - b
    d = np.where(b < 0, 0.0, d)
    b0 = np.clip(b, 0, n - 1)
    b1 = np.clip(b + 1, 0, n - 1)
    out = np.zeros(ci.shape[0], dtype=np.float64)
    for dz in (0, 1):
        zi = b1[:, 2] if dz else b0[:, 2]
        wz = d[:, 2] if dz else 1.0 - d[:, 2]
        for dy in (0, 1):
            yi = b1[:, 1] if dy else b0[:, 1]
            wy = d[:, 1] if dy else 1.0 - d[:, 1]
            for dx in (0, 1):
                xi = b1[:, 0] if dx else b0[:, 0]
                wx = d[:, 0] if dx else 1.0 - d[:, 0]
                out += wx * wy * wz * array[zi, yi, xi]
    return np.where(inside, out, default)


def resample(image: Image, transform, seed_noise=None, noise_sigma=0.0, chunk=1 << 21):
    """moving(y) = image(T(y)) on the image's own grid (ResampleImageFilter semantics)."""
    nx, ny, nz = image.GetSize()
    i2p = image.index_to_physical()
    p2i = np.linalg.inv(i2p)
    out = np.empty(nx * ny * nz, dtype=np.float32)
    total = nx * ny * nz
    for s in range(0, total, chunk):
        idx = np.arange(s, min(total, s + chunk))
        ijk = np.stack([idx % nx, (idx // nx) % ny, idx // (nx * ny)], axis=1).astype(np.float64)
        pts = ijk @ i2p.T + image.origin
        mp = transform.TransformPoint(pts)
        ci = (mp - image.origin) @ p2i.T
        out[s:s + len(idx)] = trilinear(image.array, ci).astype(np.float32)
    vol = out.reshape(nz, ny, nx)
    if noise_sigma > 0:
        rng = np.random.default_rng(seed_noise)
        vol = vol + rng.normal(0.0, noise_sigma, size=vol.shape).astype(np.float32)
    return Image(vol, spacing=image.spacing, origin=image.origin, direction=image.direction)


def multimodal(image: Image, seed, gamma=1.7, scale=1000.0, noise_sigma=5.0):
    v = np.maximum(image.array.astype(np.float64), 0.0)
    vmax = v.max() if v.max() > 0 else 1.0
    rng = np.random.default_rng(seed)
    out = scale * (v / vmax) ** gamma + rng.normal(0.0, noise_sigma, size=v.shape)
    return Image(out.astype(np.float32), spacing=image.spacing, origin=image.origin, direction=image.direction)


def gradient_image(image: Image) -> GradientImage:
    """Central-difference gradient in physical units (one-sided at the borders), as a
    CovariantVector<double,3> image; a stand-in input for the metric's gradient filter."""
    a = image.array.astype(np.float64)
    gz, gy, gx = np.gradient(a, image.spacing[2], image.spacing[1], image.spacing[0])
    g = np.stack([gx, gy, gz], axis=-1)
    g = g @ image.direction.T  # index-axis derivatives to physical (identity for these inputs)
    return GradientImage(g)


def random_points(image: Image, fraction, seed):
    """RANDOM sampling: floor(voxels * fraction) uniform voxel picks + N(0, spacing/3) jitter, float32."""
    nx, ny, nz = image.GetSize()
    total = nx * ny * nz
    n = int(np.float32(total) * np.float32(fraction))
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, total, size=n)
    ijk = np.stack([idx % nx, (idx // nx) % ny, idx // (nx * ny)], axis=1).astype(np.float64)
    pts = ijk @ image.index_to_physical().T + image.origin
    pts += rng.normal(0.0, 1.0, size=pts.shape) * (image.spacing / 3.0)
    return pts.astype(np.float32)


def dense_points(image: Image):
    nx, ny, nz = image.GetSize()
    idx = np.arange(nx * ny * nz)
    ijk = np.stack([idx % nx, (idx // nx) % ny, idx // (nx * ny)], axis=1).astype(np.float64)
    return (ijk @ image.index_to_physical().T + image.origin).astype(np.float32)


def bspline_over_image(image: Image, mesh_size):
    """BSplineTransform (order 3) whose transform domain is the image's physical extent
    (origin, spacing * (size - 1), direction), as BSplineTransformInitializer sets it up."""
    T = BSplineTransform()
    size = np.asarray(image.GetSize(), np.float64)
    T.SetTransformDomain(image.origin, image.spacing * (size - 1.0), mesh_size, image.direction)
    return T


def random_bspline_coefficients(T: BSplineTransform, seed, max_disp=4.0):
    """Uniform coefficients with |c| <= max_disp / sqrt(3) per component: the cubic B-spline weights are a
    nonnegative partition of unity, so every displacement vector is at most max_disp long."""
    rng = np.random.default_rng(seed)
    T.SetParameters(rng.uniform(-1.0, 1.0, size=T.GetNumberOfParameters()) * (max_disp / np.sqrt(3.0)))
    return T


def smooth_displacement_field(image: Image, seed, max_disp=2.0, mesh_size=(3, 3, 3)):
    """A smooth field on the image's grid: the displacement of a seeded cubic B-spline
    (at most max_disp long) at every voxel centre, as a DisplacementFieldImage."""
    B = random_bspline_coefficients(bspline_over_image(image, mesh_size), seed, max_disp)
    x = dense_points(image).astype(np.float64)
    nx, ny, nz = image.GetSize()
    u = (B.TransformPoint(x) - x).reshape(nz, ny, nx, 3)
    return DisplacementFieldImage.like(image, u)


def unique_voxel_points(image: Image, fraction, seed, jitter=0.4):
    """A point set with at most one point per voxel: distinct random voxels, each moved by
    up to `jitter` voxel along each index axis (the nearest voxel stays its own)."""
    nx, ny, nz = image.GetSize()
    total = nx * ny * nz
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(total, size=max(1, int(total * fraction)), replace=False))
    ijk = np.stack([idx % nx, (idx // nx) % ny, idx // (nx * ny)], axis=1).astype(np.float64)
    ijk += rng.uniform(-jitter, jitter, size=ijk.shape)
    return (ijk @ image.index_to_physical().T + image.origin).astype(np.float32)


def pair_bspline(size_xyz, mesh_size=(8, 8, 8), instance=0, max_disp=4.0, multimodal_map=True, config=2):
    """(fixed, moving, affine, B-spline) of the B-spline config: the blob volume; the moving image is the
    fixed one resampled under the composite [affine, B-spline] (B-spline applied first) with a seeded
    smooth displacement (at most max_disp mm), then the multimodal intensity map."""
    seed = 1000 * config + instance
    fixed = blob_volume(size_xyz, seed)
    A = random_affine(seed + 1, fixed.physical_center())
    B = random_bspline_coefficients(bspline_over_image(fixed, mesh_size), seed + 4, max_disp)
    C = CompositeTransform()
    C.AddTransform(A)
    C.AddTransform(B)
    moving = resample(fixed, C, seed_noise=seed + 2, noise_sigma=0.0 if multimodal_map else 2.0)
    if multimodal_map:
        moving = multimodal(moving, seed + 3)
    return fixed, moving, A, B


def pair_affine(size_xyz, config, instance=0, multimodal_map=False):
    """(fixed, moving, true transform) as in the MeanSquares / Mattes affine configs."""
    seed = 1000 * config + instance
    fixed = blob_volume(size_xyz, seed)
    T = random_affine(seed + 1, fixed.physical_center())
    moving = resample(fixed, T, seed_noise=seed + 2, noise_sigma=0.0 if multimodal_map else 2.0)
    if multimodal_map:
        moving = multimodal(moving, seed + 3)
    return fixed, moving, T


def batch_instance_sizes(n, seed, vmin=48 ** 3, vmax=256 * 256 * 200, aspect=(256, 256, 200)):
    """Volume sizes of the batched / served workloads: voxel counts log-uniform in
    [vmin, vmax], each axis the count's cube root scaled by the 256:256:200 aspect."""
    rng = np.random.default_rng(seed)
    v = np.exp(rng.uniform(np.log(vmin), np.log(vmax), size=n))
    a = np.asarray(aspect, np.float64)
    f = (v / np.prod(a)) ** (1.0 / 3.0)
    return [tuple(int(max(8, round(x))) for x in a * fi) for fi in f]
