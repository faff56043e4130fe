"""Shared test inputs and the bridge that runs the oracle on the same inputs
as the GPU metric (test infrastructure)."""
from __future__ import annotations

import numpy as np

from itk_gb300 import data
from itk_gb300.image import Image
from itk_gb300.transforms import AffineTransform
from oracle import oracle as O


def geom(img: Image):
    return O.Geometry(tuple(int(s) for s in img.GetSize()), tuple(img.spacing), tuple(img.origin),
                      tuple(img.direction.reshape(9)))


def oracle_transform(t):
    kind, params, fixed = t.flat()
    return O.Transform(kind, np.asarray(params, np.float64), np.asarray(fixed, np.float64))


def run_oracle(metric_kind, fixed, moving, transform, gradient=None, points=None, bins=50, nthreads=None,
               compute_derivative=True, pixel_double=False):
    """metric_kind: 'msq', 'mattes' or 'jhmi' (variance 1.5).  Returns dict(status, value, derivative, nvalid[, pdf, state])."""
    g = None if gradient is None else gradient.array
    T = oracle_transform(transform)
    if metric_kind == "jhmi":
        rc, v, d, nv, pdf = O.joint_histogram_mi(fixed.array, geom(fixed), moving.array, geom(moving), T,
                                                 bins=bins, moving_grad=g, points=points, nthreads=nthreads,
                                                 compute_derivative=compute_derivative, pixel_double=pixel_double)
        return dict(status=rc, value=v, derivative=d, nvalid=nv, pdf=pdf)
    if metric_kind == "msq":
        rc, v, d, nv = O.mean_squares(fixed.array, geom(fixed), moving.array, geom(moving), T, moving_grad=g,
                                      points=points, nthreads=nthreads, compute_derivative=compute_derivative,
                                      pixel_double=pixel_double)
        return dict(status=rc, value=v, derivative=d, nvalid=nv)
    rc, v, d, nv, pdf, st = O.mattes(fixed.array, geom(fixed), moving.array, geom(moving), T, bins=bins,
                                     moving_grad=g, points=points, nthreads=nthreads,
                                     compute_derivative=compute_derivative, pixel_double=pixel_double)
    return dict(status=rc, value=v, derivative=d, nvalid=nv, pdf=pdf, state=st)


def mattes_2d_case(n=100):
    """The reference's Mattes known-answer images (itkMattesMutualInformationImageToImageMetricv4Test.cxx:60-135)
    as a 3-D volume one voxel thick."""
    idx = np.arange(n, dtype=np.float64)
    X, Y = np.meshgrid(idx, idx, indexing="xy")
    c = n / 2.0
    s = n / 2.0
    f = np.floor(200.0 * np.exp(-((X - c) ** 2 + (Y - c) ** 2) / (s * s)))
    m = np.floor(200.0 * np.exp(-((X - c + 5) ** 2 + (Y - c + 5) ** 2) / (s * s)))
    sp, org = (3.0, 2.0, 1.0), (0.001, -0.002, 0.0)
    fixed = Image(f.reshape(1, n, n), spacing=sp, origin=org)
    moving = Image(m.reshape(1, n, n), spacing=sp, origin=org)
    return fixed, moving


def mattes_2d_sample_points(fixed: Image):
    nx, ny, _ = fixed.GetSize()
    k = np.arange(nx * ny)[::5]
    iy, ix = k // nx, k % nx
    return np.stack([fixed.origin[0] + fixed.spacing[0] * ix, fixed.origin[1] + fixed.spacing[1] * iy,
                     np.zeros_like(ix, dtype=np.float64)], 1).astype(np.float32)


def small_pair(size=(41, 37, 29), config=0, multimodal=False, seed_shift=0):
    fixed, moving, T = data.pair_affine(size, config, instance=seed_shift, multimodal_map=multimodal)
    return fixed, moving, T


def perturbed(T: AffineTransform, seed, scale=0.02, trans=1.0):
    rng = np.random.default_rng(seed)
    U = AffineTransform()
    U.SetCenter(T.GetCenter())
    M = np.eye(3) + rng.uniform(-scale, scale, size=(3, 3))
    U.SetMatrix(M)
    U.SetTranslation(rng.uniform(-trans, trans, size=3))
    return U


def shared_voxel_points(image: Image, fraction, seed, per_voxel=3, jitter=0.4):
    """A point set with `per_voxel` points in each of a random set of voxels (each moved by
    up to `jitter` voxel along each index axis, so the nearest voxel stays the same): the
    local-support derivative then sums several points' blocks into one voxel."""
    nx, ny, nz = image.GetSize()
    total = nx * ny * nz
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(total, size=max(1, int(total * fraction)), replace=False))
    ijk = np.stack([idx % nx, (idx // nx) % ny, idx // (nx * ny)], axis=1).astype(np.float64)
    ijk = np.repeat(ijk, per_voxel, axis=0) + rng.uniform(-jitter, jitter, size=(len(idx) * per_voxel, 3))
    return (ijk @ image.index_to_physical().T + image.origin).astype(np.float32)
