"""Algorithmic byte counts of one metric evaluation (for roofline fractions).

B_alg = N_s * b_pt + V_touched * (4 B fixed + 4 B moving + 12 B moving gradient),
with V_touched the number of distinct moving voxels in the union of the
2x2x2 trilinear stencils of all samples (each distinct input byte counted
once per evaluation), b_pt = 12 B (xyz float) for a sampled point set and 0
for a dense virtual grid.
"""
from __future__ import annotations

import numpy as np


def touched_voxels(points, transform, moving, chunk=1 << 21):
    """Distinct voxels of `moving` under the trilinear stencils of T(points) (inside samples only)."""
    nx, ny, nz = moving.GetSize()
    p2i = np.linalg.inv(moving.index_to_physical())
    mark = np.zeros(nx * ny * nz, dtype=bool)
    pts = np.asarray(points, np.float64).reshape(-1, 3)
    n = np.array([nx, ny, nz])
    for s in range(0, len(pts), chunk):
        y = transform.TransformPoint(pts[s:s + chunk])
        ci = (y - moving.origin) @ p2i.T
        ok = np.all((ci >= -0.5) & (ci < n - 0.5), axis=1)
        ci = ci[ok]
        b = np.clip(np.floor(ci).astype(np.int64), 0, n - 1)
        d = ci - np.floor(ci)
        for dz in (0, 1):
            for dy in (0, 1):
                for dx in (0, 1):
                    off = np.array([dx, dy, dz])
                    use = np.all((off == 0) | (d > 0), axis=1)
                    q = np.minimum(b + off, n - 1)[use]
                    mark[q[:, 0] + nx * (q[:, 1] + ny * q[:, 2])] = True
    return int(mark.sum())


def evaluation_bytes(n_samples, v_touched, sparse=True, nparams=0):
    """B_alg of one GetValueAndDerivative evaluation (+ the parameters in and the derivative out, 8 B each)."""
    return n_samples * (12 if sparse else 0) + v_touched * 20 + nparams * 16


def mattes_pass1_bspline_bytes(n_samples, v_touched, nodes):
    """Minimal DRAM traffic of the B-spline Mattes pass-1 kernel: as the affine pass 1 plus each
    sample's B-spline support record (16 B) and the float4 control nodes once (16 B each)."""
    return n_samples * 48 + v_touched * 16 + nodes * 16


def msq_bspline_bytes(n_samples, v_touched, nodes):
    """Minimal DRAM traffic of the B-spline MeanSquares kernel: sample record and support record
    read, per-sample derivative factor written (16 B each), touched voxels and nodes once."""
    return n_samples * 48 + v_touched * 16 + nodes * 16


def mattes_pass1_bytes(n_samples, v_touched):
    """Minimal DRAM traffic of the Mattes pass-1 kernel: sample records (xyz + fixed bin, 16 B),
    each touched (value, gradient) voxel once (16 B), per-sample cache written (16 B)."""
    return n_samples * 32 + v_touched * 16


def msq_bytes(n_samples, v_touched):
    """Minimal DRAM traffic of the MeanSquares kernel: sample records (16 B) + touched voxels (16 B)."""
    return n_samples * 16 + v_touched * 16


def mattes_pass1_field_bytes(n_samples, v_touched):
    """Minimal DRAM traffic of the Mattes pass-1 kernel under a dense displacement field: the
    sample record (16 B) and the sample's field value (3 doubles, 24 B) read, the per-sample cache
    written (16 B), each touched (value, gradient) voxel once (16 B)."""
    return n_samples * 56 + v_touched * 16


def msq_field_bytes(n_samples, v_touched):
    """Minimal DRAM traffic of the MeanSquares kernel under a dense displacement field: sample
    record (16 B) and field value (24 B) read, the derivative block (3 doubles, 24 B) written,
    touched voxels once (16 B)."""
    return n_samples * 64 + v_touched * 16


def mattes_pass2_field_bytes(n_samples):
    """Minimal DRAM traffic of the Mattes derivative-block kernel under a dense displacement field:
    cache and sample record read (16 B each), the derivative block written (24 B)."""
    return n_samples * 56


def jhmi_pass1_bytes(n_samples, v_touched):
    """Minimal DRAM traffic of the joint-histogram MI pass 1: sample records (16 B) read, the
    per-sample cache (moving value and gradient, 16 B) written, touched voxels once (16 B)."""
    return n_samples * 32 + v_touched * 16
