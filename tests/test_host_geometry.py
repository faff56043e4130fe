"""Host-only parts of the C ABI (no GPU needed): ShrinkImageFilter geometry from
gb_shrink_geometry against the oracle's restatement, for identity and rotated
directions, anisotropic spacing and factors that do not divide the size."""
import numpy as np
import pytest

from itk_gb300 import Image, shrink_geometry
from oracle import oracle as O


def rotation(ax, deg):
    t = np.deg2rad(deg)
    c, s = np.cos(t), np.sin(t)
    R = np.eye(3)
    i, j = [(1, 2), (0, 2), (0, 1)][ax]
    R[i, i], R[i, j], R[j, i], R[j, j] = c, -s, s, c
    return R


@pytest.mark.parametrize("factors", [(1, 1, 1), (2, 2, 2), (4, 4, 4), (3, 2, 5), (1, 4, 2)])
@pytest.mark.parametrize("direction", [np.eye(3), rotation(2, 30) @ rotation(0, -12)])
def test_shrink_geometry_matches_oracle(factors, direction):
    img = Image(np.zeros((13, 22, 37), np.float32), spacing=(0.7, 1.1, 2.3), origin=(-4.0, 5.5, 12.25),
                direction=direction)
    size, sp, org = shrink_geometry(img, factors)
    osz, osp, oorg = O.shrink_geometry(img.GetSize(), img.spacing, img.origin, img.direction, factors)
    assert np.array_equal(size, osz)
    assert np.array_equal(sp, osp)
    assert np.array_equal(org, oorg)
