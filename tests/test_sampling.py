"""Metric sample points (no GPU needed).

The oracle's MT19937 is pinned by the reference's own known answers
(itkMersenneTwisterRandomVariateGeneratorGTest.cxx: the std::mt19937
conformance value and the seed-1234 sequence) and its normal variates by the
same test's statistics; the library's host sampler (gb_sample_points) must then
equal the oracle's SetMetricSamplePoints restatement bit for bit."""
import numpy as np
import pytest

from itk_gb300 import sample_count, sample_points
from itk_gb300.registration import RANDOM, REGULAR
from oracle import oracle as O


def rotation(ax, deg):
    t = np.deg2rad(deg)
    c, s = np.cos(t), np.sin(t)
    R = np.eye(3)
    i, j = [(1, 2), (0, 2), (0, 1)][ax]
    R[i, i], R[i, j], R[j, i], R[j, j] = c, -s, s, c
    return R


def test_mt_conforms_with_std_mt19937_requirement():
    # the 10000th output of a generator seeded with 5489 is 4123659995
    assert int(O.mt_sequence(5489, 1, skip=9999)[0]) == 4123659995


def test_mt_seed_1234_known_sequence():
    # SetSeed(1234), 200 draws, then the reference's five expected values
    got = O.mt_sequence(1234, 5, skip=200)
    assert got.tolist() == [3294740812, 4175194053, 3041332341, 199851601, 3422518480]


def test_mt_matches_numpy_legacy_mt19937():
    bg = np.random.MT19937()
    if not hasattr(bg, "_legacy_seeding"):
        pytest.skip("numpy without legacy MT19937 seeding")
    for seed in (0, 1, 77, 2**31 + 5):
        bg._legacy_seeding(seed)
        assert np.array_equal(bg.random_raw(1500).astype(np.uint32), O.mt_sequence(seed, 1500))


def test_normal_variate_statistics():
    x = O.mt_normals(4321, 500000)
    assert abs(x.mean()) < 0.01 and abs(x.var() - 1.0) < 0.01


@pytest.mark.parametrize("strategy,pct", [(RANDOM, 0.2), (RANDOM, 0.013), (REGULAR, 0.1), (REGULAR, 0.33),
                                          (RANDOM, 1.0)])
def test_sample_count(strategy, pct):
    size = (37, 29, 23)
    V = 37 * 29 * 23
    want = int(np.float64(np.float32(V)) * pct) if strategy == RANDOM else len(range(0, V, int(np.ceil(1 / pct))))
    assert sample_count(strategy, size, pct) == want


@pytest.mark.parametrize("strategy", [RANDOM, REGULAR])
@pytest.mark.parametrize("geometry", [
    ((24, 20, 18), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), np.eye(3)),
    ((33, 17, 26), (0.7, 1.3, 2.1), (-11.5, 4.25, 30.0), rotation(2, 25) @ rotation(0, -10)),
    ((64, 64, 50), (4.0, 4.0, 4.0), (1.5, 1.5, 1.5), np.eye(3)),
])
@pytest.mark.parametrize("seed", [0, 12345, -7])
def test_sample_points_match_oracle(strategy, geometry, seed):
    size, sp, org, R = geometry
    pct = 0.2 if strategy == RANDOM else 0.1
    pts, nxt = sample_points(strategy, size, sp, org, R, pct, seed)
    want = O.sample_points(1 if strategy == REGULAR else 2, size, sp, org, R, pct, seed)
    assert pts.dtype == np.float32 and pts.shape == want.shape
    assert np.array_equal(pts.view(np.uint32), want.view(np.uint32))
    assert nxt == seed + (2 if strategy == RANDOM else 1)


def test_random_points_lie_in_domain():
    size, sp, org = (30, 26, 20), np.array([1.5, 1.0, 2.0]), np.array([3.0, -2.0, 5.0])
    pts, _ = sample_points(RANDOM, size, sp, org, np.eye(3), 0.5, 99)
    ci = (pts.astype(np.float64) - org) / sp
    # a jitter of N(0, 1/3 voxel) stays within 2 voxels of the grid in practice
    assert ci.min() > -2.0 and np.all(ci.max(0) < np.asarray(size) + 1.0)
    # voxels drawn with replacement, roughly uniform over the domain
    vox = np.floor(ci + 0.5).clip(0, np.asarray(size) - 1).astype(int)
    assert abs(vox[:, 0].mean() - (size[0] - 1) / 2) < 1.0


def test_seed_sequence_over_levels():
    # RANDOM consumes two seeds per level (jitter generator, then voxel iterator)
    size, sp, org = (20, 20, 20), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0)
    a, s1 = sample_points(RANDOM, size, sp, org, np.eye(3), 0.1, 40)
    b, s2 = sample_points(RANDOM, size, sp, org, np.eye(3), 0.1, s1)
    assert (s1, s2) == (42, 44)
    assert not np.array_equal(a, b)
    c, _ = sample_points(RANDOM, size, sp, org, np.eye(3), 0.1, 40)
    assert np.array_equal(a, c)


def test_sampling_percentage_range():
    # itkImageRegistrationSamplingTest: 0.1 is accepted; -0.1, 0 and 1.1 raise
    from itk_gb300 import ExceptionObject, ImageRegistrationMethodv4
    r = ImageRegistrationMethodv4()
    r.SetMetricSamplingPercentage(0.1)
    for bad in (-0.1, 0.0, 1.1):
        with pytest.raises(ExceptionObject):
            r.SetMetricSamplingPercentage(bad)
    r.SetNumberOfLevels(3)
    r.SetMetricSamplingPercentagePerLevel([0.2, 0.5, 1.0])
    with pytest.raises(ExceptionObject):
        r.SetMetricSamplingPercentagePerLevel([0.2, 1.5, 1.0])
