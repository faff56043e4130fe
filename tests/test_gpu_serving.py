"""The serving loop: requests admitted against a memory budget, advanced together,
each result the same alone and in the mix (bitwise: a registration's blocks and
reduction orders depend only on its own inputs)."""
import numpy as np
import pytest

from cases import perturbed, small_pair
from itk_gb300 import AffineTransform, RegistrationRequest, RegistrationServer
from itk_gb300 import _capi
from itk_gb300.registration import NONE, RANDOM

pytestmark = pytest.mark.gpu

SCALES = np.array([1.0] * 9 + [1.0 / 50.0] * 3)


@pytest.fixture(scope="module")
def requests():
    sizes = [(40, 36, 32), (33, 29, 41), (48, 44, 40), (28, 30, 26), (36, 36, 36)]
    out = []
    for i, size in enumerate(sizes):
        mm = i % 2 == 1
        fixed, moving, T = small_pair(size, config=1, multimodal=mm, seed_shift=10 + i)
        U = perturbed(T, 200 + i, scale=0.02, trans=1.5)
        levels = 1 + i % 3
        out.append(RegistrationRequest(
            fixed=fixed, moving=moving, transform=U, metric="mattes" if (mm or i == 4) else "msq", bins=32,
            shrink_factors=[4, 2, 1][3 - levels:], smoothing_sigmas=[2.0, 1.0, 0.0][3 - levels:],
            sampling=RANDOM if i % 2 == 1 else NONE, sampling_percentage=0.25, seed=17 + i,
            iterations=[12, 10, 8][3 - levels:], learning_rate=0.5, minimum_step_length=1e-4, scales=SCALES))
    return out


def run_alone(req):
    s = RegistrationServer(samples_per_block=(4096, 4096, 4096))
    rid = s.submit(req)
    s.drain()
    return s.results[rid]


def same(a, b):
    assert np.array_equal(a.parameters, b.parameters), f"{a.parameters} vs {b.parameters}"
    assert a.stop_conditions == b.stop_conditions and a.iterations == b.iterations and a.values == b.values
    assert a.status == b.status


def test_mix_equals_alone(requests):
    alone = [run_alone(r) for r in requests]
    s = RegistrationServer(samples_per_block=(4096, 4096, 4096), iterations_per_tick=3)
    ids = [s.submit(r) for r in requests]
    s.drain()
    for rid, a in zip(ids, alone):
        r = s.results[rid]
        same(r, a)
        assert len(r.iterations) == requests[rid].levels
        assert r.status == _capi.GB_OK
        assert r.completed >= r.admitted >= r.arrival


def test_poisson_arrivals(requests):
    alone = [run_alone(r) for r in requests]
    rng = np.random.default_rng(3)
    arrivals = np.cumsum(rng.exponential(0.02, size=len(requests)))
    s = RegistrationServer(samples_per_block=(4096, 4096, 4096), iterations_per_tick=4)
    results, wall = s.serve(requests, arrivals)
    assert wall > 0
    for r, a in zip(results, alone):
        same(r, a)
        assert r.latency > 0


def test_admission_budget(requests):
    """A budget of about one request: the memory held never exceeds it, requests are
    admitted in arrival order, results are unchanged."""
    from itk_gb300.serving import estimate_device_bytes
    budget = max(estimate_device_bytes(r) for r in requests[:3]) * 1.01
    s = RegistrationServer(hbm_budget_bytes=budget, samples_per_block=(4096, 4096, 4096))
    ids = [s.submit(r) for r in requests[:3]]
    while not s.idle():
        s.tick()
        assert s.used_bytes <= budget
    assert s.peak_bytes <= budget
    res = [s.results[i] for i in ids]
    assert res[0].admitted <= res[1].admitted <= res[2].admitted
    for r, req in zip(res, requests[:3]):
        same(r, run_alone(req))


def test_failed_request_does_not_disturb_others(requests):
    bad_t = AffineTransform()
    bad_t.SetCenter(requests[1].transform.GetCenter())
    bad_t.SetTranslation([1e4, 0.0, 0.0])
    r1 = requests[1]
    bad = RegistrationRequest(fixed=r1.fixed, moving=r1.moving, transform=bad_t, metric="mattes", bins=32,
                              sampling=RANDOM, sampling_percentage=0.25, seed=5, iterations=[10])
    s = RegistrationServer(samples_per_block=(4096, 4096, 4096))
    ib = s.submit(bad)
    ids = [s.submit(r) for r in requests[:3]]
    s.drain()
    assert s.results[ib].status == _capi.GB_ERR_NO_VALID_POINTS
    assert s.results[ib].stop_conditions == [_capi.GB_STOP_COSTFUNCTION_ERROR]
    for rid, req in zip(ids, requests[:3]):
        same(s.results[rid], run_alone(req))
    assert s.used_bytes == 0


def test_served_results_match_oracle_registrations(requests):
    """Every request served in a mix against the oracle's restatement of its levels and
    optimizer with the same sample points: per level the same stop and iteration count
    and the final value within 1e-4 (a level's images are smoothed on the device in
    FP32, the oracle smooths in FP64); final displacement within 0.05 voxel RMS."""
    from cases import geom
    from conftest import assert_value_close
    from itk_gb300.filters import shrink_geometry
    from itk_gb300.registration import sample_points
    from oracle import registration as R

    s = RegistrationServer(samples_per_block=(4096, 4096, 4096), iterations_per_tick=3)
    ids = [s.submit(r) for r in requests]
    s.drain()
    for rid, req in zip(ids, requests):
        res = s.results[rid]
        assert res.status == _capi.GB_OK
        levels, seed = [], req.seed
        for lv in range(req.levels):
            f = req.shrink_factors[lv]
            pts = None
            if req.sampling != NONE:
                size, sp, org = shrink_geometry(req.fixed, (f, f, f))
                pts, seed = sample_points(req.sampling, size, sp, org, req.fixed.direction, req.sampling_percentage,
                                          seed)
            levels.append(dict(shrink=(f,) * 3, sigma=req.smoothing_sigmas[lv], sigma_physical=True, points=pts))
        kindcode, p0, tfixed = req.transform.flat()
        out = []
        for lv, iters in zip(levels, req.iterations):
            opt = dict(learning_rate=req.learning_rate, number_of_iterations=iters,
                       minimum_step_length=req.minimum_step_length, scales=req.scales)
            p0, r = R.register(req.metric, req.fixed.array, geom(req.fixed), req.moving.array, geom(req.moving),
                               kindcode, p0, tfixed, [lv], opt, bins=req.bins)
            out.append(r[0])
        assert res.stop_conditions == [r["stop"] for r in out]
        assert res.iterations == [r["iterations"] for r in out]
        for got, r in zip(res.values, out):
            assert_value_close(got, r["value"], rtol=1e-4)
        T1 = AffineTransform()
        T1.SetCenter(req.transform.GetCenter())
        T1.SetParameters(res.parameters)
        T2 = AffineTransform()
        T2.SetCenter(req.transform.GetCenter())
        T2.SetParameters(p0)
        nx, ny, nz = req.fixed.GetSize()
        g = np.stack(np.meshgrid(*(np.arange(0, n, 3) for n in (nx, ny, nz)), indexing="ij"), -1).reshape(-1, 3)
        x = g.astype(np.float64) @ req.fixed.index_to_physical().T + req.fixed.origin
        dd = (T1.TransformPoint(x) - T2.TransformPoint(x)) / req.fixed.spacing
        rms = float(np.sqrt(np.mean(np.sum(dd * dd, axis=1))))
        assert rms <= 0.05, f"request {rid}: displacement RMS {rms:.4f} voxel"
