"""Serving: whole affine registrations arrive over time and advance together.

A request is a complete ImageRegistrationMethodv4 job (fixed and moving image,
metric, pyramid levels, sampling, RegularStep settings per level).  The server
admits requests in arrival order while the device memory they hold stays under
the HBM budget and a slot is free; every admitted request keeps its images,
level pyramid, samples and optimizer state on the device; one scheduling tick
advances every running registration by a few iterations in one batched launch
per phase (RegistrationBatch).  A request that finishes a level is set up for
the next one (device smoothing and shrink, host sample points) and rejoins the
batch; a request that finishes its last level frees its memory and slot.  A
registration's result is the same alone and in any mix: its blocks and
reduction orders depend only on its own inputs.
"""
from __future__ import annotations

import time
from concurrent.futures import FIRST_COMPLETED, ThreadPoolExecutor, wait
from dataclasses import dataclass, field

import numpy as np

from . import _capi
from ._capi import ExceptionObject
from .batch import RegistrationBatch
from .image import Image
from .metrics import MattesMutualInformationImageToImageMetricv4, MeanSquaresImageToImageMetricv4
from .optimizers import RegularStepGradientDescentOptimizerv4
from .registration import NONE, RANDOM, sample_count, setup_level
from .transforms import AffineTransform


@dataclass
class RegistrationRequest:
    fixed: Image
    moving: Image
    transform: AffineTransform            # initial transform (copied; the request's result is a new one)
    metric: str = "mattes"                # "mattes" or "msq"
    bins: int = 50
    shrink_factors: list = field(default_factory=lambda: [1])
    smoothing_sigmas: list = field(default_factory=lambda: [0.0])
    sigmas_in_physical_units: bool = True
    sampling: int = RANDOM                # registration.NONE / REGULAR / RANDOM
    sampling_percentage: float = 0.2
    seed: int = 0                         # MetricSamplingReinitializeSeed
    iterations: list = field(default_factory=lambda: [100])   # per level
    learning_rate: float = 1.0
    minimum_step_length: float = 1e-4
    relaxation_factor: float = 0.5
    gradient_magnitude_tolerance: float = 1e-4
    scales: object = None

    @property
    def levels(self) -> int:
        return len(self.shrink_factors)


@dataclass
class RegistrationResult:
    request_id: int
    parameters: np.ndarray
    stop_conditions: list
    iterations: list
    values: list
    status: int
    error: str
    arrival: float
    admitted: float
    completed: float

    @property
    def latency(self) -> float:
        return self.completed - self.arrival


def estimate_device_bytes(req: RegistrationRequest) -> int:
    """Device memory a request holds at its finest level, before it is admitted:
    fixed and moving images and their smoothed copies (4 B each per voxel), the
    packed moving value + gradient (16 B per voxel), samples and caches (32 B per
    sample) and the per-handle scratch."""
    vf = int(np.prod(req.fixed.GetSize()))
    vm = int(np.prod(req.moving.GetSize()))
    smooth = any(s > 0 for s in req.smoothing_sigmas)
    img = (vf + vm) * 4 * (2 if smooth else 1) + vm * 16
    n = vf if req.sampling == NONE else sample_count(req.sampling, req.fixed.GetSize(), req.sampling_percentage)
    return img + 32 * n + (1 << 20)


class _Job:
    def __init__(self, rid, req, arrival):
        self.rid = rid
        self.req = req
        self.arrival = arrival
        self.admitted = None
        self.level = 0
        self.seed = req.seed
        self.metric = None
        self.optimizer = None
        self.transform = None
        self.slot = None
        self.setup = None      # future of the level set-up running on a worker thread
        self.bytes = 0
        self.stops, self.iters, self.values = [], [], []


class RegistrationServer:
    """hbm_budget_bytes: device memory the admitted requests may hold together;
    max_active: registrations in flight; iterations_per_tick: iterations between
    scheduling decisions; setup_threads: host threads that set up levels (image
    upload, device smoothing and gradient, sample points) while the batch runs."""

    def __init__(self, hbm_budget_bytes: float = 120e9, max_active: int = 64, iterations_per_tick: int = 8,
                 samples_per_block=(8192, 8192, 8192), device: int = 0, clock=time.perf_counter,
                 setup_threads: int = 4):
        self.budget = float(hbm_budget_bytes)
        self.max_active = int(max_active)
        self.k = int(iterations_per_tick)
        self.clock = clock
        self.device = device
        self.batch = RegistrationBatch(device)
        self.batch.SetSamplesPerBlock(*samples_per_block)
        self.pool = ThreadPoolExecutor(max_workers=max(1, int(setup_threads)))
        self.pending = []      # arrival order
        self.active = {}       # rid -> _Job
        self.results = {}      # rid -> RegistrationResult
        self.used_bytes = 0
        self.peak_bytes = 0
        self.setup_seconds = 0.0   # worker-thread time spent setting up levels
        self.setups = 0
        self.upload_seconds = 0.0  # of which: metric creation and image upload (first level)
        self.run_seconds = 0.0     # main thread: inside the batch's iterations
        self.ticks = 0
        self._next = 0

    def __del__(self):
        try:
            self.pool.shutdown(wait=True)
        except Exception:
            pass

    # ---- requests
    def submit(self, req: RegistrationRequest, arrival: float = None) -> int:
        rid = self._next
        self._next += 1
        self.pending.append(_Job(rid, req, self.clock() if arrival is None else arrival))
        return rid

    def idle(self) -> bool:
        return not self.pending and not self.active

    # ---- scheduling
    def _admit(self):
        while self.pending and len(self.active) < self.max_active:
            job = self.pending[0]
            need = estimate_device_bytes(job.req)
            if self.used_bytes + need > self.budget and self.active:
                break  # wait for memory to free up (arrival order is kept)
            self.pending.pop(0)
            job.admitted = self.clock()
            job.bytes = need
            self.used_bytes += need
            self.active[job.rid] = job
            job.setup = self.pool.submit(self._setup_level, job)
        self.peak_bytes = max(self.peak_bytes, self.used_bytes)

    def _setup_level(self, job):
        """Worker thread: the request's metric (first level), the level's set-up and
        Initialize, and its optimizer; returns the device bytes the metric holds."""
        t0 = time.perf_counter()
        try:
            return self._setup_level_timed(job)
        finally:
            self.setup_seconds += time.perf_counter() - t0
            self.setups += 1

    def _setup_level_timed(self, job):
        r = job.req
        if job.metric is None:
            t_up = time.perf_counter()
            m = MeanSquaresImageToImageMetricv4(self.device) if r.metric == "msq" else \
                MattesMutualInformationImageToImageMetricv4(self.device)
            if r.metric != "msq":
                m.SetNumberOfHistogramBins(r.bins)
            m.SetFixedImage(r.fixed)
            m.SetMovingImage(r.moving)
            t = AffineTransform()
            t.SetCenter(r.transform.GetCenter())
            t.SetParameters(r.transform.GetParameters())
            m.SetMovingTransform(t)
            job.metric, job.transform = m, t
            self.upload_seconds += time.perf_counter() - t_up
        lv = job.level
        shrink = r.shrink_factors[lv]
        shrink = np.full(3, int(shrink)) if np.ndim(shrink) == 0 else np.asarray(shrink)
        _, job.seed = setup_level(job.metric, r.fixed, shrink, r.smoothing_sigmas[lv], r.sigmas_in_physical_units,
                                  r.sampling, r.sampling_percentage, job.seed)
        o = RegularStepGradientDescentOptimizerv4()
        o.SetMetric(job.metric)
        o.SetLearningRate(r.learning_rate)
        o.SetMinimumStepLength(r.minimum_step_length)
        o.SetRelaxationFactor(r.relaxation_factor)
        o.SetGradientMagnitudeTolerance(r.gradient_magnitude_tolerance)
        o.SetNumberOfIterations(int(r.iterations[lv]))
        o.SetScales(r.scales)
        job.optimizer = o
        return job.metric.GetDeviceBytes()

    def _join_ready(self, block: bool):
        """Registrations whose level set-up has finished join the batch."""
        waiting = [j for j in self.active.values() if j.setup is not None]
        if block and waiting and not any(j.setup.done() for j in waiting):
            wait([j.setup for j in waiting], return_when=FIRST_COMPLETED)
        for job in waiting:
            if not job.setup.done():
                continue
            fut, job.setup = job.setup, None
            try:
                actual = fut.result()
            except ExceptionObject as e:
                self._complete(job, e.code, str(e))
                continue
            self.used_bytes += actual - job.bytes
            self.peak_bytes = max(self.peak_bytes, self.used_bytes)
            job.bytes = actual
            job.slot = self.batch.Add(job.optimizer)

    def _complete(self, job, status, error):
        self.results[job.rid] = RegistrationResult(
            job.rid, job.transform.GetParameters().copy() if job.transform is not None else None, job.stops,
            job.iters, job.values, status, error, job.arrival, job.admitted, self.clock())
        del self.active[job.rid]
        self.used_bytes -= job.bytes
        job.metric = None  # frees its device memory

    def _finish_level(self, job):
        o = job.optimizer
        job.slot = None
        job.stops.append(o.GetStopCondition())
        job.iters.append(o.GetCurrentIteration())
        job.values.append(o.GetValue())
        status = getattr(o, "_batch_status", _capi.GB_OK)
        if status == _capi.GB_OK and job.level + 1 < job.req.levels:
            job.level += 1
            job.setup = self.pool.submit(self._setup_level, job)
            return
        self._complete(job, status, getattr(o, "_batch_error", ""))

    def tick(self):
        """Admit what fits, let finished level set-ups join, advance every running
        registration by up to iterations_per_tick iterations, then hand finished
        levels to the set-up threads."""
        self._admit()
        if not self.active:
            return
        running = any(j.slot is not None for j in self.active.values())
        self._join_ready(block=not running)
        if not any(j.slot is not None for j in self.active.values()):
            return
        t_run = time.perf_counter()
        self.batch.Run(self.k)
        self.run_seconds += time.perf_counter() - t_run
        self.ticks += 1
        for job in list(self.active.values()):
            if job.slot is not None and not self.batch.IsRunning(job.slot):
                self._finish_level(job)

    def drain(self):
        while not self.idle():
            self.tick()

    def serve(self, requests, arrivals):
        """Serve `requests` arriving at the given offsets (seconds from now); returns
        the results in request order and the wall time of the whole run."""
        order = np.argsort(np.asarray(arrivals, dtype=np.float64), kind="stable")
        t0 = self.clock()
        ids = [None] * len(requests)
        i = 0
        while i < len(order) or not self.idle():
            now = self.clock() - t0
            while i < len(order) and arrivals[order[i]] <= now:
                ids[order[i]] = self.submit(requests[order[i]], t0 + arrivals[order[i]])
                i += 1
            if self.idle():
                if i < len(order):
                    time.sleep(max(0.0, min(arrivals[order[i]] - now, 0.01)))
                continue
            self.tick()
        return [self.results[r] for r in ids], self.clock() - t0
