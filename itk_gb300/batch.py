"""Many affine registrations advancing together on one GPU (gb_batch_* in the C ABI).

Each registration is an initialized metric with a
RegularStepGradientDescentOptimizerv4 holding its settings; one optimizer
iteration of every running registration is one graph launch of a kernel per phase
(or, in the persistent form, one kernel launch carries several iterations).  A registration's
result does not depend on the others in the batch.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import ExceptionObject, OptimizerReport, RegularStepSettings, check, i64, ptr
from .metrics import context


class RegistrationBatch:
    def __init__(self, device: int = 0):
        self._L = _capi.lib()
        self._h = ctypes.c_void_p()
        check(self._L.gb_batch_create(context(device), ctypes.byref(self._h)))
        self._slots = {}  # slot -> (metric, optimizer)

    def __del__(self):
        try:
            if getattr(self, "_h", None) and self._h.value:
                self._L.gb_batch_destroy(self._h)
                self._h = ctypes.c_void_p()
        except Exception:
            pass

    def Add(self, optimizer) -> int:
        """StartOptimization of the optimizer's (initialized) metric inside the batch; returns its slot."""
        m = optimizer.GetMetric()
        if m is None:
            raise ExceptionObject(_capi.GB_ERR_BAD_ARG, "m_Metric must be set.")
        m._sync_params()
        s = RegularStepSettings(optimizer.GetLearningRate(), optimizer.GetRelaxationFactor(),
                                optimizer.GetMinimumStepLength(), optimizer.GetGradientMagnitudeTolerance(),
                                optimizer.GetNumberOfIterations(), int(optimizer.GetReturnBestParametersAndValue()))
        scales = optimizer.GetScales()
        slot = ctypes.c_int64()
        check(self._L.gb_batch_add(self._h, m.handle, ctypes.byref(s), ptr(scales),
                                   0 if scales is None else scales.size, ctypes.byref(slot)))
        self._slots[slot.value] = (m, optimizer)
        return slot.value

    def Run(self, max_iterations: int = 0) -> int:
        """Advance by up to max_iterations iterations (0: until every registration
        has stopped); returns how many are still running.  Finished registrations
        have their transforms and optimizer reports updated."""
        running = ctypes.c_int64()
        check(self._L.gb_batch_run(self._h, int(max_iterations), ctypes.byref(running)))
        for slot in list(self._slots):
            self._finish(slot)
        return int(running.value)

    def _finish(self, slot):
        m, opt = self._slots[slot]
        fin = ctypes.c_int()
        rep = OptimizerReport()
        rc = self._L.gb_batch_result(self._h, slot, ctypes.byref(fin), ctypes.byref(rep))
        if not fin.value:
            return
        del self._slots[slot]
        p = np.zeros(m._nparams)
        check(self._L.gb_metric_get_parameters(m.handle, ptr(p), p.size))
        m.GetMovingTransform().SetParameters(p)
        opt._report = rep
        m._value = rep.value
        opt._batch_status = rc
        opt._batch_error = _capi.last_error() if rc != _capi.GB_OK else ""

    def IsRunning(self, slot: int) -> bool:
        return slot in self._slots

    def SetSamplesPerBlock(self, msq: int, pass1: int, pass2: int):
        check(self._L.gb_batch_set_samples_per_block(self._h, ptr(i64([msq, pass1, pass2]))))

    def GetSamplesPerBlock(self):
        out = np.zeros(3, np.int64)
        check(self._L.gb_batch_get_samples_per_block(self._h, ptr(out)))
        return tuple(int(x) for x in out)

    def Autotune(self, iterations: int = 3):
        """Times the batch's evaluations for each samples-per-block candidate (no
        optimizer state changes) and keeps the fastest; returns the choice."""
        out = np.zeros(3, np.int64)
        check(self._L.gb_batch_autotune(self._h, int(iterations), ptr(out)))
        return tuple(int(x) for x in out)

    def GetStats(self):
        """(iterations launched, table rebuilds, host seconds spent rebuilding)."""
        it, rb, sec = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double()
        check(self._L.gb_batch_get_stats(self._h, ctypes.byref(it), ctypes.byref(rb), ctypes.byref(sec)))
        return int(it.value), int(rb.value), float(sec.value)

    def SetUseCudaGraphs(self, on: bool):
        check(self._L.gb_batch_set_graphs(self._h, int(bool(on))))

    def SetPersistent(self, on: bool):
        """Several iterations of every registration per kernel launch, or (default) one
        launch per phase and iteration; the results are bitwise the same."""
        check(self._L.gb_batch_set_persistent(self._h, int(bool(on))))
