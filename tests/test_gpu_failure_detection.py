"""Failure detection without a GPU fault.

A bounded device wait that runs out reports HS2G_ERR_TIMEOUT and leaves the context usable (the same wait
guards every mbarrier of the TMA sweeps); a device allocation that cannot succeed returns HS2G_ERR_NOMEM with
nothing leaked and the handle usable; host-side validation errors are covered with the parity tests."""
import ctypes
import time

import numpy as np
import pytest

from conftest import load_golden, rel_err, GOLDEN
import heatsim2_gb300 as hs
from heatsim2_gb300 import _native, workloads as W

pytestmark = pytest.mark.gpu


def _wait(limit_ns, arrive):
    st = ctypes.c_int(12345)
    t = time.perf_counter()
    rc = _native.load().hs2g_selftest_wait(0, limit_ns, arrive, ctypes.byref(st))
    return rc, st.value, time.perf_counter() - t


def _step_still_works():
    spec, times, ref = load_golden(GOLDEN + "/mixed_small.npz")
    P, S = hs.setup(*W.setup_args(hs, spec))
    T = W.initial_temperature(spec)
    vol = W.volumetric_tuple(hs, spec)
    for n, t in enumerate(times):
        T = hs.run_adi_steps(P, S, t, spec["dt"], T, spec["arrays"]["volumetric"], vol)
    assert rel_err(T, ref[len(times)]) <= 1e-12


def test_bounded_wait_reports_timeout_and_context_survives(cuda_ok):
    rc, status, elapsed = _wait(200_000_000, 0)          # 0.2 s, no arrival
    assert rc == _native.OK and status == _native.ERR_TIMEOUT
    assert 0.15 <= elapsed < 5.0
    rc, status, elapsed = _wait(200_000_000, 1)          # the arrival comes: no wait
    assert rc == _native.OK and status == _native.OK and elapsed < 0.15
    _step_still_works()


def test_wait_limit_is_validated(cuda_ok):
    st = ctypes.c_int(0)
    L = _native.load()
    assert L.hs2g_selftest_wait(0, 0, 0, ctypes.byref(st)) == _native.ERR_ARG
    assert L.hs2g_selftest_wait(0, 20_000_000_000, 0, ctypes.byref(st)) == _native.ERR_ARG


def test_device_allocation_failure_is_reported(cuda_ok):
    """A forward pass whose checkpoint store cannot be allocated (2^21 states of 2^20 voxels, 16 TB: the first
    cudaMalloc fails, nothing is partially filled) returns HS2G_ERR_NOMEM; the handle stays usable."""
    import torch
    L = _native.load()
    free0 = torch.cuda.mem_get_info()[0]
    n, nsteps = 1 << 20, 1 << 21
    g = (_native.AdjointGrid * 1)(_native.AdjointGrid(n, 1, 1, 1e-3, 1e-3, 1e-3))
    h = ctypes.c_void_p()
    assert L.hs2g_adjoint_create(1, g, 0.01, 0, ctypes.byref(h)) == _native.OK
    try:
        k, C, q = np.full(n, 50.0), np.full(n, 3.6e6), np.zeros(n)
        assert L.hs2g_adjoint_set_parameters(h, k.ctypes.data, C.ctypes.data, q.ctypes.data, 0) == _native.OK
        sched, obs, T0, loss = np.zeros(nsteps), np.zeros(nsteps), np.zeros(n), np.zeros(1)
        rc = L.hs2g_adjoint_forward(h, nsteps, sched.ctypes.data, T0.ctypes.data, obs.ctypes.data, 1,
                                    loss.ctypes.data, None, 0, None)
        assert rc == _native.ERR_NOMEM
        assert b"alloc" in L.hs2g_last_error().lower() or b"memory" in L.hs2g_last_error().lower()
        # the same handle still runs a forward pass that fits
        assert L.hs2g_adjoint_forward(h, 1, sched.ctypes.data, T0.ctypes.data, obs.ctypes.data, 1,
                                      loss.ctypes.data, None, 0, None) == _native.OK
        assert loss[0] == 0.0
    finally:
        L.hs2g_adjoint_destroy(h)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] >= free0 - (64 << 20)   # everything was released
    _step_still_works()


def test_oversized_adjoint_is_refused_before_allocating(cuda_ok):
    """2^31 voxels or more (27 per-voxel FP64 fields: over 464 GB) are refused with HS2G_ERR_ARG."""
    L = _native.load()
    g = (_native.AdjointGrid * 1)(_native.AdjointGrid(4096, 4096, 4096, 1e-3, 1e-3, 1e-3))
    h = ctypes.c_void_p()
    assert L.hs2g_adjoint_create(1, g, 0.01, 0, ctypes.byref(h)) == _native.ERR_ARG
    assert not h.value
    assert b"2^31" in L.hs2g_last_error()
    _step_still_works()
