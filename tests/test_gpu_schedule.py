"""The plain path's device-resident source schedule and its captured step graph (hs2g_set_schedule,
hs2g_set_clock / hs2g_get_clock, hs2g_run with HS2G_SCHEDULED).

hs2g_run queues the first step directly and replays a captured in-place step graph for the rest; the graph's x
sweep reads the step's class table from the handle's device schedule at the device clock, and its last kernel
advances the clock.  Each case here is compared bit for bit with the host-launched path (hs2g_run_timed, whose x
sweep takes every step's table as a kernel parameter, and hs2g_step), which the parity tests pin to the
reference's outputs: a schedule set once and run in pieces, rows past the schedule's end, rows given as a device
array, a rewound clock, the legacy default stream, per-voxel source shapes and an odd row length."""
import ctypes

import numpy as np
import pytest
import torch

import heatsim2_gb300 as hs
from heatsim2_gb300 import _native, workloads as W
from heatsim2_gb300.alternatingdirection import _ClassSources, source_table

pytestmark = pytest.mark.gpu


def _problem(shape=(24, 96, 128), nsteps=12, seed=3):
    nz, ny, nx = shape
    spec = W.composite_panel(seed=seed, nz=nz, ny=ny, nx=nx, top_layers=6, width_range=(8, 30),
                             depth_range=(2, 12), nsteps=nsteps)
    # the flash lasts two steps here (stepped source over [0, 1.5 dt]), so the schedule has active and idle rows
    spec["volumetric"][1] = ["stepped", 0.0, 1.5 * spec["dt"], 2e9]
    P, S = hs.setup(*W.setup_args(hs, spec))
    # the handle queues on the legacy default stream, torch's current stream here, so that the tensors torch
    # prepares are complete before the library reads them
    _native.check(_native.load().hs2g_set_stream(P.handle.ptr, None))
    src = _ClassSources(W.volumetric_tuple(hs, spec))
    qtabs = np.ascontiguousarray([source_table(src, t, spec["dt"], P.volume_array)[0]
                                  for t in W.step_times(spec, nsteps)])
    assert qtabs[0].any() and qtabs[1].any() and not qtabs[2:].any()
    return spec, P, qtabs


def _host_launched(P, T0, qtabs):
    """hs2g_run_timed: every step's table a kernel parameter (device tensors)."""
    L = _native.load()
    T = T0.clone()
    kms = np.zeros(4)
    q = np.ascontiguousarray(qtabs)
    _native.check(L.hs2g_run_timed(P.handle.ptr, len(q), T.data_ptr(), T.data_ptr(), q.ctypes.data,
                                   _native.DEVICE, kms.ctypes.data))
    torch.cuda.synchronize()
    return T


def _clock(P):
    v = ctypes.c_int64(-1)
    _native.check(_native.load().hs2g_get_clock(P.handle.ptr, ctypes.byref(v)))
    return v.value


def _scheduled(P, T, n, flags=_native.DEVICE | _native.SYNC):
    _native.check(_native.load().hs2g_run(P.handle.ptr, n, T.data_ptr(), T.data_ptr(), None, 0, None,
                                          flags | _native.SCHEDULED))


def test_schedule_run_in_pieces_equals_host_tables(cuda_ok):
    spec, P, qtabs = _problem()
    L = _native.load()
    T0 = torch.from_numpy(W.initial_temperature(spec)).cuda()
    ref = _host_launched(P, T0, qtabs)
    _native.check(L.hs2g_set_schedule(P.handle.ptr, len(qtabs), qtabs.ctypes.data, 0))
    assert _clock(P) == 0
    T = T0.clone()
    for n in (1, 4, 7):                       # the flash steps in the first two pieces, idle steps after
        _scheduled(P, T, n)
    assert _clock(P) == 12
    assert torch.equal(T, ref)
    assert (T - T0).abs().max().item() > 0.1
    # past the schedule's end there is no source: rows of zeros, host-launched
    _scheduled(P, T, 3)
    assert _clock(P) == 15
    ref2 = _host_launched(P, ref, np.zeros((3, _native.MAX_CLASSES)))
    assert torch.equal(T, ref2)


def test_run_with_tables_replaces_schedule_and_history(cuda_ok):
    """hs2g_run(qtabs) sets the schedule from its tables: the state and every recorded layer equal the
    host-launched steps, with T_in != T_out (first step direct, then graph replays)."""
    spec, P, qtabs = _problem(nsteps=9)
    L = _native.load()
    T0 = torch.from_numpy(W.initial_temperature(spec)).cuda()
    out = torch.empty_like(T0)
    hist = torch.empty((len(qtabs),) + tuple(T0.shape[1:]), dtype=torch.float64, device="cuda")
    _native.check(L.hs2g_run(P.handle.ptr, len(qtabs), T0.data_ptr(), out.data_ptr(), qtabs.ctypes.data, 2,
                             hist.data_ptr(), _native.DEVICE | _native.SYNC))
    assert _clock(P) == len(qtabs)
    T = T0.clone()
    for s in range(len(qtabs)):
        T = _host_launched(P, T, qtabs[s:s + 1])
        assert torch.equal(hist[s], T[2]), s
    assert torch.equal(out, T)
    # host buffers through the same call
    hout = np.empty(tuple(T0.shape))
    hhist = np.empty(tuple(hist.shape))
    T0h = W.initial_temperature(spec)
    _native.check(L.hs2g_run(P.handle.ptr, len(qtabs), T0h.ctypes.data, hout.ctypes.data, qtabs.ctypes.data, 2,
                             hhist.ctypes.data, 0))
    np.testing.assert_array_equal(hout, T.cpu().numpy())
    np.testing.assert_array_equal(hhist, hist.cpu().numpy())


def test_device_rows_and_rewound_clock(cuda_ok):
    spec, P, qtabs = _problem(nsteps=8)
    L = _native.load()
    rows = torch.from_numpy(qtabs).cuda()
    _native.check(L.hs2g_set_schedule(P.handle.ptr, len(qtabs), rows.data_ptr(), _native.DEVICE))
    del rows                                   # copied on the stream: the caller's array is not kept
    T0 = torch.from_numpy(W.initial_temperature(spec)).cuda()
    T = T0.clone()
    _scheduled(P, T, 8)
    assert torch.equal(T, _host_launched(P, T0, qtabs))
    # rewind to row 1: the second flash row first
    _native.check(L.hs2g_set_clock(P.handle.ptr, 1))
    T = T0.clone()
    _scheduled(P, T, 5)
    assert torch.equal(T, _host_launched(P, T0, qtabs[1:6]))
    assert _clock(P) == 6
    # an empty schedule: no source at all
    _native.check(L.hs2g_set_schedule(P.handle.ptr, 0, None, 0))
    T = T0.clone()
    _scheduled(P, T, 2)
    assert torch.equal(T, _host_launched(P, T0, np.zeros((2, _native.MAX_CLASSES))))


def test_scheduled_run_on_caller_streams(cuda_ok):
    """The step graph is captured on a stream of the handle's own and launched on the caller's: the legacy
    default stream and a torch side stream give the same state."""
    spec, P, qtabs = _problem(nsteps=6)
    L = _native.load()
    T0 = torch.from_numpy(W.initial_temperature(spec)).cuda()
    ref = _host_launched(P, T0, qtabs)
    for stream in (None, torch.cuda.Stream()):
        _native.check(L.hs2g_set_stream(P.handle.ptr, None if stream is None
                                        else ctypes.c_void_p(stream.cuda_stream)))
        T = T0.clone()
        torch.cuda.synchronize()
        _native.check(L.hs2g_run(P.handle.ptr, len(qtabs), T.data_ptr(), T.data_ptr(), qtabs.ctypes.data, 0, None,
                                 _native.DEVICE | _native.SYNC))
        assert torch.equal(T, ref)


@pytest.mark.parametrize("shape", [(12, 40, 64), (9, 33, 45)], ids=["even", "odd_nx"])
def test_run_with_shaped_sources_equals_single_steps(cuda_ok, shape):
    """run() with a z-decaying impulse and a point-joules source (per-voxel shapes on the device) firing inside
    the run, through the scheduled graph, against one run_adi_steps call per step (hs2g_step with host tables).
    Odd nx takes the padded-row instance of the scheduled x sweep."""
    nz, ny, nx = shape
    spec = W.composite_panel(seed=9, nz=nz, ny=ny, nx=nx, top_layers=4, width_range=(4, 12), depth_range=(2, 6),
                             nsteps=6)
    g = spec["grid"]
    P, S = hs.setup(*W.setup_args(hs, spec))
    vclass = np.zeros((g["nz"], g["ny"], g["nx"]), dtype=np.uint8)
    vclass[1:4] = 1
    vclass[5:7, 3:9, 5:11] = 2
    zc = (g["z0"] + g["dz"] * np.arange(g["nz"]))[:, None, None]
    zgrid = np.ascontiguousarray(np.broadcast_to(zc, vclass.shape))
    joules = np.random.default_rng(4).uniform(1e-4, 1e-3, int((vclass == 2).sum()))
    dt = spec["dt"]
    vol = ((hs.NO_SOURCE,),
           (hs.SPATIALLY_Z_DECAYING_TEMPORAL_IMPULSE, 2 * dt, np.array([1.0, 0.0, 0.0]), g["z0"] + 0.5 * g["dz"],
            zgrid, g["dz"], 2e4, 1.5e-3),
           (hs.IMPULSE_POINT_SOURCE_JOULES, 4 * dt, joules))
    times = W.step_times(spec, 6)
    T0 = W.initial_temperature(spec)
    T = T0
    steps = []
    for t in times:
        T = hs.run_adi_steps(P, S, t, dt, T, vclass, vol)
        steps.append(T)
    got, hist = hs.run(P, T0, times, dt, vclass, vol, record_layer=1)
    np.testing.assert_array_equal(got, steps[-1])
    for s in range(len(times)):
        np.testing.assert_array_equal(hist[s], steps[s][1])
    assert np.abs(steps[2] - steps[1]).max() > 1e-3 and np.abs(steps[4] - steps[3]).max() > 1e-6


def test_schedule_arguments(cuda_ok):
    """Bad schedule arguments are refused before anything is queued, and the handle keeps working."""
    spec, P, qtabs = _problem(shape=(8, 32, 32), nsteps=4)
    L = _native.load()
    h = P.handle.ptr
    assert L.hs2g_set_schedule(h, -1, qtabs.ctypes.data, 0) == _native.ERR_ARG
    assert L.hs2g_set_schedule(h, 3, None, 0) == _native.ERR_ARG
    assert L.hs2g_set_clock(h, -2) == _native.ERR_ARG
    assert L.hs2g_get_clock(h, None) == _native.ERR_ARG
    _native.check(L.hs2g_set_schedule(h, len(qtabs), qtabs.ctypes.data, 0))
    T0 = torch.from_numpy(W.initial_temperature(spec)).cuda()
    T = T0.clone()
    _scheduled(P, T, 4)
    assert torch.equal(T, _host_launched(P, T0, qtabs))
