"""The surface-temperature estimate on the GPU: libhs2g hs2g_surface_temperature / hs2g_run_surface.

The device estimate of a field equals the oracle's restatement of the reference's function (which the CPU
tests pin to the reference bit for bit) on the same field, for host and device inputs; ``run(...,
record_surface=True)`` records after every step exactly the estimate of that step's layers 0 and 1, also
across steps that take the single-step path (per-voxel sources)."""
import ctypes
import os

import numpy as np
import pytest
import torch

import oracle
import heatsim2_gb300 as hs
from heatsim2_gb300 import _native, workloads as W
from heatsim2_gb300.surface_temperature import insulating_z_min_surface_temperature

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "surface_temperature.npz")


def test_fields_match_oracle_host_and_device(cuda_ok):
    d = np.load(GOLDEN)
    for c in range(5):
        T, dz = d["T_%d" % c], float(d["dz_%d" % c])
        ref = oracle.insulating_z_min_surface_temperature(T, dz)
        np.testing.assert_array_equal(insulating_z_min_surface_temperature(T, dz), ref)
        out = insulating_z_min_surface_temperature(torch.tensor(T, device="cuda"), dz)
        np.testing.assert_array_equal(out.cpu().numpy(), ref)
        # against the reference's own values (computed where the fixture was made)
        assert np.abs(ref - d["surface_%d" % c]).max() <= 1e-13 * np.abs(d["surface_%d" % c]).max()


def _setup(spec):
    return hs.setup(*W.setup_args(hs, spec), **W.setup_kwargs(spec))


@pytest.mark.parametrize("spec", [W.steel_slab(nsteps=12), W.sources_small()], ids=["steel_slab", "sources"])
def test_run_records_surface_after_every_step(cuda_ok, spec):
    P, S = _setup(spec)
    vol = W.volumetric_tuple(hs, spec)
    times = W.step_times(spec)
    ve = spec["arrays"]["volumetric"]
    T0 = W.initial_temperature(spec)
    T, hist = hs.run(P, T0, times, spec["dt"], ve, vol, record_surface=True)
    _, lay0 = hs.run(P, T0, times, spec["dt"], ve, vol, record_layer=0)
    T2, lay1 = hs.run(P, T0, times, spec["dt"], ve, vol, record_layer=1)
    np.testing.assert_array_equal(T, T2)
    dz = spec["grid"]["dz"]
    for s in range(len(times)):
        np.testing.assert_array_equal(hist[s], oracle.insulating_z_min_surface_temperature(
            np.stack([lay0[s], lay1[s]]), dz))
    Td = torch.tensor(T0, device="cuda")
    Tdev, hdev = hs.run(P, Td, times, spec["dt"], ve, vol, record_surface=True)
    np.testing.assert_array_equal(hdev.cpu().numpy(), hist)
    np.testing.assert_array_equal(Tdev.cpu().numpy(), T)


def test_arguments(cuda_ok):
    spec = W.steel_slab(nsteps=2)
    P, S = _setup(spec)
    vol = W.volumetric_tuple(hs, spec)
    ve = spec["arrays"]["volumetric"]
    T0 = W.initial_temperature(spec)
    with pytest.raises(ValueError):
        hs.run(P, T0, [0.0], spec["dt"], ve, vol, record_layer=0, record_surface=True)
    L = _native.load()
    hist = np.empty((1,) + T0.shape[1:])
    out = np.empty_like(T0)
    rc = L.hs2g_run_surface(P.handle.ptr, 1, T0.ctypes.data, out.ctypes.data, None, 0.0, hist.ctypes.data, 0)
    assert rc == _native.ERR_ARG
    rc = L.hs2g_surface_temperature(0, 1, 4, 4, T0.ctypes.data, 1e-3, out.ctypes.data, None, 0)
    assert rc == _native.ERR_ARG
