"""The curved-surface mode on the GPU (hs2g_create_rows) against the reference's own outputs.

The curved golden fixtures are the reference run in its curved-surface mode (crank_nicolson.pyx:388-457,
tests/golden/make_golden.py); heatsim2_gb300.setup with the same curvature arrays must reproduce them to
1e-12 through host and device buffers."""
import ctypes

import numpy as np
import pytest

from conftest import golden_files, load_golden, rel_err
import heatsim2_gb300 as hs
from heatsim2_gb300 import _native, workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.mark.parametrize("path", golden_files(curved=True), ids=lambda p: p.rsplit("/", 1)[-1])
def test_curved_golden_parity(cuda_ok, path):
    import torch
    spec, times, ref = load_golden(path)
    P, S = hs.setup(*W.setup_args(hs, spec), **W.setup_kwargs(spec))
    assert np.ndim(P.volume_array) == 3
    vol = W.volumetric_tuple(hs, spec)
    T = W.initial_temperature(spec)
    Td = torch.from_numpy(W.initial_temperature(spec)).cuda()
    for n, t in enumerate(times):
        T = hs.run_adi_steps(P, S, t, spec["dt"], T, spec["arrays"]["volumetric"], vol)
        Td = hs.run_adi_steps(P, S, t, spec["dt"], Td, spec["arrays"]["volumetric"], vol)
        if n + 1 in ref:
            assert rel_err(T, ref[n + 1]) <= TOL, (n + 1)
    np.testing.assert_array_equal(Td.cpu().numpy(), T)


def test_curved_problem_has_no_shared_faces(cuda_ok):
    spec = W.curved(W.mixed_small(), seed=3)
    P, S = hs.setup(*W.setup_args(hs, spec), **W.setup_kwargs(spec))
    L = _native.load()
    g = np.zeros(P.shape[0] + 1)
    assert L.hs2g_get_faces(P.handle.ptr, g.ctypes.data, None, None, None, None) == _native.ERR_STATE
    cap = np.zeros(P.shape)
    assert L.hs2g_get_faces(P.handle.ptr, None, None, None, cap.ctypes.data, None) == _native.OK


def test_rows_problem_rejects_conducting_exterior(cuda_ok):
    shape = (3, 4, 5)
    rows = {n: np.zeros(shape) for n in ("zlo", "zhi", "ylo", "yhi", "xlo", "xhi")}
    rows["ylo"][:, 1:] = 10.0
    rows["ylo"][0, 0, 2] = 3.0               # an exterior side of a computed voxel
    cap = np.full(shape, 1e5)
    rp = _native.RowsProblem(*shape, *[rows[n].ctypes.data for n in ("zlo", "zhi", "ylo", "yhi", "xlo", "xhi")],
                             cap.ctypes.data, None, None)
    h = ctypes.c_void_p()
    L = _native.load()
    assert L.hs2g_create_rows(ctypes.byref(rp), 0, ctypes.byref(h)) == _native.ERR_EXTERIOR
    rows["ylo"][0, 0, 2] = 0.0
    cap[1, 2, 3] = 0.0                        # zero capacity on a computed voxel
    assert L.hs2g_create_rows(ctypes.byref(rp), 0, ctypes.byref(h)) == _native.ERR_CAPACITY
    cap[1, 2, 3] = 1e5
    assert L.hs2g_create_rows(ctypes.byref(rp), 0, ctypes.byref(h)) == _native.OK
    L.hs2g_destroy(h)
