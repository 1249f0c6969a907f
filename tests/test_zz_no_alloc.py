"""hs2g_step_static, the timestep entry point that allocates no device memory, against hs2g_step.

hs2g_step_static is for callers that cannot allocate device memory themselves -- a plugin whose host
application owns every device allocation.  It takes the problem (face conductances, capacities, fixed mask,
source) in caller-owned device memory and keeps its intermediates in a static device array, so it must give the
same timestep as a compiled handle (hs2g_create_dense + hs2g_step) on the same inputs.  The tensors below are
allocated by the test, not by the entry point.  Tolerance: 1e-12 relative max error, as for every GPU parity
test.  Two calls in a row check that the shared array's leftover contents do not leak into the next call.
"""
import ctypes

import numpy as np
import pytest

from heatsim2_gb300 import _native

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _problem(seed, nz=9, ny=14, nx=17):
    rng = np.random.default_rng(seed)
    Gz = rng.uniform(1e5, 1e6, (nz + 1, ny, nx))
    Gy = rng.uniform(1e5, 1e6, (nz, ny + 1, nx))
    Gx = rng.uniform(1e5, 1e6, (nz, ny, nx + 1))
    Gz[0] = Gz[-1] = 0.0                       # insulating exterior
    Gy[:, 0] = Gy[:, -1] = 0.0
    Gx[:, :, 0] = Gx[:, :, -1] = 0.0
    Gz[4, 3:9, 2:11] = 0.0                     # an insulating flaw
    M = rng.uniform(2e5, 8e5, (nz, ny, nx))
    fixed = (rng.random((nz, ny, nx)) < 0.05).astype(np.uint8)
    Q = rng.uniform(0.0, 1e8, (nz, ny, nx)) * (rng.random((nz, ny, nx)) < 0.3)
    T = 293.0 + rng.uniform(0.0, 5.0, (nz, ny, nx))
    return Gz, Gy, Gx, M, fixed, Q, T


def test_static_step_matches_compiled_step_on_two_calls(cuda_ok):
    import torch
    L = _native.load()
    Gz, Gy, Gx, M, fixed, Q, T = _problem(31)
    nz, ny, nx = T.shape
    dense = _native.DenseProblem(nz, ny, nx, Gz.ctypes.data, Gy.ctypes.data, Gx.ctypes.data, M.ctypes.data,
                                 fixed.ctypes.data, None)
    h = ctypes.c_void_p()
    _native.check(L.hs2g_create_dense(ctypes.byref(dense), torch.cuda.current_device(), ctypes.byref(h)))
    try:
        dev = torch.device("cuda", torch.cuda.current_device())
        d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
             for k, v in dict(Gz=Gz, Gy=Gy, Gx=Gx, M=M, fixed=fixed, Q=Q, T=T).items()}
        stream = torch.cuda.current_stream()
        _native.check(L.hs2g_set_stream(h, ctypes.c_void_p(stream.cuda_stream)))
        t_ref, t_new = d["T"].clone(), d["T"].clone()
        for call in range(2):
            out_ref, out_new = torch.empty_like(t_ref), torch.empty_like(t_new)
            _native.check(L.hs2g_step(h, t_ref.data_ptr(), out_ref.data_ptr(), None, d["Q"].data_ptr(), None,
                                      _native.DEVICE))
            _native.check(L.hs2g_step_static(nz, ny, nx, d["Gz"].data_ptr(), d["Gy"].data_ptr(),
                                             d["Gx"].data_ptr(), d["M"].data_ptr(), d["fixed"].data_ptr(),
                                             d["Q"].data_ptr(), t_new.data_ptr(), out_new.data_ptr(),
                                             ctypes.c_void_p(stream.cuda_stream)))
            torch.cuda.synchronize()
            ref, new = out_ref.cpu().numpy(), out_new.cpu().numpy()
            err = float(np.abs(new - ref).max() / np.abs(ref).max())
            assert err <= TOL, (call, err)
            assert np.abs(ref - T).max() > 1e-3          # the step actually changed the field
            assert np.array_equal(new[fixed == 1], t_new.cpu().numpy()[fixed == 1])
            t_ref, t_new = out_ref, out_new
    finally:
        L.hs2g_destroy(h)


def test_static_step_rejects_grids_beyond_the_maximum(cuda_ok):
    L = _native.load()
    nz, ny, nx = 128, 128, 65          # 1,064,960 voxels > HS2G_STATIC_MAX_VOXELS
    assert nz * ny * nx > _native.STATIC_MAX_VOXELS
    dummy = ctypes.c_void_p(16)        # never dereferenced: the size check comes first
    rc = L.hs2g_step_static(nz, ny, nx, dummy, dummy, dummy, dummy, None, None, dummy, dummy, None)
    assert rc == _native.ERR_ARG
    assert b"HS2G_STATIC_MAX_VOXELS" in L.hs2g_last_error()
