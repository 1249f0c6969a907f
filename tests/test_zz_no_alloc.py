"""hs2g_step_static, the timestep entry point that allocates no device memory, against hs2g_step and against
the reference's own outputs.

hs2g_step_static is for callers that cannot allocate device memory themselves -- a plugin whose host
application owns every device allocation.  It takes the problem (face conductances, capacities, fixed mask,
source) in caller-owned device memory and keeps its intermediates in a static device array, so it must give the
same timestep as a compiled handle (hs2g_create_dense + hs2g_step) on the same inputs.  The tensors below are
allocated by the test, not by the entry point.  Tolerance: 1e-12 relative max error, as for every GPU parity
test.  Two calls in a row check that the shared array's leftover contents do not leak into the next call; the
reference fixtures (tests/golden) pin the entry point to the reference itself over whole runs.
"""
import ctypes

import numpy as np
import pytest

from conftest import GOLDEN, load_golden, rel_err
import heatsim2_gb300 as hs
from heatsim2_gb300 import _native
from heatsim2_gb300 import workloads as W

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


def _source_field(spec, P, t):
    """The per-voxel source (W/m^3) of a fixture at time t, as the reference's numpy loop forms it (the
    oracle's restatement of alternatingdirection_c_pyx.pyx:294-386)."""
    import oracle
    from oracle_shim import HS
    return np.ascontiguousarray(oracle.source_field(P.shape, P.volume_array, t, spec["dt"],
                                                    np.asarray(spec["arrays"]["volumetric"]),
                                                    W.volumetric_tuple(HS, spec)))


@pytest.mark.parametrize("name", ["mixed_small", "sources_small", "steel_slab"])
def test_static_step_vs_reference_fixture(cuda_ok, name):
    """hs2g_step_static fed a reference fixture's compiled faces (P.faces()) and its sources as a per-voxel
    field reproduces the reference's temperatures within 1e-12: the no-allocation step is pinned to the
    reference itself (fixed voxels, every source kind and the 200-step steel slab)."""
    import torch
    L = _native.load()
    spec, times, ref = load_golden(GOLDEN + "/%s.npz" % name)
    P, _ = hs.setup(*W.setup_args(hs, spec))
    Gz, Gy, Gx, M, fixed = P.faces()
    nz, ny, nx = P.shape
    dev = torch.device("cuda", P.device)
    g = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
         for k, v in dict(Gz=Gz, Gy=Gy, Gx=Gx, M=M, fixed=fixed).items()}
    stream = torch.cuda.current_stream(dev)
    T = torch.from_numpy(W.initial_temperature(spec)).to(dev)
    out = torch.empty_like(T)
    for n, t in enumerate(times):
        Q = torch.from_numpy(_source_field(spec, P, t)).to(dev)
        _native.check(L.hs2g_step_static(nz, ny, nx, g["Gz"].data_ptr(), g["Gy"].data_ptr(), g["Gx"].data_ptr(),
                                         g["M"].data_ptr(), g["fixed"].data_ptr(), Q.data_ptr(), T.data_ptr(),
                                         out.data_ptr(), ctypes.c_void_p(stream.cuda_stream)))
        T, out = out, T
        if n + 1 in ref:
            err = rel_err(T.cpu().numpy(), ref[n + 1])
            assert err <= TOL, (n + 1, err)


def test_static_step_rejects_bad_capacity(cuda_ok):
    """A computed voxel with a non-positive capacity is reported (HS2G_ERR_CAPACITY, with its index), and the
    next call with valid inputs succeeds: the status word is cleared per call."""
    import torch
    L = _native.load()
    Gz, Gy, Gx, M, fixed, Q, T = _problem(7, nz=4, ny=5, nx=6)
    fixed[:] = 0
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream()
    bad_values = ((0.0, _native.ERR_CAPACITY), (-3.0, _native.ERR_CAPACITY), (float("nan"), _native.ERR_CAPACITY),
                  (None, _native.OK))
    for bad, expect in bad_values:
        Mb = M.copy()
        if bad is not None:
            Mb[2, 3, 4] = bad
        d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
             for k, v in dict(Gz=Gz, Gy=Gy, Gx=Gx, M=Mb, fixed=fixed, T=T).items()}
        out = torch.empty_like(d["T"])
        rc = L.hs2g_step_static(4, 5, 6, d["Gz"].data_ptr(), d["Gy"].data_ptr(), d["Gx"].data_ptr(),
                                d["M"].data_ptr(), d["fixed"].data_ptr(), None, d["T"].data_ptr(),
                                out.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        assert rc == expect, (bad, rc, L.hs2g_last_error())
        if bad is not None:
            assert b"[2,3,4]" in L.hs2g_last_error()
