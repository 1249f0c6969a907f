"""GPU parity: the CUDA path (libhs2g through heatsim2_gb300.setup / run_adi_steps) against the reference's
golden outputs and the oracle.  Bar: max|T_gpu - T_ref| / max|T_ref| <= 1e-12 (FP64, the tolerance the
reference comparison is specified at)."""
import numpy as np
import pytest

from conftest import golden_files, load_golden, rel_err, GOLDEN
import oracle
from oracle_shim import HS
import heatsim2_gb300 as hs
from heatsim2_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _setup(spec):
    return hs.setup(*W.setup_args(hs, spec))


def _run_host(spec, times, P, S, T=None):
    vol = W.volumetric_tuple(hs, spec)
    T = W.initial_temperature(spec) if T is None else T
    out = {}
    for n, t in enumerate(times):
        T = hs.run_adi_steps(P, S, t, spec["dt"], T, spec["arrays"]["volumetric"], vol)
        out[n + 1] = T
    return out


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.rsplit("/", 1)[-1])
def test_golden_parity(cuda_ok, path):
    spec, times, ref = load_golden(path)
    P, S = _setup(spec)
    got = _run_host(spec, times, P, S)
    for n, T in ref.items():
        assert rel_err(got[n], T) <= TOL, (n, rel_err(got[n], T))


def test_device_tensor_path_equals_host_path(cuda_ok):
    import torch
    spec, times, ref = load_golden(GOLDEN + "/steel_slab.npz")
    P, S = _setup(spec)
    vol = W.volumetric_tuple(hs, spec)
    T = torch.from_numpy(W.initial_temperature(spec)).cuda()
    host = _run_host(spec, times[:50], P, S)
    for n, t in enumerate(times[:50]):
        T = hs.run_adi_steps(P, S, t, spec["dt"], T, spec["arrays"]["volumetric"], vol)
    np.testing.assert_array_equal(T.cpu().numpy(), host[50])
    assert rel_err(T.cpu().numpy(), ref[50]) <= TOL


@pytest.mark.parametrize("shape", [(16, 256, 256), (17, 250, 240)])
def test_overlapped_host_copies_equal_device_path(cuda_ok, shape):
    """Host-buffer steps of >= 2^20 voxels upload in slabs of planes and download in blocks of rows while the
    sweeps run; the result is the device path's bit for bit (uneven slab and block sizes included)."""
    import torch
    nz, ny, nx = shape
    spec = W.composite_panel(seed=4, nz=nz, ny=ny, nx=nx, top_layers=4, width_range=(10, 40), depth_range=(2, 10),
                             nsteps=3)
    assert W.voxels(spec) >= 1 << 20
    P, S = _setup(spec)
    vol = W.volumetric_tuple(hs, spec)
    times = W.step_times(spec)
    host = _run_host(spec, times, P, S)
    T = torch.from_numpy(W.initial_temperature(spec)).cuda()
    for t in times:
        T = hs.run_adi_steps(P, S, t, spec["dt"], T, spec["arrays"]["volumetric"], vol)
    np.testing.assert_array_equal(T.cpu().numpy(), host[len(times)])


def test_run_equals_single_steps_and_records_history(cuda_ok):
    spec, times, ref = load_golden(GOLDEN + "/sources_small.npz")
    P, S = _setup(spec)
    vol = W.volumetric_tuple(hs, spec)
    host = _run_host(spec, times, P, S)
    T, hist = hs.run(P, W.initial_temperature(spec), times, spec["dt"], spec["arrays"]["volumetric"], vol,
                     record_layer=0)
    np.testing.assert_array_equal(T, host[len(times)])
    for n in range(len(times)):
        np.testing.assert_array_equal(hist[n], host[n + 1][0])


def test_run_device_many_steps(cuda_ok):
    import torch
    spec, times, ref = load_golden(GOLDEN + "/steel_slab.npz")
    P, S = _setup(spec)
    vol = W.volumetric_tuple(hs, spec)
    T0 = torch.from_numpy(W.initial_temperature(spec)).cuda()
    T, hist = hs.run(P, T0, times, spec["dt"], spec["arrays"]["volumetric"], vol, record_layer=0)
    assert rel_err(T.cpu().numpy(), ref[200]) <= TOL
    assert rel_err(hist[9].cpu().numpy(), ref[10][0]) <= TOL
    assert torch.equal(T0, torch.from_numpy(W.initial_temperature(spec)).cuda())   # input untouched


def _coo_dense(z, prefix, n):
    M = np.zeros((n, n))
    np.add.at(M, (z[prefix + "_row"], z[prefix + "_col"]), z[prefix + "_val"])
    return M


@pytest.mark.parametrize("name", ["mixed_small", "sources_small"])
def test_compiled_stage_matrices_match_reference(cuda_ok, name):
    """The device coefficient compiler produces the reference's stage matrices (pyadi_step.Amat/Bmat/Cmats/Dvec)."""
    spec, _, _ = load_golden(GOLDEN + "/%s.npz" % name)
    st = np.load(GOLDEN + "/stages_%s.npz" % name)
    P, S = _setup(spec)
    n = W.voxels(spec)
    for s in range(3):
        np.testing.assert_allclose(S[s].Amat, st["A_%d" % s], rtol=1e-14, atol=0)
        np.testing.assert_array_equal(S[s].Dvec, st["D_%d" % s])
        np.testing.assert_allclose(S[s].Bmat.toarray(), _coo_dense(st, "B_%d" % s, n), rtol=1e-13, atol=1e-6)
        for c in range(s):
            np.testing.assert_allclose(S[s].Cmats[c].toarray(), _coo_dense(st, "C_%d_%d" % (s, c), n),
                                       rtol=1e-13, atol=1e-6)
        assert S[s].permuteorder == tuple(st["perm_%d" % s])


def _compare_with_oracle(spec, nsteps, tol=TOL):
    P, S = _setup(spec)
    Po, _ = oracle.setup(*W.setup_args(HS, spec))
    vol = W.volumetric_tuple(hs, spec)
    volo = W.volumetric_tuple(HS, spec)
    T = W.initial_temperature(spec)
    To = T.copy()
    worst = 0.0
    for n, t in enumerate(W.step_times(spec, nsteps)):
        T = hs.run_adi_steps(P, S, t, spec["dt"], T, spec["arrays"]["volumetric"], vol)
        To = oracle.run_adi_steps(Po, None, t, spec["dt"], To, spec["arrays"]["volumetric"], volo)
        worst = max(worst, rel_err(T, To))
    assert worst <= tol, worst
    return T


def test_fixed_planes_at_both_ends_vs_oracle(cuda_ok):
    """Planes of fixed voxels at the top (the ambient layer) and at the bottom: host-buffer steps match the
    oracle, and a run in place on the device matches the single steps."""
    spec = W.composite_panel(seed=8, nz=20, ny=40, nx=48, top_layers=6, width_range=(4, 12), depth_range=(2, 12),
                             nsteps=6)
    spec["arrays"]["material"][-2:] = 2             # two fixed planes at the bottom
    T = _compare_with_oracle(spec, 6)
    import torch
    P, S = _setup(spec)
    got = hs.run(P, torch.from_numpy(W.initial_temperature(spec)).cuda(), W.step_times(spec, 6), spec["dt"],
                 spec["arrays"]["volumetric"], W.volumetric_tuple(hs, spec))
    np.testing.assert_array_equal(got.cpu().numpy(), T)


def test_composite_panel_midsize_vs_oracle(cuda_ok):
    spec = W.composite_panel(seed=3, nz=40, ny=96, nx=80, top_layers=10, width_range=(8, 30),
                             depth_range=(3, 30))
    _compare_with_oracle(spec, 25)


@pytest.mark.parametrize("shape", [(20, 70, 66), (9, 33, 41), (13, 48, 80)])
def test_sweep_kernel_variants_agree_bitwise(cuda_ok, monkeypatch, shape):
    """Every selectable sweep kernel does the same FMAs in the same order, so the results are identical: TMA
    bulk-copy or plain-load y / z sweeps, the plain z sweep with or without dropping its forward values from
    L2 (planes of a multiple of 16 voxels, as 48x80, let whole warps drop them), and the y sweep's arrays
    unpadded (even nx) or padded to a row pitch of 64 (odd nx always gets one pad column, so that the TMA sweep
    applies)."""
    nz, ny, nx = shape
    spec = W.composite_panel(seed=5, nz=nz, ny=ny, nx=nx, top_layers=4, width_range=(5, 20), depth_range=(2, 6))
    outs = []
    variants = (("tma", "plain", "2", "1"), ("plain", "tma", "2", "1"), ("plain", "plain", "2", "1"),
                ("tma", "plain", "64", "1"), ("plain", "plain", "64", "1"), ("tma", "plain", "2", "0"))
    for y_mode, z_mode, pitch, discard in variants:
        monkeypatch.setenv("HS2G_LINE_SWEEP", y_mode)
        monkeypatch.setenv("HS2G_Z_SWEEP", z_mode)
        monkeypatch.setenv("HS2G_Z_DISCARD", discard)
        monkeypatch.setenv("HS2G_ROW_PITCH", pitch)   # rows of the y-sweep arrays padded to this multiple
        P, S = _setup(spec)
        outs.append(_run_host(spec, W.step_times(spec, 5), P, S)[5])
    for o in outs[1:]:
        np.testing.assert_array_equal(outs[0], o)


def test_uneven_instances_vs_oracle(cuda_ok):
    for spec in W.uneven_batch(seed=2, n=3, nz_range=(16, 24), nxy_range=(40, 70)):
        _compare_with_oracle(spec, 6)


def test_full_size_composite_panel_first_steps_vs_oracle(cuda_ok):
    """The benchmark workload itself (65x512x512 with the ambient layer), the bench's timed step count (20
    steps, the flash included) against the oracle, every step."""
    spec = W.composite_panel(seed=1)
    _compare_with_oracle(spec, 20)


def test_composite_panel_128_device_run_vs_reference(cuda_ok):
    """The benchmark's composite-panel recipe at 65x128x128 (reference-generated fixture, 100 steps): the
    device-resident multi-step path (hs.run on a CUDA tensor) at steps 1, 20 and 100."""
    import torch
    spec, times, ref = load_golden(GOLDEN + "/composite_panel_128.npz")
    assert sorted(ref) == [1, 20, 100]
    P, S = _setup(spec)
    vol = W.volumetric_tuple(hs, spec)
    T = torch.from_numpy(W.initial_temperature(spec)).cuda()
    done = 0
    for n in (1, 20, 100):
        T = hs.run(P, T, times[done:n], spec["dt"], spec["arrays"]["volumetric"], vol)
        done = n
        assert rel_err(T.cpu().numpy(), ref[n]) <= TOL, (n, rel_err(T.cpu().numpy(), ref[n]))


def _class_sources(spec, P, t):
    from heatsim2_gb300.alternatingdirection import _ClassSources, source_table
    q, _ = source_table(_ClassSources(W.volumetric_tuple(hs, spec)), t, spec["dt"], P.volume_array)
    return q


@pytest.mark.parametrize("name", ["mixed_small", "steel_slab"])
def test_dense_handle_from_compiled_faces_vs_reference(cuda_ok, name):
    """hs2g_create_dense fed the compiled face conductances, capacities and fixed mask of a reference fixture
    (P.faces()) reproduces the reference's temperatures: the dense entry point is pinned to the reference, not
    only to the class-compiled path."""
    import ctypes
    from heatsim2_gb300 import _native
    spec, times, ref = load_golden(GOLDEN + "/%s.npz" % name)
    P, S = _setup(spec)
    Gz, Gy, Gx, M, fixed = P.faces()
    vclass = np.ascontiguousarray(spec["arrays"]["volumetric"], dtype=np.uint8)
    nz, ny, nx = P.shape
    L = _native.load()
    dense = _native.DenseProblem(nz, ny, nx, Gz.ctypes.data, Gy.ctypes.data, Gx.ctypes.data, M.ctypes.data,
                                 fixed.ctypes.data, vclass.ctypes.data)
    h = ctypes.c_void_p()
    _native.check(L.hs2g_create_dense(ctypes.byref(dense), P.device, ctypes.byref(h)))
    try:
        T = W.initial_temperature(spec)
        for n, t in enumerate(times):
            q = _class_sources(spec, P, t)
            out = np.empty_like(T)
            _native.check(L.hs2g_step(h, T.ctypes.data, out.ctypes.data, q.ctypes.data, None, None, 0))
            T = out
            if n + 1 in ref:
                assert rel_err(T, ref[n + 1]) <= TOL, (n + 1, rel_err(T, ref[n + 1]))
    finally:
        L.hs2g_destroy(h)


def test_full_size_energy_conservation(cuda_ok):
    """Insulated composite panel at full size: with every exterior face insulating and no fixed voxels the
    Douglas step conserves energy exactly in real arithmetic (the conductance operator has zero column sums),
    so sum(rho*c*dT)*V equals the injected source energy to rounding."""
    import torch
    spec = W.composite_panel(seed=1)
    a = spec["arrays"]
    a["material"][0] = 0                        # ambient layer becomes composite
    a["boundary_z"][1] = 0                      # joined by the conducting class
    P, S = _setup(spec)
    vol = W.volumetric_tuple(hs, spec)
    T0 = torch.from_numpy(W.initial_temperature(spec)).cuda()
    times = W.step_times(spec, 12)
    T = hs.run(P, T0, times, spec["dt"], a["volumetric"], vol)
    rc = np.where(a["material"] == 0, 1550.0 * 1100.0, 2700.0 * 900.0)
    dV = spec["grid"]["dz"] * spec["grid"]["dy"] * spec["grid"]["dx"]
    energy = float(((T - T0).cpu().numpy() * rc).sum() * dV)
    injected = 2e9 * spec["dt"] * dV * float((a["volumetric"] == 1).sum())
    assert abs(energy - injected) <= 1e-9 * injected, (energy, injected)


def test_uniform_state_is_steady(cuda_ok):
    spec = W.composite_panel(seed=1, nz=16, ny=64, nx=64, top_layers=4, width_range=(4, 20), depth_range=(2, 12))
    spec["volumetric"] = [["none"], ["none"]]
    P, S = _setup(spec)
    T = W.initial_temperature(spec)
    for t in W.step_times(spec, 5):
        T = hs.run_adi_steps(P, S, t, spec["dt"], T, spec["arrays"]["volumetric"], W.volumetric_tuple(hs, spec))
    assert np.abs(T - 293.0).max() <= 1e-12 * 293.0


def test_in_place_device_step(cuda_ok):
    import torch
    from heatsim2_gb300 import _native
    spec, times, ref = load_golden(GOLDEN + "/mixed_small.npz")
    P, S = _setup(spec)
    T = torch.from_numpy(W.initial_temperature(spec)).cuda()
    L = _native.load()
    from heatsim2_gb300.alternatingdirection import _ClassSources, source_table
    src = _ClassSources(W.volumetric_tuple(hs, spec))
    for t in times:
        q, _ = source_table(src, t, spec["dt"], P.volume_array)
        _native.check(L.hs2g_set_stream(P.handle.ptr, torch.cuda.current_stream().cuda_stream))
        _native.check(L.hs2g_step(P.handle.ptr, T.data_ptr(), T.data_ptr(), q.ctypes.data, None, None,
                                  _native.DEVICE | _native.SYNC))
    assert rel_err(T.cpu().numpy(), ref[len(times)]) <= TOL


def test_replaced_source_class_map(cuda_ok):
    spec = W.steel_slab(seed=4, nz=8, ny=12, nx=10, flaw=4, depth_range=(2, 5))
    P, S = _setup(spec)
    Po, _ = oracle.setup(*W.setup_args(HS, spec))
    other = np.zeros_like(spec["arrays"]["volumetric"])
    other[:, 3:6, 2:7] = 1
    vol, volo = W.volumetric_tuple(hs, spec), W.volumetric_tuple(HS, spec)
    T = To = W.initial_temperature(spec)
    for t in W.step_times(spec, 3):
        T = hs.run_adi_steps(P, S, t, spec["dt"], T, other, vol)
        To = oracle.run_adi_steps(Po, None, t, spec["dt"], To, other, volo)
    assert rel_err(T, To) <= TOL


def test_dense_source_on_device(cuda_ok):
    import torch
    spec, times, ref = load_golden(GOLDEN + "/sources_small.npz")
    P, S = _setup(spec)
    vol = W.volumetric_tuple(hs, spec)
    T = torch.from_numpy(W.initial_temperature(spec)).cuda()
    for t in times:
        T = hs.run_adi_steps(P, S, t, spec["dt"], T, spec["arrays"]["volumetric"], vol)
    assert rel_err(T.cpu().numpy(), ref[len(times)]) <= TOL


def test_per_voxel_sources_on_device_at_full_size(cuda_ok, monkeypatch):
    """A z-decaying impulse and an array-valued point source on the benchmark grid (65x512x512, class map
    replaced by the call).  Their values are evaluated on the device (pyx:307-384): a repeat firing step with the
    same z coordinates uploads nothing but T (the z-coordinate array stays on the device, the shape call is
    flagged REUSE and no per-voxel field goes up), and the step equals one given the source field as the
    reference's numpy loop forms it (oracle restatement) within 1e-12."""
    import ctypes
    from heatsim2_gb300 import _native
    spec = W.composite_panel(seed=1)
    g = spec["grid"]
    nz, ny, nx = g["nz"], g["ny"], g["nx"]
    P, S = _setup(spec)
    vclass = np.zeros((nz, ny, nx), dtype=np.uint8)
    vclass[1:9] = 1                                     # z-decaying absorption in the top compute layers
    vclass[20:26, 100:140, 300:330] = 2                 # a buried block with per-voxel point energies
    zc = (g["z0"] + g["dz"] * np.arange(nz))[:, None, None]
    zgrid = np.ascontiguousarray(np.broadcast_to(zc, (nz, ny, nx)))
    rng = np.random.default_rng(17)
    joules = rng.uniform(1e-4, 1e-3, int((vclass == 2).sum()))

    def vol(jpm2):
        return ((hs.NO_SOURCE,),
                (hs.SPATIALLY_Z_DECAYING_TEMPORAL_IMPULSE, 0.0, np.array([1.0, 0.0, 0.0]), g["z0"] + 0.5 * g["dz"],
                 zgrid, g["dz"], jpm2, 1.5e-3),
                (hs.IMPULSE_POINT_SOURCE_JOULES, 0.0, joules))

    L = _native.load()
    calls = []
    for name in ("hs2g_source_zdecay", "hs2g_source_point", "hs2g_set_source_classes", "hs2g_step"):
        fn = getattr(L, name)

        def spy(*args, _fn=fn, _name=name):
            calls.append((_name, args))
            return _fn(*args)
        monkeypatch.setattr(L, name, spy)
    T0 = W.initial_temperature(spec)
    first = hs.run_adi_steps(P, S, 0.0, spec["dt"], T0, vclass, vol(2e4))
    assert {c[0] for c in calls} >= {"hs2g_source_zdecay", "hs2g_source_point", "hs2g_set_source_classes"}
    calls.clear()
    second_vol = vol(3e4)                               # new amplitude, same z coordinates and joules
    second = hs.run_adi_steps(P, S, 0.0, spec["dt"], T0, vclass, second_vol)
    names = [c[0] for c in calls]
    assert "hs2g_set_source_classes" not in names       # the class map is already on the device
    assert "hs2g_source_point" not in names             # unchanged source: its shape is kept
    (zcall,) = [c for c in calls if c[0] == "hs2g_source_zdecay"]
    assert zcall[1][-1] & _native.REUSE                 # z coordinates reused from the device copy
    (step,) = [c for c in calls if c[0] == "hs2g_step"]
    assert step[1][4] is None and step[1][5] is None    # no per-voxel source field, no class map uploaded
    # the same step with the reference-form source field handed over explicitly
    from oracle_shim import HS
    Q = oracle.source_field(P.shape, P.volume_array, 0.0, spec["dt"], vclass, second_vol)
    assert Q[1].max() > 0 and Q[vclass == 2].min() > 0
    ref = np.empty_like(T0)
    _native.check(L.hs2g_step(P.handle.ptr, T0.ctypes.data, ref.ctypes.data, None, Q.ctypes.data, None, 0))
    assert rel_err(second, ref) <= TOL, rel_err(second, ref)
    assert np.abs(first - T0).max() > 0.1 and np.abs(second - first).max() > 0.01


# ---- errors where the reference errors (or silently computes outside the domain) ----------------------
def _expect_setup_error(spec, exc):
    with pytest.raises(exc):
        _setup(spec)


def test_conducting_exterior_face_is_rejected(cuda_ok):
    for key, sl in (("boundary_x", (slice(None), slice(None), -1)), ("boundary_y", (slice(None), 0)),
                    ("boundary_z", (0,))):
        spec = W.line_grid((3, 4, 5))
        spec["arrays"][key][sl] = 0
        _expect_setup_error(spec, ValueError)


def test_scalar_class_on_matrix_k_is_rejected(cuda_ok):
    spec = W.line_grid((3, 4, 5))
    spec["materials"][0][1] = W.COMPOSITE_K
    _expect_setup_error(spec, ValueError)


def test_unaligned_anisotropy_is_rejected(cuda_ok):
    spec = W.line_grid((3, 4, 5))
    spec["materials"][0][1] = [[5.0, 0.3, 0.0], [0.3, 5.0, 0.0], [0.0, 0.0, 5.0]]
    spec["boundaries"][0] = ["conducting_anisotropic"]
    with pytest.raises(AssertionError):
        _setup(spec)


def test_zero_capacity_is_rejected(cuda_ok):
    spec = W.line_grid((3, 4, 5))
    spec["materials"][0][2] = 0.0
    _expect_setup_error(spec, ValueError)


def test_fixed_voxels_hold_their_temperature(cuda_ok):
    spec, times, ref = load_golden(GOLDEN + "/mixed_small.npz")
    P, S = _setup(spec)
    got = _run_host(spec, times, P, S)
    fixed = spec["arrays"]["material"] == 3
    assert fixed.any()
    np.testing.assert_array_equal(got[len(times)][fixed], 293.0)


def test_install_as_heatsim2_runs_user_boundary_module(cuda_ok):
    import sys
    import types
    hs.install_as_heatsim2()
    try:
        from heatsim2.expression import group   # the name user boundary classes import
        m = types.ModuleType("user_thin")

        def q(kl, kh, dz, dy, dx, Tl, Th, *rest):
            return -1000.0 * group(Th - Tl)
        m.qz = m.qy = m.qx = q
        spec = W.steel_slab(seed=0, nz=6, ny=8, nx=8, flaw=3, depth_range=(2, 3))
        args = list(W.setup_args(hs, spec))
        args[11] = (args[11][0], args[11][1], (m,))      # user module in place of the thin-layer class
        P, S = sys.modules["heatsim2"].setup(*args)
        Po, _ = oracle.setup(*W.setup_args(HS, spec))
        T = To = W.initial_temperature(spec)
        vol, volo = W.volumetric_tuple(hs, spec), W.volumetric_tuple(HS, spec)
        for t in W.step_times(spec, 4):
            T = hs.run_adi_steps(P, S, t, spec["dt"], T, spec["arrays"]["volumetric"], vol)
            To = oracle.run_adi_steps(Po, None, t, spec["dt"], To, spec["arrays"]["volumetric"], volo)
        assert rel_err(T, To) <= TOL
    finally:
        for k in [k for k in sys.modules if k == "heatsim2" or k.startswith("heatsim2.")]:
            del sys.modules[k]
