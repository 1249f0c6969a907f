"""The adjoint's mathematics, checked on the CPU before any GPU run.

1. ``torch_adi`` (the small FP64 PyTorch ADI that autograd differentiates) is pinned to the oracle -- itself
   pinned to the reference's outputs -- on a multi-material class problem with conducting interior faces
   and an insulating exterior, the per-voxel form of the reference's step.
2. ``adjoint_model`` (libhs2g's adjoint kernels restated in numpy, checkpoint bookkeeping included) agrees
   with autograd through ``torch_adi`` for every checkpoint interval: the derivation of the discrete
   adjoint is exact to rounding.
3. The adjoint workloads are deterministic and shaped as documented."""
import numpy as np
import pytest
import torch

from conftest import rel_err
import adjoint_model as AM
import oracle
import torch_adi as TA
from oracle_shim import HS
import heatsim2_gb300 as hs
from heatsim2_gb300 import workloads as W


def _multi_material(seed=11, shape=(5, 6, 7), d=(1e-3, 1.1e-3, 0.9e-3), dt=0.02):
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    mats = [(HS.TEMPERATURE_COMPUTE, 54.0, 7850.0, 470.0), (HS.TEMPERATURE_COMPUTE, 0.4, 40.0, 1500.0),
            (HS.TEMPERATURE_COMPUTE, 167.0, 2700.0, 900.0)]
    me = rng.integers(0, 3, size=shape).astype(np.uint8)
    a = {"boundary_z": np.zeros((nz + 1, ny, nx), np.uint8), "boundary_y": np.zeros((nz, ny + 1, nx), np.uint8),
         "boundary_x": np.zeros((nz, ny, nx + 1), np.uint8)}
    a["boundary_z"][[0, -1]] = 1
    a["boundary_y"][:, [0, -1]] = 1
    a["boundary_x"][:, :, [0, -1]] = 1
    ve = np.zeros(shape, np.uint8)
    ve[0] = 1
    vol = ((HS.NO_SOURCE,), (HS.STEPPED_SOURCE, 0.0, 0.5 * dt, 3e8))
    args = (0.0, 0.0, 0.0, d[0], d[1], d[2], nz, ny, nx, dt, tuple(mats),
            ((HS.boundary_conducting,), (HS.boundary_insulating,)), vol, me, a["boundary_z"], a["boundary_y"],
            a["boundary_x"], ve)
    k = np.array([m[1] for m in mats])[me]
    C = np.array([m[2] * m[3] for m in mats])[me]
    return args, k, C, ve, vol


def test_torch_adi_matches_oracle():
    args, k, C, ve, vol = _multi_material()
    P, _ = oracle.setup(*args)
    shape, d, dt = (args[6], args[7], args[8]), args[3:6], args[9]
    T = np.full(shape, 293.0) + np.random.default_rng(1).random(shape)
    Tt = torch.tensor(T)
    times = [dt * n for n in range(6)]
    for t in times:
        Q = oracle.source_field(shape, d[0] * d[1] * d[2], t, dt, ve, vol)
        T = oracle.run_adi_steps(P, None, t, dt, T, ve, vol)
        Tt = TA.step(Tt, torch.tensor(k), torch.tensor(C), torch.tensor(Q), 1.0, dt, d)
        assert rel_err(Tt.numpy(), T) <= 1e-13
        assert np.abs(Tt.numpy() - T).max() <= 1e-11


def _random_problem(seed, shape, N):
    rng = np.random.default_rng(seed)
    sp = (1e-3, 1.2e-3, 0.9e-3)
    k = 54 * np.exp(0.3 * rng.standard_normal(shape))
    C = 7850 * 470 * (1 + 0.2 * rng.random(shape))
    q = rng.random(shape) * 1e8
    T0 = 293 + rng.random(shape)
    sched = rng.random(N)
    obs = 293 + rng.random((N,) + shape[1:])
    return k, C, q, T0, sched, obs, sp


@pytest.mark.parametrize("shape", [(4, 5, 6), (1, 3, 4), (3, 1, 5), (2, 4, 1)])
@pytest.mark.parametrize("ckpt", [1, 3, 7, 100])
def test_adjoint_model_matches_autograd(shape, ckpt):
    N, dt = 7, 0.01
    k, C, q, T0, sched, obs, sp = _random_problem(0, shape, N)
    tk = [torch.tensor(a, requires_grad=True) for a in (k, C, q, T0)]
    J = TA.misfit(tk[3], tk[0], tk[1], tk[2], sched, torch.tensor(obs), dt, sp)
    J.backward()
    m = AM.Model(k, C, q, dt, sp)
    Jm = m.forward(T0, sched, obs, ckpt)
    assert abs(Jm - J.item()) <= 1e-13 * J.item()
    for g, t in zip(m.backward(), tk):
        assert rel_err(g, t.grad.numpy()) <= 1e-12


def test_adjoint_model_matches_central_differences():
    """Autograd and the adjoint agree with central differences of the loss (torch_adi in FP64)."""
    N, dt = 5, 0.01
    shape = (3, 4, 5)
    k, C, q, T0, sched, obs, sp = _random_problem(2, shape, N)
    m = AM.Model(k, C, q, dt, sp)
    m.forward(T0, sched, obs, 2)
    gk, gC, gq, _ = m.backward()

    def J(k_, C_, q_):
        return TA.misfit(torch.tensor(T0), torch.tensor(k_), torch.tensor(C_), torch.tensor(q_), sched,
                         torch.tensor(obs), dt, sp).item()

    rng = np.random.default_rng(5)
    for idx in [tuple(int(rng.integers(0, n)) for n in shape) for _ in range(6)]:
        for which, (arr, g) in enumerate(((k, gk), (C, gC), (q, gq))):
            h = 1e-4 * abs(arr[idx]) if arr[idx] != 0 else 1.0
            p = [k.copy(), C.copy(), q.copy()]
            p[which][idx] += h
            Jp = J(*p)
            p[which][idx] -= 2 * h
            Jm = J(*p)
            fd = (Jp - Jm) / (2 * h)
            assert abs(fd - g[idx]) <= 1e-5 * max(abs(g[idx]), 1e-3 * np.abs(g).max()), (which, idx)


def _flaw_problem(seed=13, shape=(6, 7, 8), d=(1e-3, 1.1e-3, 0.9e-3), dt=0.02):
    """A class problem with every face kind the forward path has: steel and a composite-like scalar-k material,
    a thin insulating layer patch (h = 1000) and an insulating delamination inside, insulating exterior, a
    fixed-temperature bottom layer and two fixed voxels inside, a flash on the top layer."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    mats = [(HS.TEMPERATURE_COMPUTE, 54.0, 7850.0, 470.0), (HS.TEMPERATURE_COMPUTE, 5.0, 1550.0, 1100.0),
            (HS.TEMPERATURE_FIXED, 0.0, 0.0, 0.0)]
    me = rng.integers(0, 2, size=shape).astype(np.uint8)
    me[-1] = 2
    me[2, 3, 4] = me[3, 1, 6] = 2
    bz = np.zeros((nz + 1, ny, nx), np.uint8)
    by = np.zeros((nz, ny + 1, nx), np.uint8)
    bx = np.zeros((nz, ny, nx + 1), np.uint8)
    bz[[0, -1]] = 1
    by[:, [0, -1]] = 1
    bx[:, :, [0, -1]] = 1
    bz[2, 1:5, 2:6] = 2          # thin insulating layer
    bz[4, 3:6, 1:4] = 1          # delamination
    bx[1:3, 2:5, 4] = 2          # a thin layer across x
    ve = np.zeros(shape, np.uint8)
    ve[0] = 1
    vol = ((HS.NO_SOURCE,), (HS.STEPPED_SOURCE, 0.0, 0.5 * dt, 3e8))
    bnd = ((HS.boundary_conducting,), (HS.boundary_insulating,), (HS.boundary_thininsulatinglayer, 1000.0))
    args = (0.0, 0.0, 0.0, d[0], d[1], d[2], nz, ny, nx, dt, tuple(mats), bnd, vol, me, bz, by, bx, ve)
    k = np.array([54.0, 5.0, 17.0])[me]          # a fixed voxel's own k never matters
    C = np.array([7850.0 * 470.0, 1550.0 * 1100.0, 1.0e6])[me]
    fixed = me == 2
    # the same classes as the package's boundary modules, which the adjoint evaluates into face forms
    pkg = ((hs.boundary_conducting,), (hs.boundary_insulating,), (hs.boundary_thininsulatinglayer, 1000.0))
    return args, k, C, fixed, (pkg, bz, by, bx), ve, vol


def test_torch_adi_with_face_classes_matches_oracle():
    """The PyTorch ADI with face classes and fixed voxels (the adjoint's reference model) reproduces the oracle
    on a class problem with thin-layer, insulating and conducting faces and fixed voxels; the face forms come
    from the adjoint's own boundary-class evaluation (heatsim2_gb300.adjoint.face_forms)."""
    from heatsim2_gb300.adjoint import face_classes
    args, k, C, fixed, faces, ve, vol = _flaw_problem()
    P, _ = oracle.setup(*args)
    shape, d, dt = (args[6], args[7], args[8]), args[3:6], args[9]
    forms, low = face_classes(shape, d, faces, fixed)
    T = np.full(shape, 293.0) + np.random.default_rng(1).random(shape)
    Tt = torch.tensor(T)
    for n in range(6):
        t = dt * n
        Q = oracle.source_field(shape, d[0] * d[1] * d[2], t, dt, ve, vol)
        T = oracle.run_adi_steps(P, None, t, dt, T, ve, vol)
        Tt = TA.run(Tt, torch.tensor(k), torch.tensor(C), None, [1.0], dt, d, qfields=[torch.tensor(Q)],
                    forms=forms, low=low, fixed=fixed)[-1]
        assert rel_err(Tt.numpy(), T) <= 1e-13, n
    np.testing.assert_array_equal(Tt.numpy()[fixed], T[fixed])


@pytest.mark.parametrize("ckpt", [1, 4])
def test_adjoint_model_with_face_classes_matches_autograd(ckpt):
    """The restatement of the device's face-class adjoint (fixed voxels as an effectively infinite capacity,
    gradients of fixed voxels' k, C, q set to zero) equals autograd through the PyTorch ADI's exact model."""
    from heatsim2_gb300.adjoint import face_classes
    N = 6
    args, k, C, fixed, faces, ve, vol = _flaw_problem(seed=17)
    shape, d, dt = (args[6], args[7], args[8]), args[3:6], args[9]
    forms, low = face_classes(shape, d, faces, fixed)
    rng = np.random.default_rng(3)
    k = k * np.exp(0.2 * rng.standard_normal(shape))
    q = rng.random(shape) * 1e8
    T0 = 293 + rng.random(shape)
    sched = rng.random(N)
    obs = 293 + rng.random((N,) + shape[1:])
    tk = [torch.tensor(a, requires_grad=True) for a in (k, C, q, T0)]
    J = TA.misfit(tk[3], tk[0], tk[1], tk[2], sched, torch.tensor(obs), dt, d, forms=forms, low=low, fixed=fixed)
    J.backward()
    m = AM.Model(k, C, q, dt, d, forms=forms, low=low, fixed=fixed)
    Jm = m.forward(T0, sched, obs, ckpt)
    assert abs(Jm - J.item()) <= 1e-13 * J.item()
    for name, g, t in zip(("k", "C", "q", "T0"), m.backward(), tk):
        assert rel_err(g, t.grad.numpy()) <= 1e-11, name
        if name != "T0":     # a fixed voxel's k, C and q do not enter the step
            assert not g[fixed].any() and not t.grad.numpy()[fixed].any(), name


def test_face_classes_reject_what_the_reference_rejects():
    from heatsim2_gb300.adjoint import face_classes
    args, k, C, fixed, (bnd, bz, by, bx), ve, vol = _flaw_problem()
    shape, d = (args[6], args[7], args[8]), args[3:6]
    bad = bz.copy()
    bad[0, 2, 2] = 0                           # conducting exterior face beside a computed voxel
    with pytest.raises(ValueError):
        face_classes(shape, d, (bnd, bad, by, bx), fixed)
    with pytest.raises(ValueError):            # a tensor-k class
        face_classes(shape, d, (bnd + ((hs.boundary_conducting_anisotropic,),), bz, by, bx), fixed)


def test_adjoint_workloads_are_deterministic():
    a = W.adjoint_steel(nz=4, ny=8, nx=6, nsteps=5)
    b = W.adjoint_steel(nz=4, ny=8, nx=6, nsteps=5)
    for key in ("k", "C", "q", "T0", "schedule", "obs"):
        np.testing.assert_array_equal(a[key], b[key])
    assert a["obs"].shape == (5, 8, 6) and a["k"].shape == (4, 8, 6)
    assert a["schedule"][0] == 1.0 and not a["schedule"][1:].any()
    assert (a["q"][0] == 1e9).all() and not a["q"][1:].any()
    batch = W.adjoint_batch(n=3, nz_range=(4, 6), nxy_range=(8, 12), nsteps=4)
    assert len(batch) == 3
    for inst in batch:
        nz, ny, nx = inst["shape"]
        assert 4 <= nz <= 6 and 8 <= ny <= 12 and 8 <= nx <= 12
        assert set(np.unique(inst["k"])) <= {5.0, 0.3}
        assert (inst["k"] == 0.3).mean() >= 0.1
        assert inst["obs"].shape == (4, ny, nx)
