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
