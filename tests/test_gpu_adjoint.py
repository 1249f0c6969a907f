"""The CUDA adjoint (libhs2g hs2g_adjoint_*) on the GPU.

Forward states match the FP64 PyTorch ADI (pinned to the oracle in test_adjoint_cpu.py); gradients with
respect to per-voxel k, rho*c, q and T0 match autograd through that PyTorch ADI and central finite
differences of the GPU loss; checkpoint intervals and batching change nothing; the torch.autograd.Function
forms carry the incoming gradient."""
import numpy as np
import pytest
import torch

from conftest import rel_err
import torch_adi as TA
from heatsim2_gb300 import workloads as W
from heatsim2_gb300.adjoint import Adjoint, surface_misfit, batch_surface_misfit

pytestmark = pytest.mark.gpu


def _problem(seed, shape, N, sp=(1e-3, 1.2e-3, 0.9e-3)):
    rng = np.random.default_rng(seed)
    k = 54 * np.exp(0.3 * rng.standard_normal(shape))
    C = 7850 * 470 * (1 + 0.2 * rng.random(shape))
    q = rng.random(shape) * 1e9
    T0 = 293 + rng.random(shape)
    sched = rng.random(N)
    obs = 293 + 2 * rng.random((N,) + shape[1:])
    return dict(k=k, C=C, q=q, T0=T0, schedule=sched, obs=obs, spacing=sp, shape=shape)


def _adjoint(p, dt, ckpt, return_state=False):
    a = Adjoint([(p["shape"], p["spacing"])], dt)
    a.set_parameters(p["k"], p["C"], p["q"])
    r = a.forward(p["T0"], p["obs"], p["schedule"], ckpt, return_state=return_state)
    return a, r


@pytest.mark.parametrize("shape", [(6, 10, 12), (1, 7, 5), (9, 1, 3), (4, 6, 1), (1, 1, 1)])
def test_forward_matches_torch_adi(cuda_ok, shape):
    dt, N = 0.01, 9
    p = _problem(1, shape, N)
    a, (loss, T) = _adjoint(p, dt, 4, return_state=True)
    states = TA.run(torch.tensor(p["T0"]), torch.tensor(p["k"]), torch.tensor(p["C"]), torch.tensor(p["q"]),
                    p["schedule"], dt, p["spacing"])
    assert rel_err(T, states[-1].numpy()) <= 1e-12
    J = sum(float(((s[0].numpy() - p["obs"][n]) ** 2).sum()) for n, s in enumerate(states))
    assert abs(loss[0] - J) <= 1e-11 * J


def test_gradients_match_autograd(cuda_ok):
    """(8,16,16) FP64, 40 steps: every gradient matches autograd through the PyTorch ADI."""
    dt, N = 0.01, 40
    p = _problem(2, (8, 16, 16), N)
    a, loss = _adjoint(p, dt, 10)
    g = a.backward()
    tk = [torch.tensor(p[n], requires_grad=True) for n in ("k", "C", "q", "T0")]
    J = TA.misfit(tk[3], tk[0], tk[1], tk[2], p["schedule"], torch.tensor(p["obs"]), dt, p["spacing"])
    J.backward()
    assert abs(loss[0] - J.item()) <= 1e-12 * J.item()
    for name, mine, t in zip(("k", "C", "q", "T0"), g, tk):
        assert rel_err(mine, t.grad.numpy()) <= 1e-10, name


def _faces_problem(seed, shape, N, sp=(1e-3, 1.1e-3, 0.9e-3)):
    """_problem with the forward path's face classes and fixed voxels: a thin insulating layer patch (h = 1000
    W/m^2/K) and an insulating delamination under the surface, a thin layer across x, an insulating exterior,
    a fixed-temperature bottom layer and two fixed voxels inside."""
    import heatsim2_gb300 as hs
    p = _problem(seed, shape, N, sp)
    nz, ny, nx = shape
    bz = np.zeros((nz + 1, ny, nx), np.uint8)
    by = np.zeros((nz, ny + 1, nx), np.uint8)
    bx = np.zeros((nz, ny, nx + 1), np.uint8)
    bz[[0, -1]] = 1
    by[:, [0, -1]] = 1
    bx[:, :, [0, -1]] = 1
    bz[2, 2:ny - 3, 3:nx - 2] = 2
    bz[4, ny // 2:, 1:nx // 2] = 1
    bx[1:4, 3:ny - 2, nx // 2] = 2
    fixed = np.zeros(shape, dtype=bool)
    fixed[-1] = True
    fixed[3, 4, 5] = fixed[5, 2, nx - 3] = True
    bnd = ((hs.boundary_conducting,), (hs.boundary_insulating,), (hs.boundary_thininsulatinglayer, 1000.0))
    p.update(faces=(bnd, bz, by, bx), fixed=fixed)
    return p


def test_face_class_gradients_match_autograd(cuda_ok):
    """(8,16,16) FP64, 40 steps, with a thin-layer flaw, an insulating delamination, a thin layer across x and
    fixed voxels (a fixed bottom layer): the forward states match the PyTorch ADI's class-problem model and every
    gradient matches autograd through it (fixed voxels' k, rho*c and q get none)."""
    from heatsim2_gb300.adjoint import face_classes
    dt, N = 0.01, 40
    p = _faces_problem(2, (8, 16, 16), N)
    a = Adjoint([(p["shape"], p["spacing"])], dt)
    a.set_faces(p["faces"], p["fixed"])
    a.set_parameters(p["k"], p["C"], p["q"])
    loss, T = a.forward(p["T0"], p["obs"], p["schedule"], 10, return_state=True)
    g = a.backward()
    forms, low = face_classes(p["shape"], p["spacing"], p["faces"], p["fixed"])
    tk = [torch.tensor(p[n], requires_grad=True) for n in ("k", "C", "q", "T0")]
    kw = dict(forms=forms, low=low, fixed=p["fixed"])
    states = TA.run(tk[3], tk[0], tk[1], tk[2], p["schedule"], dt, p["spacing"], **kw)
    assert rel_err(T, states[-1].detach().numpy()) <= 1e-12
    np.testing.assert_array_equal(T[p["fixed"]], p["T0"][p["fixed"]])
    J = TA.misfit(tk[3], tk[0], tk[1], tk[2], p["schedule"], torch.tensor(p["obs"]), dt, p["spacing"], **kw)
    J.backward()
    assert abs(loss[0] - J.item()) <= 1e-12 * J.item()
    for name, mine, t in zip(("k", "C", "q", "T0"), g, tk):
        assert rel_err(mine, t.grad.numpy()) <= 1e-10, name
        if name != "T0":
            assert not mine[p["fixed"]].any(), name


def test_face_class_batch_equals_single_instances(cuda_ok):
    """Face classes and fixed voxels per instance in one batch give each instance's single-handle loss and
    gradients bit for bit (the forms table is per instance: the spacings differ), and clearing the faces
    restores the default model bit for bit."""
    dt, N = 0.005, 10
    probs = [_faces_problem(20 + i, s, N, sp) for i, (s, sp) in enumerate(
        [((6, 9, 10), (1e-3, 1e-3, 1e-3)), ((7, 8, 12), (5e-4, 6e-4, 7e-4))])]
    probs[1]["schedule"] = probs[0]["schedule"]
    b = Adjoint([(p["shape"], p["spacing"]) for p in probs], dt)
    b.set_faces([p["faces"] for p in probs], [p["fixed"] for p in probs])
    b.set_parameters([p["k"] for p in probs], [p["C"] for p in probs], [p["q"] for p in probs])
    lb = b.forward([p["T0"] for p in probs], [p["obs"] for p in probs], probs[0]["schedule"], 4)
    gb = b.backward()
    for i, p in enumerate(probs):
        a = Adjoint([(p["shape"], p["spacing"])], dt)
        a.set_faces(p["faces"], p["fixed"])
        a.set_parameters(p["k"], p["C"], p["q"])
        la = a.forward(p["T0"], p["obs"], p["schedule"], 4)
        ga = a.backward()
        assert lb[i] == la[0]
        for x, y in zip(gb, ga):
            np.testing.assert_array_equal(x[i], y)
        a.set_faces(None)
        a.set_parameters(p["k"], p["C"], p["q"])
        lc = a.forward(p["T0"], p["obs"], p["schedule"], 4)
        fresh, lf = _adjoint(p, dt, 4)
        assert lc[0] == lf[0]
        for x, y in zip(a.backward(), fresh.backward()):
            np.testing.assert_array_equal(x, y)


def test_autograd_function_with_faces(cuda_ok):
    """surface_misfit with face classes and fixed voxels carries the incoming gradient onto the numpy-driven
    adjoint's gradients; a following call without faces on a pooled handle is the default model again."""
    dt, N = 0.01, 12
    p = _faces_problem(5, (6, 8, 9), N)
    a = Adjoint([(p["shape"], p["spacing"])], dt)
    a.set_faces(p["faces"], p["fixed"])
    a.set_parameters(p["k"], p["C"], p["q"])
    loss = a.forward(p["T0"], p["obs"], p["schedule"], 5)
    g = a.backward()
    dev = torch.device("cuda", torch.cuda.current_device())
    t = {n: torch.tensor(p[n], device=dev, requires_grad=n != "obs") for n in ("k", "C", "q", "T0", "obs")}
    J = surface_misfit(t["k"], t["C"], t["q"], t["T0"], t["obs"], p["schedule"], p["spacing"], dt, ckpt=5,
                       faces=p["faces"], fixed=p["fixed"])
    assert abs(J.item() - loss[0]) <= 1e-13 * loss[0]
    (2.0 * J).backward()
    for name, ref in zip(("k", "C", "q", "T0"), g):
        assert rel_err(t[name].grad.cpu().numpy(), 2.0 * ref) <= 1e-12, name
    J0 = surface_misfit(t["k"], t["C"], t["q"], t["T0"], t["obs"], p["schedule"], p["spacing"], dt, ckpt=5)
    fresh, l0 = _adjoint(p, dt, 5)
    assert abs(J0.item() - l0[0]) <= 1e-13 * l0[0]


def test_checkpoint_interval_changes_nothing(cuda_ok):
    dt, N = 0.01, 23
    p = _problem(3, (5, 9, 11), N)
    ref = None
    for ckpt in (1, 4, 7, 23, 1000):
        a, loss = _adjoint(p, dt, ckpt)
        g = a.backward()
        if ref is None:
            ref = (loss, g)
        else:
            np.testing.assert_array_equal(loss, ref[0])
            for x, y in zip(g, ref[1]):
                np.testing.assert_array_equal(x, y)


def test_repeated_evaluations_on_one_handle(cuda_ok):
    """From the second evaluation on, the forward pass leaves its last segment in the backward pass's store and
    the backward pass skips recomputing it; gradients stay equal bit for bit to a fresh handle's, also when the
    checkpoint interval changes between evaluations (one segment, more, an interval whose store is too small)."""
    dt, N = 0.01, 23
    p = _problem(3, (5, 9, 11), N)
    a = Adjoint([(p["shape"], p["spacing"])], dt)
    a.set_parameters(p["k"], p["C"], p["q"])
    for ckpt in (4, 4, 23, 7, 1, 10, 5):
        fresh, lf = _adjoint(p, dt, ckpt)
        gf = fresh.backward()
        la = a.forward(p["T0"], p["obs"], p["schedule"], ckpt)
        ga = a.backward()
        np.testing.assert_array_equal(la, lf)
        for x, y in zip(ga, gf):
            np.testing.assert_array_equal(x, y)


def test_batch_equals_single_instances(cuda_ok):
    """Uneven instances in one concatenated state give, per instance, the single-instance loss and gradients
    bit for bit."""
    dt, N = 0.005, 12
    probs = [_problem(10 + i, s, N, sp) for i, (s, sp) in enumerate(
        [((4, 6, 8), (1e-3, 1e-3, 1e-3)), ((7, 3, 5), (5e-4, 6e-4, 7e-4)), ((1, 9, 2), (1e-3, 2e-3, 1e-3)),
         ((3, 5, 5), (2e-3, 1e-3, 1e-3))])]
    for p in probs[1:]:
        p["schedule"] = probs[0]["schedule"]
    b = Adjoint([(p["shape"], p["spacing"]) for p in probs], dt)
    b.set_parameters([p["k"] for p in probs], [p["C"] for p in probs], [p["q"] for p in probs])
    lb = b.forward([p["T0"] for p in probs], [p["obs"] for p in probs], probs[0]["schedule"], 5)
    gb = b.backward()
    for i, p in enumerate(probs):
        a, la = _adjoint(p, dt, 5)
        ga = a.backward()
        assert lb[i] == la[0]
        for x, y in zip(gb, ga):
            np.testing.assert_array_equal(x[i], y)


def test_batch_equals_single_instances_across_line_kernels(cuda_ok):
    """The batch has enough y- and z-lines for the register-blocked line kernels; the instances run alone have
    few enough for the shared-memory few-line kernels (y for all, z for the two smaller).  Both give the same
    bits."""
    dt, N = 0.005, 6
    shapes = [(48, 144, 144), (48, 144, 144), (40, 100, 100), (30, 120, 160)]
    probs = [_problem(40 + i, s, N) for i, s in enumerate(shapes)]
    for p in probs[1:]:
        p["schedule"] = probs[0]["schedule"]
    b = Adjoint([(p["shape"], p["spacing"]) for p in probs], dt)
    b.set_parameters([p["k"] for p in probs], [p["C"] for p in probs], [p["q"] for p in probs])
    lb = b.forward([p["T0"] for p in probs], [p["obs"] for p in probs], probs[0]["schedule"], 3)
    gb = b.backward()
    for i, p in enumerate(probs):
        a, la = _adjoint(p, dt, 3)
        ga = a.backward()
        assert lb[i] == la[0]
        for x, y in zip(gb, ga):
            np.testing.assert_array_equal(x[i], y)


def _flash_problem(seed, shape, N, sp=(1e-3, 1e-3, 1e-3), dt=0.01):
    """A realistic inverse problem: lognormal k, flash in the top layer during the first step, observations
    from the semi-infinite-body response plus noise."""
    rng = np.random.default_rng(seed)
    k = 54 * np.exp(0.2 * rng.standard_normal(shape))
    C = 7850 * 470 * (1 + 0.1 * rng.random(shape))
    q = np.zeros(shape)
    q[0] = 1e9
    sched = np.zeros(N)
    sched[0] = 1.0
    obs = W.flash_observations(rng, shape, N, dt, sp[0], 54.0, 7850 * 470.0, 1e9)
    return dict(k=k, C=C, q=q, T0=np.full(shape, 293.0), schedule=sched, obs=obs, spacing=sp, shape=shape)


def _perturbed_losses(p, dt, ckpt, perts, chunk=64):
    """Losses of copies of problem p, copy i with p[name][idx] += delta for perts[i] = (name, idx, delta),
    evaluated as instances of batched forward passes on the device."""
    dev = torch.device("cuda", torch.cuda.current_device())
    nv = int(np.prod(p["shape"]))
    shift = float(np.mean(p["T0"]))
    base = {n: torch.tensor(p[n], device=dev).reshape(-1) for n in ("k", "C", "q")}
    T0 = torch.tensor(p["T0"] - shift, device=dev).reshape(-1)
    obs = torch.tensor(p["obs"] - shift, device=dev).reshape(-1)
    out = []
    for c0 in range(0, len(perts), chunk):
        part = perts[c0:c0 + chunk]
        m = len(part)
        a = Adjoint([(p["shape"], p["spacing"])] * m, dt)
        arrs = {n: base[n].repeat(m) for n in base}
        for i, (name, idx, delta) in enumerate(part):
            f = i * nv + int(np.ravel_multi_index(idx, p["shape"]))
            arrs[name][f] = float(p[name][idx]) + delta
        a.set_parameters_device(arrs["k"], arrs["C"], arrs["q"])
        out.extend(a.forward_device(T0.repeat(m), obs.repeat(m), p["schedule"], ckpt))
        del a
    return np.array(out)


def _fd_errors(p, dt, ckpt, voxels, h_rel=5e-2, floor=1e-3):
    """Errors of the adjoint against central differences at the given voxels, relative to the gradient entry
    or, where that is smaller, to `floor` times the largest gradient magnitude of the field: a double-precision
    loss difference cannot resolve entries far below the field's scale (deep voxels the surface barely sees).
    k and C use central differences at steps h, h/2, h/4 combined by two Richardson levels (error O(h^6)), so
    h can be large enough for the loss difference to stand well above the loss's rounding noise; J is
    quadratic in q, so a single central difference is exact there up to rounding."""
    a, loss = _adjoint(p, dt, ckpt)
    grads = dict(zip(("k", "C", "q"), a.backward()[:3]))
    gmax = {n: float(np.abs(g).max()) for n, g in grads.items()}
    perts, plan = [], []
    for name in ("k", "C", "q"):
        scale = np.abs(p[name]).max()
        for idx in voxels:
            h = h_rel * (abs(p[name][idx]) if p[name][idx] != 0 else scale)
            steps = (h, h / 2, h / 4) if name != "q" else (h,)
            plan.append((name, idx, steps, len(perts)))
            for hh in steps:
                perts += [(name, idx, hh), (name, idx, -hh)]
    J = _perturbed_losses(p, dt, ckpt, perts)
    errs = {}
    for name, idx, steps, at in plan:
        d = [(J[at + 2 * i] - J[at + 2 * i + 1]) / (2 * hh) for i, hh in enumerate(steps)]
        if len(d) == 1:
            fd = d[0]
        else:
            r1 = [(4 * d[i + 1] - d[i]) / 3 for i in range(2)]
            fd = (16 * r1[1] - r1[0]) / 15
        g = grads[name][idx]
        floored = abs(g) < floor * gmax[name]
        errs[(name, idx)] = (abs(fd - g) / max(abs(g), floor * gmax[name]), floored)
    return errs


def _check_fd(errs, tol=1e-6, label=""):
    """Every entry within tol: relative to the entry itself where it lies above the floor, relative to the floor
    where it lies below.  Reports how many entries of each field the floor decided; returns those counts."""
    floored = {}
    for (name, _), (_, f) in errs.items():
        floored[name] = floored.get(name, 0) + int(f)
    total = {}
    for (name, _) in errs:
        total[name] = total.get(name, 0) + 1
    rel = {key: e for key, (e, f) in errs.items() if not f}
    flo = {key: e for key, (e, f) in errs.items() if f}
    print("%s FD check: floor decided %s of %s entries; largest relative error above the floor %.2e, largest "
          "floor-relative error below it %.2e" % (label, floored, total, max(rel.values(), default=0.0),
                                                  max(flo.values(), default=0.0)))
    worst = sorted(errs.items(), key=lambda kv: -kv[1][0])[:4]
    assert max(rel.values(), default=0.0) <= tol, worst
    assert max(flo.values(), default=0.0) <= tol, worst
    return floored, total


def test_gradients_match_central_differences(cuda_ok):
    """Central differences of the GPU loss at random voxels agree with the adjoint to 1e-6 relative (floored
    at 1e-3 of the field's largest gradient; the number of entries the floor decided is reported and bounded)."""
    dt, N = 0.01, 80
    p = _flash_problem(4, (10, 24, 20), N)
    rng = np.random.default_rng(6)
    vox = [tuple(int(rng.integers(0, n)) for n in p["shape"]) for _ in range(12)]
    errs = _fd_errors(p, dt, 16, vox)
    floored, total = _check_fd(errs, label="flash (10,24,20)")
    # a shallow grid: the surface sees every voxel, so the relative criterion decides most entries
    assert sum(floored.values()) <= sum(total.values()) // 4, floored


@pytest.mark.slow
def test_steel_adjoint_central_differences_64_voxels(cuda_ok):
    """The (32,128,128) steel inverse problem, 500 steps of 10 ms, checkpoint every 50: k, rho*c and q
    gradients at 64 random voxels agree with central differences to 1e-6 relative (floored at 1e-3 of the
    field's largest gradient).  Entries above the floor are judged by their own relative error; how many the
    floor decided is printed, and 32 further voxels in the top two layers must all be judged relatively."""
    w = W.adjoint_steel()
    p = dict(k=w["k"], C=w["C"], q=w["q"], T0=w["T0"], schedule=w["schedule"], obs=w["obs"],
             spacing=w["spacing"], shape=w["shape"])
    rng = np.random.default_rng(8)
    vox = [tuple(int(rng.integers(0, n)) for n in w["shape"]) for _ in range(64)]
    # 32 more in the two layers under the observed surface, where every gradient entry stands above the floor
    top = [(int(rng.integers(0, 2)), int(rng.integers(0, w["shape"][1])), int(rng.integers(0, w["shape"][2])))
           for _ in range(32)]
    errs = _fd_errors(p, w["dt"], w["ckpt"], vox + top)
    floored, total = _check_fd(errs, label="steel (32,128,128)")
    # uniform voxels over the depth: most lie deeper than the flash reaches in 5 s, and the floor decides those
    # (counts printed above); the top-layer voxels must all be judged by their own relative error
    top_floored = [key for key in errs if key[1] in set(top) and errs[key][1]]
    assert not top_floored, top_floored


def test_autograd_function_single(cuda_ok):
    dt, N = 0.01, 15
    p = _problem(7, (5, 8, 6), N)
    a, loss = _adjoint(p, dt, 4)
    g = a.backward()
    dev = torch.device("cuda", torch.cuda.current_device())
    t = {n: torch.tensor(p[n], device=dev, requires_grad=n != "obs") for n in ("k", "C", "q", "T0", "obs")}
    J = surface_misfit(t["k"], t["C"], t["q"], t["T0"], t["obs"], p["schedule"], p["spacing"], dt, ckpt=4)
    assert abs(J.item() - loss[0]) <= 1e-13 * loss[0]
    (3.0 * J).backward()
    for name, ref in zip(("k", "C", "q", "T0"), g):
        assert rel_err(t[name].grad.cpu().numpy(), 3.0 * ref) <= 1e-12, name


def test_autograd_function_batch_weights(cuda_ok):
    dt, N = 0.01, 10
    shapes = [(4, 6, 5), (3, 7, 9)]
    probs = [_problem(20 + i, s, N) for i, s in enumerate(shapes)]
    for p in probs[1:]:
        p["schedule"] = probs[0]["schedule"]
    dev = torch.device("cuda", torch.cuda.current_device())
    ts = [{n: torch.tensor(p[n], device=dev, requires_grad=n != "obs") for n in ("k", "C", "q", "T0", "obs")}
          for p in probs]
    L = batch_surface_misfit([t["k"] for t in ts], [t["C"] for t in ts], [t["q"] for t in ts],
                             [t["T0"] for t in ts], [t["obs"] for t in ts], probs[0]["schedule"],
                             probs[0]["spacing"], dt, ckpt=3)
    assert L.shape == (2,)
    (2.0 * L[0] - 0.5 * L[1]).backward()
    for i, (p, w) in enumerate(zip(probs, (2.0, -0.5))):
        a, loss = _adjoint(p, dt, 3)
        assert abs(L[i].item() - loss[0]) <= 1e-13 * loss[0]
        for name, ref in zip(("k", "C", "q", "T0"), a.backward()):
            assert rel_err(ts[i][name].grad.cpu().numpy(), w * ref) <= 1e-12, name


def test_errors(cuda_ok):
    a = Adjoint([((2, 3, 4), (1e-3, 1e-3, 1e-3))], 0.01)
    with pytest.raises(RuntimeError):
        a.backward()          # no forward pass yet
    with pytest.raises(ValueError):
        a.set_parameters(np.ones((2, 3, 4)), -np.ones((2, 3, 4)), np.zeros((2, 3, 4)))
    with pytest.raises(ValueError):
        a.set_parameters(np.ones((2, 3, 5)), np.ones((2, 3, 4)), np.zeros((2, 3, 4)))
