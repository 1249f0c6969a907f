"""Seeded synthetic heat-conduction problems with the shapes of heatsim2's flash-thermography workloads.

A problem is held as a plain, module-independent *spec* (numpy class arrays plus JSON-able material, boundary
and source descriptions).  ``setup_args(hs, spec)`` turns a spec into the positional arguments of
``hs.setup`` for any module ``hs`` that follows the heatsim2 API (this package, or the reference
``heatsim2`` package -- the builders only use the public names ``TEMPERATURE_COMPUTE``, ``boundary_*``,
``STEPPED_SOURCE`` ... that both define, heatsim2/__init__.py:42-50 in the reference).

Spec vocabulary
---------------
materials:  ["compute", k, rho, c] with k a float or a 3x3 nested list (z,y,x order), or ["fixed"]
boundaries: ["insulating"], ["conducting"], ["conducting_anisotropic"], ["thininsulatinglayer", h]
volumetric: ["none"], ["impulse", t0, J_per_m3], ["stepped", t0, t1, W_per_m3],
            ["point_joules", t0, J] (J a float, or the name of an array in spec["arrays"]),
            ["zdecay", t0, [dz,dy,dx direction], offset, "<array name of z_ndgrid>", dz, J_per_m2, length]

Workloads (grid shapes, materials, boundaries and seeds follow the benchmark configurations):
  * ``steel_slab``      -- (20,40,40) steel slab, 1 mm cells, thin-insulating-layer 8x8 flaw, 10 ms flash.
  * ``composite_panel`` -- anisotropic composite over aluminium under a fixed-temperature ambient layer
                           coupled by an h=10 W/m^2/K thin layer, three insulating delaminations.
  * ``uneven_batch``    -- a list of steel / composite instances of uneven size.
"""
import json

import numpy as np

T_AMBIENT = 293.0


# ----------------------------------------------------------------------------------------------------------
# spec -> module tuples
# ----------------------------------------------------------------------------------------------------------
def _k_value(k):
    if isinstance(k, (list, tuple)):
        return np.array(k, dtype="d")
    return float(k)


def materials_tuple(hs, spec):
    out = []
    for m in spec["materials"]:
        if m[0] == "compute":
            out.append((hs.TEMPERATURE_COMPUTE, _k_value(m[1]), float(m[2]), float(m[3])))
        elif m[0] == "fixed":
            out.append((hs.TEMPERATURE_FIXED,))
        else:
            raise ValueError("unknown material kind %r" % (m[0],))
    return tuple(out)


def boundaries_tuple(hs, spec):
    out = []
    for b in spec["boundaries"]:
        mod = getattr(hs, "boundary_" + b[0])
        out.append((mod,) + tuple(float(v) for v in b[1:]))
    return tuple(out)


def volumetric_tuple(hs, spec):
    arrays = spec.get("arrays", {})
    out = []
    for v in spec["volumetric"]:
        kind = v[0]
        if kind == "none":
            out.append((hs.NO_SOURCE,))
        elif kind == "impulse":
            out.append((hs.IMPULSE_SOURCE, float(v[1]), float(v[2])))
        elif kind == "stepped":
            out.append((hs.STEPPED_SOURCE, float(v[1]), float(v[2]), float(v[3])))
        elif kind == "point_joules":
            J = arrays[v[2]] if isinstance(v[2], str) else float(v[2])
            out.append((hs.IMPULSE_POINT_SOURCE_JOULES, float(v[1]), J))
        elif kind == "zdecay":
            out.append((hs.SPATIALLY_Z_DECAYING_TEMPORAL_IMPULSE, float(v[1]), np.array(v[2], dtype="d"),
                        float(v[3]), arrays[v[4]], float(v[5]), float(v[6]), float(v[7])))
        else:
            raise ValueError("unknown source kind %r" % (kind,))
    return tuple(out)


def setup_args(hs, spec):
    """Positional arguments of ``hs.setup`` for this spec."""
    g = spec["grid"]
    a = spec["arrays"]
    return (g["z0"], g["y0"], g["x0"], g["dz"], g["dy"], g["dx"], g["nz"], g["ny"], g["nx"], spec["dt"],
            materials_tuple(hs, spec), boundaries_tuple(hs, spec), volumetric_tuple(hs, spec),
            a["material"], a["boundary_z"], a["boundary_y"], a["boundary_x"], a["volumetric"])


def setup_kwargs(spec):
    """Keyword arguments of ``hs.setup`` for this spec: the surface curvatures of a curved spec, else none."""
    a = spec.get("arrays", {})
    if "curv_y" in a or "curv_x" in a:
        return {"top_surface_y_curvatures": a.get("curv_y"), "top_surface_x_curvatures": a.get("curv_x")}
    return {}


def curved(spec, seed=0, ky=None, kx=None, amplitude=20.0):
    """A copy of ``spec`` in the reference's curved-surface mode: curvatures (1/m, positive concave) along y and
    x per surface cell, given or seeded uniform in [-amplitude, amplitude]."""
    g = spec["grid"]
    rng = np.random.default_rng(seed)
    shape = (g["ny"], g["nx"])
    ky = rng.uniform(-amplitude, amplitude, shape) if ky is None else np.broadcast_to(ky, shape).astype("d")
    kx = rng.uniform(-amplitude, amplitude, shape) if kx is None else np.broadcast_to(kx, shape).astype("d")
    out = dict(spec)
    out["name"] = "curved_" + spec["name"]
    out["arrays"] = dict(spec["arrays"], curv_y=np.ascontiguousarray(ky), curv_x=np.ascontiguousarray(kx))
    return out


def initial_temperature(spec):
    g = spec["grid"]
    return np.full((g["nz"], g["ny"], g["nx"]), float(spec.get("T0", T_AMBIENT)), dtype="d")


def step_times(spec, nsteps=None):
    """The t values a time loop passes to run_adi_steps: t0 + n*dt (as the reference demos build them)."""
    n = spec["nsteps"] if nsteps is None else nsteps
    return [spec.get("t0", 0.0) + spec["dt"] * c for c in range(n)]


def voxels(spec):
    g = spec["grid"]
    return g["nz"] * g["ny"] * g["nx"]


# ----------------------------------------------------------------------------------------------------------
# (de)serialisation: npz arrays + json metadata
# ----------------------------------------------------------------------------------------------------------
def spec_to_npz_dict(spec, prefix="spec_"):
    meta = {k: v for k, v in spec.items() if k != "arrays"}
    d = {prefix + "meta": np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)}
    for name, arr in spec["arrays"].items():
        d[prefix + "arr_" + name] = arr
    return d


def spec_from_npz(npz, prefix="spec_"):
    meta = json.loads(bytes(npz[prefix + "meta"]).decode())
    arrays = {}
    for key in npz.files:
        if key.startswith(prefix + "arr_"):
            arrays[key[len(prefix) + 4:]] = np.array(npz[key])
    meta["arrays"] = arrays
    return meta


# ----------------------------------------------------------------------------------------------------------
# builders
# ----------------------------------------------------------------------------------------------------------
def _zero_arrays(nz, ny, nx):
    return {
        "material": np.zeros((nz, ny, nx), dtype=np.uint8),
        "boundary_z": np.zeros((nz + 1, ny, nx), dtype=np.uint8),
        "boundary_y": np.zeros((nz, ny + 1, nx), dtype=np.uint8),
        "boundary_x": np.zeros((nz, ny, nx + 1), dtype=np.uint8),
        "volumetric": np.zeros((nz, ny, nx), dtype=np.uint8),
    }


def _insulate_exterior(a, insulating):
    a["boundary_z"][0] = insulating
    a["boundary_z"][-1] = insulating
    a["boundary_y"][:, 0, :] = insulating
    a["boundary_y"][:, -1, :] = insulating
    a["boundary_x"][:, :, 0] = insulating
    a["boundary_x"][:, :, -1] = insulating


def _grid(nz, ny, nx, d):
    # cell centres of a grid whose boundaries start at 0 (build_grid(0,nz*d,nz, ...) in the reference API)
    return {"z0": d / 2, "y0": d / 2, "x0": d / 2, "dz": d, "dy": d, "dx": d, "nz": nz, "ny": ny, "nx": nx}


def steel_slab(seed=0, nz=20, ny=40, nx=40, d=1e-3, dt=0.01, nsteps=200, h=1000.0, flaw=8,
               depth_range=(3, 15), power=1e9):
    """(20,40,40) steel slab at 1 mm: k=54, rho=7850, c=470, insulating outside, an 8x8 thin-insulating-layer
    (h=1000 W/m^2/K) flaw at a seeded depth in 3..15, flash 1e9 W/m^3 in the top layer for one 10 ms step."""
    rng = np.random.default_rng(seed)
    a = _zero_arrays(nz, ny, nx)
    # boundary classes: 0 conducting, 1 insulating, 2 thin layer
    _insulate_exterior(a, 1)
    hi = min(depth_range[1], nz - 1)          # an interior z-face (the exterior ones must stay insulating)
    depth = int(rng.integers(min(depth_range[0], hi), hi + 1)) if hi >= 1 else 0
    y0 = int(rng.integers(0, ny - flaw + 1))
    x0 = int(rng.integers(0, nx - flaw + 1))
    if depth >= 1:
        a["boundary_z"][depth, y0:y0 + flaw, x0:x0 + flaw] = 2
    a["volumetric"][0] = 1
    return {
        "name": "steel_slab", "grid": _grid(nz, ny, nx, d), "dt": dt, "t0": 0.0, "nsteps": nsteps,
        "T0": T_AMBIENT,
        "materials": [["compute", 54.0, 7850.0, 470.0]],
        "boundaries": [["conducting"], ["insulating"], ["thininsulatinglayer", h]],
        "volumetric": [["none"], ["stepped", 0.0, 0.5 * dt, power]],
        "arrays": a,
        "flaw": {"depth": depth, "y0": y0, "x0": x0, "w": flaw},
    }


COMPOSITE_K = [[0.6, 0.0, 0.0], [0.0, 5.0, 0.0], [0.0, 0.0, 5.0]]
ALUMINIUM_K = [[167.0, 0.0, 0.0], [0.0, 167.0, 0.0], [0.0, 0.0, 167.0]]


def composite_panel(seed=1, nz=64, ny=512, nx=512, d=0.5e-3, dt=0.005, nsteps=1000, top_layers=16,
                    n_delams=3, width_range=(10, 60), depth_range=(4, 40), power=2e9, h_top=10.0):
    """Two-layer composite: ``top_layers`` anisotropic layers (kz=0.6, ky=kx=5, rho=1550, c=1100) over
    aluminium (k=167, rho=2700, c=900), ``nz`` compute layers of ``d`` cells.  The conducting top (h=10 W/m^2/K
    to ambient) is a fixed-temperature ambient layer 0 joined to the first compute layer by a thin-insulating-layer
    face, since an exterior face must be insulating.  Seeded rectangular insulating delaminations at
    z-faces ``1+depth`` (depth in ``depth_range`` below the first compute layer).  Flash in the first compute
    layer for one step.  The grid has nz+1 layers; nz*ny*nx are computed."""
    rng = np.random.default_rng(seed)
    NZ = nz + 1
    a = _zero_arrays(NZ, ny, nx)
    # materials: 0 composite, 1 aluminium, 2 fixed ambient
    a["material"][0] = 2
    a["material"][1:1 + top_layers] = 0
    a["material"][1 + top_layers:] = 1
    # boundaries: 0 anisotropic conducting, 1 insulating, 2 thin layer h_top
    _insulate_exterior(a, 1)
    a["boundary_z"][1] = 2
    delams = []
    dmax = min(depth_range[1], nz - 1)
    dmin = min(depth_range[0], dmax)
    for _ in range(n_delams if dmax >= 1 else 0):
        wy = int(rng.integers(width_range[0], width_range[1] + 1))
        wx = int(rng.integers(width_range[0], width_range[1] + 1))
        wy, wx = min(wy, ny), min(wx, nx)
        depth = int(rng.integers(dmin, dmax + 1))
        y0 = int(rng.integers(0, ny - wy + 1))
        x0 = int(rng.integers(0, nx - wx + 1))
        a["boundary_z"][1 + depth, y0:y0 + wy, x0:x0 + wx] = 1
        delams.append({"depth": depth, "y0": y0, "x0": x0, "wy": wy, "wx": wx})
    a["volumetric"][1] = 1
    return {
        "name": "composite_panel", "grid": _grid(NZ, ny, nx, d), "dt": dt, "t0": 0.0, "nsteps": nsteps,
        "T0": T_AMBIENT, "compute_voxels": nz * ny * nx,
        "materials": [["compute", COMPOSITE_K, 1550.0, 1100.0], ["compute", ALUMINIUM_K, 2700.0, 900.0],
                      ["fixed"]],
        "boundaries": [["conducting_anisotropic"], ["insulating"], ["thininsulatinglayer", h_top]],
        "volumetric": [["none"], ["stepped", 0.0, 0.5 * dt, power]],
        "arrays": a,
        "delaminations": delams,
    }


def uneven_batch(seed=2, n=256, nz_range=(16, 64), nxy_range=(64, 256), dt=0.01, nsteps=500, power=1e9):
    """``n`` instances of uneven size: nz uniform in nz_range, ny,nx uniform in nxy_range, each a steel slab
    (1 mm) with one thin-layer flaw or a composite panel (0.5 mm, ambient layer included) with one insulating
    delamination (p=1/2); flaw width 4..32 voxels, depth 2..nz/2; flash 1e9 W/m^3 for one step."""
    rng = np.random.default_rng(seed)
    specs = []
    for c in range(n):
        nz = int(rng.integers(nz_range[0], nz_range[1] + 1))
        ny = int(rng.integers(nxy_range[0], nxy_range[1] + 1))
        nx = int(rng.integers(nxy_range[0], nxy_range[1] + 1))
        sub = int(rng.integers(0, 2 ** 31))
        w = int(rng.integers(4, 33))
        depth_hi = max(2, nz // 2)
        if rng.random() < 0.5:
            s = steel_slab(seed=sub, nz=nz, ny=ny, nx=nx, dt=dt, nsteps=nsteps, flaw=min(w, ny, nx),
                           depth_range=(2, depth_hi), power=power)
        else:
            s = composite_panel(seed=sub, nz=nz, ny=ny, nx=nx, dt=dt, nsteps=nsteps, n_delams=1,
                                width_range=(min(w, ny, nx), min(w, ny, nx)), depth_range=(2, depth_hi),
                                power=power)
        s["instance"] = c
        specs.append(s)
    return specs


def mixed_small(seed=5, nz=5, ny=6, nx=7, dt=0.02, nsteps=6):
    """A small grid that exercises every built-in boundary class on every axis, scalar- and matrix-k
    materials in separate regions, fixed-temperature voxels inside the grid and two kinds of source."""
    rng = np.random.default_rng(seed)
    a = _zero_arrays(nz, ny, nx)
    # materials: 0 steel (scalar k), 1 foam (scalar), 2 composite (matrix), 3 fixed, 4 titanium (matrix)
    a["material"][:] = rng.integers(0, 2, size=(nz, ny, nx))
    a["material"][:, :, nx // 2:] = rng.choice([2, 4], size=(nz, ny, nx - nx // 2))
    a["material"][1, 2, 1] = 3
    a["material"][3, 4, 5] = 3
    # boundaries: 0 conducting, 1 insulating, 2 thin h=500, 3 anisotropic, 4 thin h=50
    for key in ("boundary_z", "boundary_y", "boundary_x"):
        a[key][:] = rng.choice([0, 1, 2, 4], size=a[key].shape)
    # faces touching the matrix-k half use the anisotropic class (or a k-independent class)
    a["boundary_x"][:, :, nx // 2:] = rng.choice([3, 1, 2], size=a["boundary_x"][:, :, nx // 2:].shape)
    a["boundary_z"][:, :, nx // 2:] = rng.choice([3, 4], size=a["boundary_z"][:, :, nx // 2:].shape)
    a["boundary_y"][:, :, nx // 2:] = rng.choice([3, 2], size=a["boundary_y"][:, :, nx // 2:].shape)
    # the x-faces between the scalar-k and matrix-k halves must not depend on k
    a["boundary_x"][:, :, nx // 2] = rng.choice([1, 2], size=(nz, ny))
    _insulate_exterior(a, 1)
    a["volumetric"][0] = 1
    a["volumetric"][2, 1:3, 1:4] = 2
    a["volumetric"][3, 4, 5] = 2           # a source on a fixed voxel has no effect
    return {
        "name": "mixed_small", "grid": _grid(nz, ny, nx, 1e-3), "dt": dt, "t0": 0.0, "nsteps": nsteps,
        "T0": T_AMBIENT,
        "materials": [["compute", 54.0, 7850.0, 470.0], ["compute", 0.4, 40.0, 1500.0],
                      ["compute", COMPOSITE_K, 1550.0, 1100.0], ["fixed"],
                      ["compute", [[6.7, 0, 0], [0, 7.5, 0], [0, 0, 8.25]], 4430.0, 526.3]],
        "boundaries": [["conducting"], ["insulating"], ["thininsulatinglayer", 500.0],
                       ["conducting_anisotropic"], ["thininsulatinglayer", 50.0]],
        "volumetric": [["none"], ["impulse", 0.0, 1e7], ["stepped", 0.02, 0.06, 3e8]],
        "arrays": a,
    }


def line_grid(shape, seed=7, nsteps=5, dt=0.01):
    """Degenerate grids (1xN lines, planes, single voxels): steel, conducting inside, insulating outside,
    an impulse in the first layer (or first voxel) and a thin layer in the middle of the longest axis."""
    nz, ny, nx = shape
    a = _zero_arrays(nz, ny, nx)
    _insulate_exterior(a, 1)
    axis = int(np.argmax(shape))
    n = shape[axis]
    if n > 2:
        key = ("boundary_z", "boundary_y", "boundary_x")[axis]
        idx = [slice(None)] * 3
        idx[axis] = n // 2
        a[key][tuple(idx)] = 2
    a["volumetric"].reshape(-1)[0] = 1
    return {
        "name": "line_grid_%dx%dx%d" % shape, "grid": _grid(nz, ny, nx, 1e-3), "dt": dt, "t0": 0.0,
        "nsteps": nsteps, "T0": T_AMBIENT,
        "materials": [["compute", 54.0, 7850.0, 470.0]],
        "boundaries": [["conducting"], ["insulating"], ["thininsulatinglayer", 200.0]],
        "volumetric": [["none"], ["impulse", 0.0, 5e6]],
        "arrays": a,
    }


def sources_small(seed=9, nz=6, ny=5, nx=4, dt=0.01, nsteps=5):
    """Every volumetric source kind: impulse, stepped window with inclusive ends, point joules (scalar and
    per-voxel array), and the spatially z-decaying impulse."""
    rng = np.random.default_rng(seed)
    a = _zero_arrays(nz, ny, nx)
    _insulate_exterior(a, 1)
    a["volumetric"][0, :, :2] = 1          # impulse at t=0.01
    a["volumetric"][0, :, 2:] = 2          # stepped 0.01..0.03 inclusive
    a["volumetric"][3, 2, 1] = 3           # point joules, scalar
    a["volumetric"][4, 1:3, 1:3] = 4       # point joules, per-voxel array
    a["volumetric"][1:3, :, :] = 5         # z-decaying impulse at t=0.02
    z = (np.arange(nz) + 0.5) * 1e-3
    zgrid = np.broadcast_to(z[:, None, None], (nz, ny, nx)).copy()
    pj = rng.uniform(0.1, 0.5, size=int((a["volumetric"] == 4).sum()))
    return {
        "name": "sources_small", "grid": _grid(nz, ny, nx, 1e-3), "dt": dt, "t0": 0.0, "nsteps": nsteps,
        "T0": T_AMBIENT,
        "materials": [["compute", 54.0, 7850.0, 470.0]],
        "boundaries": [["conducting"], ["insulating"]],
        "volumetric": [["none"], ["impulse", 0.01, 2e7], ["stepped", 0.01, 0.03, 4e8],
                       ["point_joules", 0.02, 0.3], ["point_joules", 0.03, "pj"],
                       ["zdecay", 0.02, [1.0, 0.0, 0.0], 0.0005, "zgrid", 1e-3, 1e4, 0.0007]],
        "arrays": dict(a, zgrid=zgrid, pj=pj),
    }


# ----------------------------------------------------------------------------------------------------------
# adjoint (inverse-problem) workloads: per-voxel parameters, top-surface observations
# ----------------------------------------------------------------------------------------------------------
def flash_observations(rng, shape, nsteps, dt, d, k, C, q_top, T0=T_AMBIENT, noise=0.01):
    """Seeded synthetic top-surface temperatures (nsteps, ny, nx): the semi-infinite-body response to a flash
    of q_top W/m^3 absorbed in a top layer of depth d during the first step, T0 + E / (e sqrt(pi t)) with
    E = q_top d dt (J/m^2) and effusivity e = sqrt(k C), plus Gaussian noise of `noise` K."""
    nz, ny, nx = shape
    t = dt * (np.arange(nsteps) + 1.0)
    rise = q_top * d * dt / (np.sqrt(k * C) * np.sqrt(np.pi * t))
    obs = T0 + rise[:, None, None] + noise * rng.standard_normal((nsteps, ny, nx))
    return obs


def adjoint_steel(seed=3, nz=32, ny=128, nx=128, d=1e-3, dt=0.01, nsteps=500, ckpt=50, sigma=0.2,
                  power=1e9):
    """Single-instance adjoint workload: (32,128,128) steel at 1 mm, per-voxel k lognormal around 54 W/m/K
    (sigma 0.2), rho*c = 7850*470, flash ``power`` W/m^3 in the top layer during the first 10 ms step, T0 = 293 K,
    500 steps of 10 ms, checkpoint every 50; observations of the top surface seeded-synthetic."""
    rng = np.random.default_rng(seed)
    shape = (nz, ny, nx)
    k = 54.0 * np.exp(sigma * rng.standard_normal(shape) - 0.5 * sigma * sigma)
    C = np.full(shape, 7850.0 * 470.0)
    q = np.zeros(shape)
    q[0] = power
    schedule = np.zeros(nsteps)
    schedule[0] = 1.0
    obs = flash_observations(rng, shape, nsteps, dt, d, 54.0, 7850.0 * 470.0, power)
    return {"name": "adjoint_steel", "shape": shape, "spacing": (d, d, d), "dt": dt, "nsteps": nsteps,
            "ckpt": ckpt, "k": k, "C": C, "q": q, "T0": np.full(shape, T_AMBIENT), "schedule": schedule,
            "obs": obs}


def two_phase_k(rng, shape, matrix=5.0, inclusion=0.3, fraction=0.1, radius_range=(1, 4)):
    """Matrix conductivity with seeded box inclusions (half-widths in radius_range) of `inclusion` W/m/K, added
    sixteen at a time until they cover at least `fraction` of the voxels."""
    nz, ny, nx = shape
    k = np.full(shape, matrix)
    mask = np.zeros(shape, dtype=bool)
    target = fraction * mask.size
    while mask.sum() < target:
        for _ in range(16):
            r = rng.integers(radius_range[0], radius_range[1] + 1, size=3)
            c = [int(rng.integers(0, n)) for n in shape]
            sl = tuple(slice(max(0, c[a] - r[a]), min(shape[a], c[a] + r[a] + 1)) for a in range(3))
            mask[sl] = True
    k[mask] = inclusion
    return k


def adjoint_batch(seed=4, n=32, nz_range=(24, 48), nxy_range=(96, 192), d=0.5e-3, dt=0.005, nsteps=400,
                  ckpt=40, power=2e9):
    """Batched adjoint workload: ``n`` instances, nz uniform in nz_range and ny,nx in nxy_range, per-voxel k a
    two-phase field (matrix 5 W/m/K, inclusions 0.3 W/m/K at 10% volume fraction), rho*c = 1550*1100, flash
    ``power`` W/m^3 in the top layer during the first 5 ms step, 400 steps, checkpoint every 40."""
    rng = np.random.default_rng(seed)
    out = []
    for c in range(n):
        nz = int(rng.integers(nz_range[0], nz_range[1] + 1))
        ny = int(rng.integers(nxy_range[0], nxy_range[1] + 1))
        nx = int(rng.integers(nxy_range[0], nxy_range[1] + 1))
        shape = (nz, ny, nx)
        k = two_phase_k(rng, shape)
        Cv = 1550.0 * 1100.0
        q = np.zeros(shape)
        q[0] = power
        schedule = np.zeros(nsteps)
        schedule[0] = 1.0
        obs = flash_observations(rng, shape, nsteps, dt, d, 5.0, Cv, power)
        out.append({"name": "adjoint_batch_%d" % c, "shape": shape, "spacing": (d, d, d), "dt": dt,
                    "nsteps": nsteps, "ckpt": ckpt, "k": k, "C": np.full(shape, Cv), "q": q,
                    "T0": np.full(shape, T_AMBIENT), "schedule": schedule, "obs": obs})
    return out
