"""Generate the golden fixtures in tests/golden/ by running the reference heatsim2 itself.

Run in a container where the reference sources are mounted (the reference is built into oracle/_ref by
oracle/build_ref.py first):

    python oracle/build_ref.py && python tests/golden/make_golden.py [curved | surface | composite128 | uneven |
        unaligned]

Each fixture ``<name>.npz`` holds the problem spec (heatsim2_gb300.workloads serialisation), the t values
passed to the reference's run_adi_steps, and the temperature field the reference returned after selected
steps.  ``stages_<name>.npz`` additionally holds the reference's per-stage tridiagonal A, sparse B / C and D
(alternatingdirection_c_pyx.pyx:120-284) for the coefficient-compiler tests, and ``tridiag.npz`` holds
tridiaglu / tridiagsolve results (tridiag.pyx:9-69) on random diagonally dominant systems.
"""
import contextlib
import io
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import build_ref  # noqa: E402
from heatsim2_gb300 import workloads as W  # noqa: E402


def quiet(fn, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


def run_reference(hs, spec, save_steps):
    P, S = quiet(hs.setup, *W.setup_args(hs, spec), **W.setup_kwargs(spec))
    vol = W.volumetric_tuple(hs, spec)
    T = W.initial_temperature(spec)
    times = W.step_times(spec)
    out = {}
    for n, t in enumerate(times):
        T = hs.run_adi_steps(P, S, t, spec["dt"], T, spec["arrays"]["volumetric"], vol)
        if (n + 1) in save_steps:
            out["T_%d" % (n + 1)] = np.array(T)
    return P, S, times, out


def save_fixture(name, spec, save_steps, hs, stages=False):
    P, S, times, res = run_reference(hs, spec, save_steps)
    d = W.spec_to_npz_dict(spec)
    d.update(res)
    d["times"] = np.array(times)
    d["save_steps"] = np.array(sorted(save_steps))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    if stages:
        sd = {}
        for s, st in enumerate(S):
            sd["A_%d" % s] = np.array(st.Amat)
            sd["D_%d" % s] = np.array(st.Dvec)
            sd["perm_%d" % s] = np.array(st.permuteorder)
            B = st.Bmat.tocoo()
            sd["B_%d_row" % s], sd["B_%d_col" % s], sd["B_%d_val" % s] = B.row, B.col, B.data
            for c, C in enumerate(st.Cmats):
                C = C.tocoo()
                sd["C_%d_%d_row" % (s, c)], sd["C_%d_%d_col" % (s, c)], sd["C_%d_%d_val" % (s, c)] = \
                    C.row, C.col, C.data
        np.savez_compressed(os.path.join(HERE, "stages_" + name + ".npz"), **sd)
    print("wrote", name, sorted(res))


def tridiag_fixture(hs_tridiag):
    rng = np.random.default_rng(11)
    d = {}
    for c, n in enumerate((1, 2, 5, 40, 64)):
        A = rng.uniform(-1, 1, size=(n, 3))
        A[:, 1] = 2.5 + rng.uniform(0, 1, size=n)
        A[0, 0] = 0.0
        A[-1, 2] = 0.0
        b = rng.uniform(-1, 1, size=n)
        L, U = hs_tridiag.tridiaglu(A.copy())
        x = hs_tridiag.tridiagsolve(L, U, b.copy())
        d["A_%d" % c], d["b_%d" % c], d["L_%d" % c], d["U_%d" % c], d["x_%d" % c] = A, b, L, U, x
    np.savez_compressed(os.path.join(HERE, "tridiag.npz"), **d)
    print("wrote tridiag")


def curved_fixtures(hs):
    """The reference's curved-surface mode (crank_nicolson.pyx:388-457)."""
    save_fixture("curved_mixed_small", W.curved(W.mixed_small(), seed=21), set(range(1, 7)), hs)
    save_fixture("curved_sources_small", W.curved(W.sources_small(), ky=15.0, kx=-10.0), set(range(1, 6)), hs)
    save_fixture("curved_steel_slab", W.curved(W.steel_slab(nsteps=20), seed=22, amplitude=8.0), {1, 5, 20}, hs)


def surface_fixture(hs):
    """The reference's surface-temperature estimate (heatsim2/surface_temperature.py:4-36) of seeded random
    fields and of the reference's own steel-slab states, for several layer thicknesses."""
    import heatsim2.surface_temperature as ref_surface
    rng = np.random.default_rng(31)
    d = {}
    fields = [293.0 + rng.random((2, 7, 9)), 293.0 + 50.0 * rng.random((5, 16, 12)),
              rng.standard_normal((3, 1, 4)) * 1e3]
    _, _, _, states = run_reference(hs, W.steel_slab(nsteps=12), {1, 12})
    fields += [np.ascontiguousarray(states["T_1"][:3]), np.ascontiguousarray(states["T_12"][:3])]
    dzs = [1e-3, 5e-4, 3.7e-3, 1e-3, 1e-3]
    for c, (F, dz) in enumerate(zip(fields, dzs)):
        d["T_%d" % c], d["dz_%d" % c] = F, np.float64(dz)
        d["surface_%d" % c] = ref_surface.insulating_z_min_surface_temperature(F, dz)
    np.savez_compressed(os.path.join(HERE, "surface_temperature.npz"), **d)
    print("wrote surface_temperature")


def composite_panel_128(hs):
    """The benchmark's composite panel recipe (anisotropic composite over aluminium, fixed ambient layer behind
    a thin-layer face h = 10, three seeded delaminations, 2e9 W/m^3 flash) at 65 x 128 x 128, 100 steps of the
    reference.  Only the layers that left the ambient temperature are stored (the rest are checked to be
    exactly 293 K), which keeps the fixture small."""
    spec = W.composite_panel(seed=1, nz=64, ny=128, nx=128, nsteps=100)
    P, S, times, res = run_reference(hs, spec, {1, 20, 100})
    d = W.spec_to_npz_dict(spec)
    d["times"] = np.array(times)
    d["save_steps"] = np.array([1, 20, 100])
    for key, T in res.items():
        moved = np.nonzero((T != 293.0).any(axis=(1, 2)))[0]
        nk = int(moved.max()) + 1 if moved.size else 0
        d[key + "_top"] = np.ascontiguousarray(T[:nk])
        d[key + "_nz"] = np.int64(T.shape[0])
        print(key, "layers away from ambient:", nk)
    np.savez_compressed(os.path.join(HERE, "composite_panel_128.npz"), **d)
    print("wrote composite_panel_128")


def uneven_batch_sample(hs):
    """Instances 0 (steel slab, 57 x 114 x 85) and 2 (composite panel, 60 x 74 x 171) of the 256-instance
    uneven batch the benchmark runs (seed 2), 10 steps of the reference each.  Stored per instance: the spec, the
    top plane after step 1 and, after step 10, the top plane and the x-z and y-z slices through the middle of the
    grid (the whole fields would make the fixture megabytes)."""
    specs = W.uneven_batch(seed=2, n=3, nsteps=10)
    d = {"instances": np.array([0, 2])}
    for n in (0, 2):
        spec = specs[n]
        _, _, times, res = run_reference(hs, spec, {1, 10})
        for key, val in W.spec_to_npz_dict(spec).items():
            d["i%d_%s" % (n, key)] = val
        d["i%d_times" % n] = np.array(times)
        T1, T10 = res["T_1"], res["T_10"]
        nz, ny, nx = T10.shape
        d["i%d_top_1" % n] = np.ascontiguousarray(T1[0])
        d["i%d_top_10" % n] = np.ascontiguousarray(T10[0])
        d["i%d_xz_10" % n] = np.ascontiguousarray(T10[:, ny // 2, :])
        d["i%d_yz_10" % n] = np.ascontiguousarray(T10[:, :, nx // 2])
        print("instance", n, T10.shape, "max |T - 293| %.3g" % np.abs(T10 - 293.0).max())
    np.savez_compressed(os.path.join(HERE, "uneven_batch_sample.npz"), **d)
    print("wrote uneven_batch_sample")


def unaligned_fixture(hs):
    """What the reference's setup does with unaligned_anisotropic=True (alternatingdirection_c_pyx.pyx:511-564,
    crank_nicolson.pyx:140-143) on a tensor aligned with the axes, an unaligned tensor and a scalar-k slab with
    fixed voxels: the exception type and where it was raised, or the stage count if it returned."""
    import json
    import traceback
    cases = {}
    for label, k, bnd in (("aligned_tensor", [[5.0, 0, 0], [0, 4.0, 0], [0, 0, 3.0]], "conducting_anisotropic"),
                          ("unaligned_tensor", [[5.0, 0.3, 0.0], [0.3, 5.0, 0.0], [0.0, 0.0, 5.0]],
                           "conducting_anisotropic"),
                          ("scalar_k", None, None)):
        spec = W.line_grid((3, 4, 5)) if k is not None else W.mixed_small()
        if k is not None:
            spec["boundaries"][0] = [bnd]
            spec["materials"][0][1] = k
        try:
            P, S = quiet(hs.setup, *W.setup_args(hs, spec), unaligned_anisotropic=True)
            cases[label] = {"returned_stages": len(S)}
        except Exception as e:
            fr = traceback.extract_tb(e.__traceback__)[-1]
            cases[label] = {"raised": type(e).__name__, "file": os.path.basename(fr.filename), "line": fr.lineno}
    with open(os.path.join(HERE, "unaligned_anisotropic.json"), "w") as fh:
        json.dump(cases, fh, indent=1, sort_keys=True)
    print("wrote unaligned_anisotropic", cases)


def main():
    if not build_ref.available():
        build_ref.build()
    hs = build_ref.import_reference()
    if len(sys.argv) > 1 and sys.argv[1] == "curved":
        curved_fixtures(hs)
        return
    if len(sys.argv) > 1 and sys.argv[1] == "unaligned":
        unaligned_fixture(hs)
        return
    if len(sys.argv) > 1 and sys.argv[1] == "composite128":
        composite_panel_128(hs)
        return
    if len(sys.argv) > 1 and sys.argv[1] == "surface":
        surface_fixture(hs)
        return
    if len(sys.argv) > 1 and sys.argv[1] == "uneven":
        uneven_batch_sample(hs)
        return
    import heatsim2.tridiag as ref_tridiag
    tridiag_fixture(ref_tridiag)

    save_fixture("steel_slab", W.steel_slab(), {1, 2, 10, 50, 200}, hs)
    save_fixture("composite_small",
                 W.composite_panel(seed=1, nz=24, ny=32, nx=32, top_layers=6, width_range=(4, 12),
                                   depth_range=(2, 12), nsteps=20),
                 {1, 5, 20}, hs, stages=False)
    save_fixture("mixed_small", W.mixed_small(), set(range(1, 7)), hs, stages=True)
    save_fixture("sources_small", W.sources_small(), set(range(1, 6)), hs, stages=True)
    for shape in ((1, 1, 7), (7, 1, 1), (1, 7, 1), (1, 1, 1), (1, 5, 6), (4, 1, 5), (3, 4, 1)):
        save_fixture("line_%dx%dx%d" % shape, W.line_grid(shape), set(range(1, 6)), hs)
    curved_fixtures(hs)
    surface_fixture(hs)
    composite_panel_128(hs)
    uneven_batch_sample(hs)
    unaligned_fixture(hs)


if __name__ == "__main__":
    main()
