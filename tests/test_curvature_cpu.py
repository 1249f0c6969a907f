"""The curved-surface mode's host compile against the reference's own outputs, on the CPU.

heatsim2_gb300.curvature turns a curved problem into per-row face conductances; tests/delta_model.py repeats
the device's factorisation and step on them in numpy.  On the curved golden fixtures (the reference run in
its curved-surface mode, crank_nicolson.pyx:388-457, by tests/golden/make_golden.py) the two agree with the
reference to rounding."""
import numpy as np
import pytest

from conftest import golden_files, load_golden, rel_err
import delta_model as DM
import oracle
import heatsim2_gb300 as hs
from heatsim2_gb300 import curvature, workloads as W
from heatsim2_gb300.crank_nicolson import ClassProblem

CURVED = golden_files(curved=True)


def test_curved_fixtures_exist():
    assert len(CURVED) >= 3


@pytest.mark.parametrize("path", CURVED, ids=lambda p: p.rsplit("/", 1)[-1])
def test_curved_rows_reproduce_reference(path):
    spec, times, ref = load_golden(path)
    args = W.setup_args(hs, spec)
    kw = W.setup_kwargs(spec)
    cp = ClassProblem(*args, **kw)
    r, volume = curvature.rows(cp, args[11], *cp.curvature)
    comp = r["fixed"] == 0
    c = DM.factor_rows(r["zlo"], r["zhi"], r["ylo"], r["yhi"], r["xlo"], r["xhi"], r["capacity"], comp)
    (z0, y0, x0, dz, dy, dx, nz, ny, nx, dt, mats, bnds, vol, me, bz, by, bx, ve) = args
    T = W.initial_temperature(spec)
    for n, t in enumerate(times):
        # the reference's source field with per-cell volumes (pyx:309-313) on the per-volume rows
        Q = oracle.source_field((nz, ny, nx), volume, t, dt, ve, vol)
        T = DM.step(c, T, Q)
        if n + 1 in ref:
            assert rel_err(T, ref[n + 1]) <= 1e-13, (n + 1)


def test_zero_curvature_rows_equal_flat_faces():
    spec = W.mixed_small()
    args = W.setup_args(hs, spec)
    cp = ClassProblem(*args)
    Gz, Gy, Gx, M, comp = DM.faces_from_classes(cp.shape, args[10], args[11], *cp.spacing, args[9], cp.mat, cp.bz,
                                                cp.by, cp.bx)
    zero = np.zeros(cp.shape[1:])
    r, volume = curvature.rows(cp, args[11], zero, zero)
    np.testing.assert_allclose(volume, np.prod(cp.spacing), rtol=1e-15)
    for name, g in (("zlo", Gz[:-1]), ("zhi", Gz[1:]), ("ylo", Gy[:, :-1]), ("yhi", Gy[:, 1:]),
                    ("xlo", Gx[:, :, :-1]), ("xhi", Gx[:, :, 1:])):
        np.testing.assert_allclose(r[name], np.where(comp, g, 0.0), rtol=1e-14, atol=0)


def test_non_monomial_boundary_class_is_refused():
    import types
    from heatsim2_gb300.expression import group
    mod = types.ModuleType("odd_boundary")

    def q(kl, kh, dz, dy, dx, Tl, Th, *rest):
        return -(kl + kh) * 0.5 * group((Th - Tl) * (1.0 / dy + 1.0 / dx))
    mod.qz = mod.qy = mod.qx = q
    with pytest.raises(NotImplementedError):
        curvature.flux_model((mod,), 1, 1e-3, 1e-3, 1e-3, [1.1], [0.9])


def test_batched_form_refuses_curved_problems():
    from heatsim2_gb300.batch import Batch
    spec = W.curved(W.mixed_small(), seed=1)
    kw = W.setup_kwargs(spec)
    args = W.setup_args(hs, spec) + (kw["top_surface_y_curvatures"], kw["top_surface_x_curvatures"])
    with pytest.raises(NotImplementedError):
        Batch([args], precision=64)
