"""The scaled delta-form Douglas step the CUDA kernels compute equals the reference's stage equations.

tests/delta_model.py repeats the kernels' arithmetic in numpy; here it runs on the small golden fixtures
(generated by the reference) on the CPU, with the oracle's source evaluation.  Agreement is at rounding level
(<= 1e-13 relative), far inside the 1e-12 bar the GPU path is held to."""
import numpy as np
import pytest

from conftest import golden_files, load_golden, rel_err
import delta_model as DM
import oracle
import heatsim2_gb300 as hs
from heatsim2_gb300 import workloads as W

SMALL = [p for p in golden_files()
         if not p.endswith(("steel_slab.npz", "composite_small.npz", "composite_panel_128.npz"))]


@pytest.mark.parametrize("path", SMALL, ids=lambda p: p.rsplit("/", 1)[-1])
def test_delta_form_matches_reference(path):
    spec, times, ref = load_golden(path)
    (z0, y0, x0, dz, dy, dx, nz, ny, nx, dt, mats, bnds, vol, me, bz, by, bx, ve) = W.setup_args(hs, spec)
    Gz, Gy, Gx, M, comp = DM.faces_from_classes((nz, ny, nx), mats, bnds, dz, dy, dx, dt, me, bz, by, bx)
    c = DM.factor(Gz, Gy, Gx, M, comp)
    T = W.initial_temperature(spec)
    for n, t in enumerate(times):
        Q = oracle.source_field((nz, ny, nx), dz * dy * dx, t, dt, ve, vol)
        T = DM.step(c, T, Q)
        if n + 1 in ref:
            assert rel_err(T, ref[n + 1]) <= 1e-13
