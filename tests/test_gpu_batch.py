"""Batched form (heatsim2_gb300.batch.Batch): uneven instances advanced together must give, instance by
instance, the single-problem result (FP64: bit for bit, the same FMAs in the same order), and the FP32 variant
stays within its stated error of FP64."""
import numpy as np
import pytest

from conftest import load_uneven_sample, rel_err, uneven_sample_slices
import oracle
from oracle_shim import HS
import heatsim2_gb300 as hs
from heatsim2_gb300 import workloads as W
from heatsim2_gb300.batch import Batch

pytestmark = pytest.mark.gpu


def _instances():
    return [
        W.steel_slab(seed=11, nz=7, ny=13, nx=10, flaw=4, depth_range=(2, 4), nsteps=6),
        W.composite_panel(seed=12, nz=9, ny=20, nx=33, top_layers=3, n_delams=2, width_range=(3, 9),
                          depth_range=(2, 6), nsteps=6),
        W.steel_slab(seed=13, nz=5, ny=34, nx=71, flaw=6, depth_range=(1, 3), nsteps=6),
        W.composite_panel(seed=14, nz=12, ny=9, nx=40, top_layers=4, n_delams=1, width_range=(3, 7),
                          depth_range=(2, 8), nsteps=6),
        W.line_grid((1, 1, 9)),
    ]


def _single(spec, nsteps):
    P, S = hs.setup(*W.setup_args(hs, spec))
    vol = W.volumetric_tuple(hs, spec)
    T = W.initial_temperature(spec)
    for t in W.step_times(spec, nsteps):
        T = hs.run_adi_steps(P, S, t, spec["dt"], T, spec["arrays"]["volumetric"], vol)
    return T


def _batch(specs, nsteps, precision=64, tune=False, split=None):
    b = Batch([W.setup_args(hs, s) for s in specs], precision=precision)
    b.set_temperature([W.initial_temperature(s) for s in specs])
    b.set_sources(W.step_times(specs[0], nsteps), specs[0]["dt"])
    if tune:
        b.autotune()
    if split:
        b.run(split)
        b.run(nsteps - split)
    else:
        b.run(nsteps)
    return b.get_temperature()


def test_batch_fp64_equals_single_problem_path(cuda_ok):
    specs = _instances()
    for s in specs:
        s["dt"] = 0.01      # one source schedule for the batch
    got = _batch(specs, 6)
    for spec, T in zip(specs, got):
        np.testing.assert_array_equal(T, _single(spec, 6))


def test_batch_autotune_and_split_runs_keep_results(cuda_ok):
    specs = _instances()
    for s in specs:
        s["dt"] = 0.01
    a = _batch(specs, 5)
    b = _batch(specs, 5, tune=True, split=2)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_batch_fp32_error_against_fp64(cuda_ok):
    specs = _instances()[:4]
    for s in specs:
        s["dt"] = 0.01
    f64 = _batch(specs, 6)
    f32 = _batch(specs, 6, precision=32)
    worst = max(rel_err(b, a) for a, b in zip(f64, f32))
    # float state as offsets from the initial mean: relative error ~1e-8 of max|T| (1e-6 without the offset)
    assert worst < 1e-7, worst


def _oracle(spec, nsteps):
    Po, _ = oracle.setup(*W.setup_args(HS, spec))
    vol = W.volumetric_tuple(HS, spec)
    T = W.initial_temperature(spec)
    for t in W.step_times(spec, nsteps):
        T = oracle.run_adi_steps(Po, None, t, spec["dt"], T, spec["arrays"]["volumetric"], vol)
    return T


def test_benchmark_batch_instances_vs_oracle(cuda_ok):
    """The first 8 instances of the 256-instance benchmark batch (seed 2: nz 16..64, ny and nx 64..256, odd
    row widths among them, steel and composite), 10 steps in one batched state.  Each instance is compared
    with the oracle: FP64 within 1e-12 of max|T|, the FP32 variant within 1e-7 (its stated error is ~1e-8)."""
    nsteps = 10
    specs = W.uneven_batch(seed=2, n=8, nsteps=nsteps)
    assert sum(s["grid"]["nx"] % 2 for s in specs) >= 3
    assert max(s["grid"]["ny"] for s in specs) >= 200
    f64 = _batch(specs, nsteps)
    f32 = _batch(specs, nsteps, precision=32)
    worst64 = worst32 = 0.0
    for spec, a, b in zip(specs, f64, f32):
        ref = _oracle(spec, nsteps)
        assert np.abs(ref - 293.0).max() > 1.0            # the flash reached the field
        worst64 = max(worst64, rel_err(a, ref))
        worst32 = max(worst32, rel_err(b, ref))
    print("batch vs oracle: FP64 %.2e, FP32 %.2e" % (worst64, worst32))
    assert worst64 <= 1e-12, worst64
    assert worst32 <= 1e-7, worst32


def test_benchmark_batch_instances_vs_reference(cuda_ok):
    """Instances 0 and 2 of the benchmark's 256-instance uneven batch (57x114x85 steel slab, 60x74x171 composite
    panel: odd row widths), advanced together in one batched state and compared with the reference's own output
    (tests/golden/uneven_batch_sample.npz): the top plane after step 1 and, after step 10, the top plane and the
    x-z / y-z slices through the middle of each grid.  FP64 within 1e-12 of max|T|, FP32 within 1e-7."""
    sample = load_uneven_sample()
    specs = [sample[n][0] for n in sorted(sample)]
    times = sample[min(sample)][1]
    assert all(sample[n][1] == times for n in sample)     # one source schedule for the batch
    for precision, tol in ((64, 1e-12), (32, 1e-7)):
        b = Batch([W.setup_args(hs, s) for s in specs], precision=precision)
        b.set_temperature([W.initial_temperature(s) for s in specs])
        b.set_sources(times, specs[0]["dt"])
        b.run(1)
        worst = 0.0
        for n, T in zip(sorted(sample), b.get_temperature()):
            worst = max(worst, rel_err(T[0], sample[n][2]["top_1"]))
        b.run(len(times) - 1)
        for n, T in zip(sorted(sample), b.get_temperature()):
            sl = uneven_sample_slices(T)
            for key in ("top", "xz", "yz"):
                worst = max(worst, rel_err(sl[key], sample[n][2][key + "_10"]))
        print("batch FP%d vs reference: %.2e" % (precision, worst))
        assert worst <= tol, (precision, worst)
