"""The oracle (oracle/adi_oracle.c + oracle/oracle.py) pinned against the reference's own outputs.

tests/golden/*.npz were generated by running the reference heatsim2 (tests/golden/make_golden.py); the oracle
must reproduce them.  It restates the reference's arithmetic in the same order, so agreement is bit-exact on
every fixture; the tolerance allows 1e-14 to stay robust to compiler contraction differences."""
import numpy as np
import pytest

from conftest import golden_files, load_golden, load_uneven_sample, rel_err, uneven_sample_slices, GOLDEN

import oracle
from oracle_shim import HS  # noqa: F401  (module-like names for the oracle)
from heatsim2_gb300 import workloads as W


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.rsplit("/", 1)[-1])
def test_oracle_matches_reference(path):
    spec, times, ref = load_golden(path)
    P, _ = oracle.setup(*W.setup_args(HS, spec))
    vol = W.volumetric_tuple(HS, spec)
    T = W.initial_temperature(spec)
    for n, t in enumerate(times):
        T = oracle.run_adi_steps(P, None, t, spec["dt"], T, spec["arrays"]["volumetric"], vol)
        if n + 1 in ref:
            assert rel_err(T, ref[n + 1]) <= 1e-14, (n + 1)


def test_oracle_matches_reference_on_benchmark_batch_instances():
    """Instances 0 and 2 of the benchmark's 256-instance uneven batch (a 57x114x85 steel slab and a 60x74x171
    composite panel, odd row widths), 10 steps: the oracle reproduces the reference's stored planes and slices."""
    for n, (spec, times, ref) in load_uneven_sample().items():
        P, _ = oracle.setup(*W.setup_args(HS, spec))
        vol = W.volumetric_tuple(HS, spec)
        T = W.initial_temperature(spec)
        for k, t in enumerate(times):
            T = oracle.run_adi_steps(P, None, t, spec["dt"], T, spec["arrays"]["volumetric"], vol)
            if k == 0:
                assert rel_err(T[0], ref["top_1"]) <= 1e-14, n
        sl = uneven_sample_slices(T)
        for key in ("top", "xz", "yz"):
            assert rel_err(sl[key], ref[key + "_10"]) <= 1e-14, (n, key)


def test_oracle_tridiag_matches_reference():
    z = np.load(GOLDEN + "/tridiag.npz")
    c = 0
    while "A_%d" % c in z.files:
        A, b = z["A_%d" % c], z["b_%d" % c]
        L, U = oracle.tridiaglu(A)
        np.testing.assert_array_equal(L, z["L_%d" % c])
        np.testing.assert_array_equal(U, z["U_%d" % c])
        np.testing.assert_array_equal(oracle.tridiagsolve(L, U, b), z["x_%d" % c])
        c += 1
    assert c == 5


def _coo_dense(z, prefix, n):
    M = np.zeros((n, n))
    np.add.at(M, (z[prefix + "_row"], z[prefix + "_col"]), z[prefix + "_val"])
    return M


@pytest.mark.parametrize("name", ["mixed_small", "sources_small"])
def test_oracle_stage_matrices_match_reference(name):
    spec, _, _ = load_golden(GOLDEN + "/%s.npz" % name)
    st = np.load(GOLDEN + "/stages_%s.npz" % name)
    P, _ = oracle.setup(*W.setup_args(HS, spec))
    n = W.voxels(spec)
    for s in range(3):
        A, (br, bc, bv), Cs, D = P.stage_matrices(s)
        np.testing.assert_allclose(A, st["A_%d" % s], rtol=1e-14, atol=0)
        np.testing.assert_array_equal(D, st["D_%d" % s])
        B = np.zeros((n, n))
        np.add.at(B, (br, bc), bv)
        np.testing.assert_allclose(B, _coo_dense(st, "B_%d" % s, n), rtol=1e-13, atol=1e-6)
        for c, (cr, cc, cv) in enumerate(Cs):
            C = np.zeros((n, n))
            np.add.at(C, (cr, cc), cv)
            np.testing.assert_allclose(C, _coo_dense(st, "C_%d_%d" % (s, c), n), rtol=1e-13, atol=1e-6)


def test_oracle_rejects_conducting_exterior_face():
    spec = W.line_grid((2, 3, 4))
    spec["arrays"]["boundary_x"][:, :, -1] = 0      # conducting class on the exterior
    with pytest.raises(ValueError):
        oracle.setup(*W.setup_args(HS, spec))
