import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libhs2g.so")
    config.addinivalue_line("markers", "slow: long-running")


def golden_files(include_big=True, curved=False):
    """The reference's output fixtures: flat problems, or (curved=True) those in the curved-surface mode."""
    out = []
    for f in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        b = os.path.basename(f)
        if b.startswith("stages_") or b in ("tridiag.npz", "surface_temperature.npz", "uneven_batch_sample.npz"):
            continue
        if b.startswith("curved_") != curved:
            continue
        out.append(f)
    return out


def load_golden(path):
    """(spec, times, {step: T}) of a fixture.  A fixture may store only the leading z layers of a field that
    left the ambient temperature ("T_<n>_top", with the layer count in "T_<n>_nz"); the rest of the field was
    exactly the ambient 293 K in the reference's output and is filled in here."""
    from heatsim2_gb300 import workloads as W
    z = np.load(path)
    spec = W.spec_from_npz(z)
    steps = {}
    for k in z.files:
        if not k.startswith("T_"):
            continue
        if k.endswith("_top"):
            n = int(k[2:-4])
            top = np.array(z[k])
            T = np.full((int(z["T_%d_nz" % n]),) + top.shape[1:], 293.0)
            T[:top.shape[0]] = top
            steps[n] = T
        elif not k.endswith("_nz"):
            steps[int(k[2:])] = np.array(z[k])
    return spec, [float(t) for t in z["times"]], steps


def load_uneven_sample():
    """The reference's outputs for instances 0 and 2 of the benchmark's uneven batch (tests/golden/make_golden.py
    uneven): {instance: (spec, times, {"top_1", "top_10", "xz_10", "yz_10"})} -- the top plane after steps 1 and
    10 and the x-z / y-z slices through the middle of the grid after step 10."""
    from heatsim2_gb300 import workloads as W
    z = np.load(os.path.join(GOLDEN, "uneven_batch_sample.npz"))
    out = {}
    for n in (int(v) for v in z["instances"]):
        spec = W.spec_from_npz(z, prefix="i%d_spec_" % n)
        ref = {k: np.array(z["i%d_%s" % (n, k)]) for k in ("top_1", "top_10", "xz_10", "yz_10")}
        out[n] = (spec, [float(t) for t in z["i%d_times" % n]], ref)
    return out


def uneven_sample_slices(T):
    """The slices of a field that the uneven-batch fixture stores: top plane, middle x-z and y-z slices."""
    nz, ny, nx = T.shape
    return {"top": T[0], "xz": T[:, ny // 2, :], "yz": T[:, :, nx // 2]}


def rel_err(a, ref):
    a = np.asarray(a)
    ref = np.asarray(ref)
    return float(np.abs(a - ref).max() / np.abs(ref).max())


@pytest.fixture(scope="session")
def cuda_ok():
    try:
        import torch
    except ImportError:
        pytest.skip("torch missing")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return True
