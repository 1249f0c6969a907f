"""libhs2g.so loads and exports every entry point include/hs2g.h declares; host-only entry points behave.

No GPU needed: only calls that return before touching CUDA are made here."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from heatsim2_gb300 import _native
import oracle


def _declared():
    src = open(os.path.join(ROOT, "include", "hs2g.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|int64_t|const char\*)\s+(hs2g_\w+)\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_native.LIB_PATH):
        from heatsim2_gb300 import build
        build.build()
    return _native.load()


def test_exports_every_declared_symbol(lib):
    declared = _declared()
    assert set(declared) == set(_native.EXPORTED)
    for name in declared:
        assert hasattr(lib, name), name


def test_abi_version(lib):
    assert lib.hs2g_abi_version() == _native.ABI_VERSION


def test_struct_layouts_match_header():
    assert ctypes.sizeof(_native.Material) == 4 + 4 + 8 * _native.K_ENTRIES + 8
    assert ctypes.sizeof(_native.FaceForm) == 8 * _native.FORM_LEN + 4 + 4 * _native.MAX_ZERO_FORMS + 4 + \
        8 * _native.FORM_LEN * _native.MAX_ZERO_FORMS


def test_create_rejects_bad_arguments_before_touching_the_device(lib):
    prob = _native.ClassProblem()
    h = ctypes.c_void_p()
    assert lib.hs2g_create_classes(None, 0, ctypes.byref(h)) == _native.ERR_ARG
    assert lib.hs2g_create_classes(ctypes.byref(prob), 0, ctypes.byref(h)) == _native.ERR_ARG
    assert b"null" in lib.hs2g_last_error()
    assert lib.hs2g_step(None, None, None, None, None, None, 0) == _native.ERR_ARG


SOURCES = [
    (0, []), (1, [0.02, 5e4]), (2, [0.01, 0.03, 7e8]), (3, [0.02, 0.25]), (2, [0.0, 0.005, 2e9]),
]


@pytest.mark.parametrize("t", [0.0, 0.005, 0.01, 0.02, 0.03, 0.030000000000000002, 0.04])
def test_source_table_matches_oracle(lib, t):
    dt, vol = 0.01, 1e-9
    kind = np.array([k for k, _ in SOURCES], dtype=np.int32)
    params = np.zeros((len(SOURCES), 4))
    for c, (_, p) in enumerate(SOURCES):
        params[c, :len(p)] = p
    q = np.zeros(256)
    n = lib.hs2g_source_table(len(SOURCES), kind.ctypes.data, params.ctypes.data, t, dt, vol, q.ctypes.data)
    assert n == int(np.count_nonzero(q))
    ve = np.arange(len(SOURCES), dtype=np.uint8).reshape(1, 1, -1)
    tuples = [(k,) + tuple(p) for k, p in SOURCES]
    ref = oracle.source_field(ve.shape, vol, t, dt, ve, tuples).reshape(-1)
    np.testing.assert_array_equal(q[:len(SOURCES)], ref)
    assert not q[len(SOURCES):].any()


def test_source_table_rejects_per_voxel_kinds(lib):
    kind = np.array([4], dtype=np.int32)
    params = np.zeros((1, 4))
    q = np.zeros(256)
    assert lib.hs2g_source_table(1, kind.ctypes.data, params.ctypes.data, 0.0, 0.01, 1.0, q.ctypes.data) == \
        _native.ERR_ARG
