"""The surface-temperature estimate (reference heatsim2/surface_temperature.py:4-36) without a GPU.

The oracle's restatement equals the reference's own function bit for bit on the golden fixture (seeded random
fields and the reference's steel-slab states, tests/golden/make_golden.py); the package's drop-in function and
``run(record_surface=True)`` refuse inputs the estimate is not defined for before any device work."""
import os

import numpy as np
import pytest

import oracle
from heatsim2_gb300 import surface_temperature as ST

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "surface_temperature.npz")


def test_oracle_matches_reference_fixture():
    d = np.load(GOLDEN)
    n = sum(1 for k in d.files if k.startswith("T_"))
    assert n == 5
    for c in range(n):
        out = oracle.insulating_z_min_surface_temperature(d["T_%d" % c], float(d["dz_%d" % c]))
        np.testing.assert_array_equal(out, d["surface_%d" % c])


def test_estimate_is_between_extrapolations():
    """Constant layers give the layer value; a linear profile gives T0 - (5/16)(T1 - T0)."""
    T = np.empty((2, 3, 4))
    T[0], T[1] = 300.0, 300.0
    np.testing.assert_array_equal(oracle.insulating_z_min_surface_temperature(T, 1e-3), np.full((3, 4), 300.0))
    T[1] = 301.6
    out = oracle.insulating_z_min_surface_temperature(T, 1e-3)
    assert np.allclose(out, 300.0 - 5.0 / 16.0 * 1.6, rtol=0, atol=1e-12)


@pytest.mark.parametrize("shape", [(1, 4, 4), (4, 4)])
def test_drop_in_refuses_fields_without_two_layers(shape):
    with pytest.raises(ValueError):
        ST.insulating_z_min_surface_temperature(np.zeros(shape), 1e-3)


def test_installed_as_heatsim2_submodule():
    """``import heatsim2.surface_temperature`` resolves to the drop-in after install_as_heatsim2()."""
    import sys
    import heatsim2_gb300
    saved = {k: v for k, v in sys.modules.items() if k == "heatsim2" or k.startswith("heatsim2.")}
    try:
        heatsim2_gb300.install_as_heatsim2()
        import heatsim2.surface_temperature as m
        assert m is ST
        assert m.insulating_z_min_surface_temperature is ST.insulating_z_min_surface_temperature
    finally:
        for k in [k for k in sys.modules if k == "heatsim2" or k.startswith("heatsim2.")]:
            del sys.modules[k]
        sys.modules.update(saved)
