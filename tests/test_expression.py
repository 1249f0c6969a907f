"""Boundary classes evaluate into the face conductances the reference's heat balance implies
(crank_nicolson.pyx:359-363 with the four boundary_* modules), and forms the 3-stage step cannot solve are
flagged.  Pure host logic, no GPU."""
import types

import numpy as np
import pytest

import heatsim2_gb300 as hs
from heatsim2_gb300 import _native
from heatsim2_gb300.crank_nicolson import evaluate_boundary
from heatsim2_gb300.expression import linear_expression, group, ExpressionError

DZ, DY, DX = 1e-3, 2e-3, 0.5e-3
D = (DZ, DY, DX)
K = _native.K_ENTRIES


def _entries(G):
    return {i: v for i, v in enumerate(G) if v}


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_conducting(axis):
    G, zeros = evaluate_boundary((hs.boundary_conducting,), axis, *D)
    d = D[axis]
    assert zeros == []
    assert _entries(G) == pytest.approx({1: 0.5 / d / d, 1 + K: 0.5 / d / d}, rel=1e-15)


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_anisotropic(axis):
    G, zeros = evaluate_boundary((hs.boundary_conducting_anisotropic,), axis, *D)
    d = D[axis]
    e = 1 + 1 + 4 * axis                                  # K[axis][axis]
    assert _entries(G) == pytest.approx({e: 0.5 / d / d, e + K: 0.5 / d / d}, rel=1e-15)
    # cross terms K[axis][b != axis] must vanish on every face: all flagged as unaligned
    assert zeros and all(code == _native.ERR_UNALIGNED for code, _ in zeros)
    used = {i for _, f in zeros for i, v in enumerate(f) if v}
    diag = {1 + 1 + 4 * axis, 1 + 1 + 4 * axis + K}
    assert used and not (used & diag)


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_thin_layer(axis):
    G, zeros = evaluate_boundary((hs.boundary_thininsulatinglayer, 250.0), axis, *D)
    assert zeros == []
    assert _entries(G) == pytest.approx({0: 250.0 / D[axis]}, rel=1e-15)


def test_insulating():
    for axis in range(3):
        G, zeros = evaluate_boundary((hs.boundary_insulating,), axis, *D)
        assert not np.any(G) and zeros == []


def _module(qz):
    m = types.ModuleType("custom_boundary")
    m.qz = m.qy = m.qx = qz
    return m


def test_ungrouped_flux_is_flagged():
    m = _module(lambda kl, kh, dz, dy, dx, Tl, Th, *rest: -5.0 * (Th - Tl))
    G, zeros = evaluate_boundary((m,), 0, *D)
    assert not np.any(G)
    assert [c for c, _ in zeros] == [_native.ERR_FORM, _native.ERR_FORM] or \
        {c for c, _ in zeros} == {_native.ERR_FORM}


def test_unbalanced_flux_is_flagged():
    m = _module(lambda kl, kh, dz, dy, dx, Tl, Th, *rest: -5.0 * group(Th - 0.5 * Tl))
    G, zeros = evaluate_boundary((m,), 0, *D)
    assert _entries(G) == pytest.approx({0: 5.0 / DZ})
    assert [c for c, _ in zeros] == [_native.ERR_FORM]


def test_constant_flux_is_flagged():
    m = _module(lambda kl, kh, dz, dy, dx, Tl, Th, *rest: 3.0 - 2.0 * group(Th - Tl))
    _, zeros = evaluate_boundary((m,), 1, *D)
    assert [c for c, _ in zeros] == [_native.ERR_FORM]


def test_mixed_group_is_flagged():
    def q(kl, kh, dz, dy, dx, Tl, Th, T1, T2, *rest):
        return -(kl + kh) * group((Th - Tl) + 0.1 * (T2 - T1))
    _, zeros = evaluate_boundary((_module(q),), 2, *D)
    assert {c for c, _ in zeros} == {_native.ERR_UNALIGNED}


def test_user_module_with_k_dependent_thin_layer():
    # q = -(k_lo/l) (T_hi - T_lo): conductance depends on one side's k only
    m = _module(lambda kl, kh, dz, dy, dx, Tl, Th, *rest: -(kl * 100.0) * group(Th - Tl))
    G, zeros = evaluate_boundary((m,), 0, *D)
    assert zeros == [] and _entries(G) == pytest.approx({1: 100.0 / DZ})


def test_nonlinear_expressions_raise():
    k = linear_expression("kmat_lo")
    T = linear_expression("Tp55")
    with pytest.raises(ExpressionError):
        k * k
    with pytest.raises(ExpressionError):
        T * T
    with pytest.raises(ExpressionError):
        1.0 / T
    with pytest.raises(ExpressionError):
        T[0, 0]


def test_group_and_index_algebra():
    k = linear_expression("kmat_lo") + linear_expression("kmat_hi")
    e = -(k * 0.5)[1, 1] * group(linear_expression("T5p5") - linear_expression("T5m5")) / 2.0
    terms = e.temperature_terms()
    assert len(terms) == 2
    (t1, g1), (t2, g2) = sorted(terms)
    assert g1 == g2 and g1 is not None
    assert sorted(c for _, _, c in terms[(t1, g1)]) == [0.25, 0.25] or \
        sorted(c for _, _, c in terms[(t1, g1)]) == [-0.25, -0.25]
