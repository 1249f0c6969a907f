"""CPU oracle for heatsim2's ADI Crank-Nicolson timestep -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs may import this module, and
only as the checker (or the timed CPU baseline); the product path never routes through it.

Pinned against the reference itself: tests/test_oracle.py checks this oracle against the golden fixtures in
tests/golden/, which tests/golden/make_golden.py generated by running the reference heatsim2 (built from its
.pyx sources by oracle/build_ref.py).

``setup`` / ``run_adi_steps`` take the reference's arguments (crank_nicolson.pyx:128-142,
alternatingdirection_c_pyx.pyx:287) with any module's boundary classes; the four built-in boundary classes are
recognised by module name.  The heat balance, stage matrices and solves are in adi_oracle.c (plain C);
the source field is evaluated here (``source_field``, restating alternatingdirection_c_pyx.pyx:294-386).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libadi_oracle.so")

COMPUTE, FIXED = 0, 1          # heatsim2/__init__.py:42-43
NO_SOURCE, IMPULSE_SOURCE, STEPPED_SOURCE, IMPULSE_POINT_SOURCE_JOULES, \
    SPATIALLY_Z_DECAYING_TEMPORAL_IMPULSE = 0, 1, 2, 3, 4   # heatsim2/__init__.py:46-50
BND_KIND = {"boundary_insulating": 0, "boundary_conducting": 1, "boundary_conducting_anisotropic": 2,
            "boundary_thininsulatinglayer": 3}
ERRORS = {-2: "non-insulating exterior face", -3: "boundary class does not match the material's k type",
          -4: "out of memory", -5: "bad argument"}


def build(force=False):
    """Compile adi_oracle.c into oracle/libadi_oracle.so (plain gcc, no other dependencies)."""
    src = os.path.join(HERE, "adi_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-shared", "-fPIC", "-o", LIB_PATH, src])
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp, i64, dp = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double
        L.oracle_setup.argtypes = [i64, i64, i64, dp, dp, dp, vp, vp, vp, vp, ctypes.c_int, vp, vp, vp, vp,
                                   ctypes.c_int, vp, vp, ctypes.POINTER(vp)]
        L.oracle_setup.restype = ctypes.c_int
        L.oracle_step.argtypes = [vp, vp, vp, vp]
        L.oracle_step.restype = ctypes.c_int
        L.oracle_free.argtypes = [vp]
        L.oracle_export.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp]
        L.oracle_export.restype = i64
        L.oracle_tridiaglu.argtypes = [i64, vp, vp, vp]
        L.oracle_tridiagsolve.argtypes = [i64, vp, vp, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def tridiaglu(A):
    A = np.ascontiguousarray(A, dtype="d")
    L = np.zeros_like(A)
    U = np.zeros_like(A)
    lib().oracle_tridiaglu(A.shape[0], _p(A), _p(L), _p(U))
    return L, U


def tridiagsolve(L, U, b):
    L, U, b = (np.ascontiguousarray(v, dtype="d") for v in (L, U, b))
    x = np.zeros_like(b)
    lib().oracle_tridiagsolve(b.shape[0], _p(L), _p(U), _p(b), _p(x))
    return x


class OracleParams:
    """What the oracle's setup returns in place of the reference's (ADI_params, ADI_steps)."""

    def __init__(self, handle, shape, volume):
        self.handle = handle
        self.shape = shape
        self.volume_array = volume

    def __del__(self):
        if self.handle and _lib is not None:
            _lib.oracle_free(self.handle)
            self.handle = None

    def stage_matrices(self, s):
        """(A (n,3), B COO triple, [C_j COO triples], D) of stage s, rows/cols in the stage's permuted order."""
        n = int(np.prod(self.shape))
        A = np.zeros((n, 3))
        D = np.zeros(n)
        out = []
        for which in range(1 + s):
            cnt = lib().oracle_export(self.handle, s, which, None, None, None, None, None)
            r = np.zeros(cnt, dtype=np.int64)
            c = np.zeros(cnt, dtype=np.int64)
            v = np.zeros(cnt)
            lib().oracle_export(self.handle, s, which, _p(A), _p(D), _p(r), _p(c), _p(v))
            out.append((r, c, v))
        return A, out[0], out[1:], D


def _module_kind(mod):
    name = getattr(mod, "__name__", "").rsplit(".", 1)[-1]
    if name not in BND_KIND:
        raise NotImplementedError("oracle knows only the four built-in boundary classes, got %r" % (name,))
    return BND_KIND[name]


def setup(z0, y0, x0, dz, dy, dx, nz, ny, nx, dt, materials, boundaries, volumetric, material_elements,
          boundary_z_elements, boundary_y_elements, boundary_x_elements, volumetric_elements, **kwargs):
    """crank_nicolson.pyx:128-498 (no curvature, aligned anisotropy only)."""
    if kwargs.get("top_surface_y_curvatures") is not None or kwargs.get("top_surface_x_curvatures") is not None:
        raise NotImplementedError("curvature")
    nmat = len(materials)
    kind = np.zeros(nmat, dtype=np.int32)
    ismat = np.zeros(nmat, dtype=np.int32)
    kk = np.zeros((nmat, 3))
    M = np.zeros(nmat)
    for m, mat in enumerate(materials):
        if mat[0] == COMPUTE:
            (_, k, rho, c) = mat
            kind[m] = COMPUTE
            if isinstance(k, np.ndarray) and k.ndim == 2:
                if np.any(k - np.diag(np.diag(k))):
                    raise NotImplementedError("unaligned anisotropy")
                ismat[m] = 1
                kk[m] = np.diag(k)
            else:
                kk[m, 0] = float(k)
            M[m] = rho * c * (1.0 / dt)          # crank_nicolson.pyx:378
        else:
            kind[m] = FIXED
    nb = len(boundaries)
    bk = np.zeros(nb, dtype=np.int32)
    bh = np.zeros(nb)
    for b, bnd in enumerate(boundaries):
        bk[b] = _module_kind(bnd[0])
        if bk[b] == 3:
            bh[b] = float(bnd[1])
    arrs = [np.ascontiguousarray(a, dtype=np.uint8) for a in
            (material_elements, boundary_z_elements, boundary_y_elements, boundary_x_elements)]
    h = ctypes.c_void_p()
    rc = lib().oracle_setup(int(nz), int(ny), int(nx), float(dz), float(dy), float(dx), *[_p(a) for a in arrs],
                            nmat, _p(kind), _p(ismat), _p(kk), _p(M), nb, _p(bk), _p(bh), ctypes.byref(h))
    if rc != 0:
        raise ValueError("oracle setup failed: %s" % ERRORS.get(rc, rc))
    return OracleParams(h, (int(nz), int(ny), int(nx)), dz * dy * dx), None


def source_field(shape, volume, t, dt, volumetric_elements, volumetric):
    """The volumetric source array of alternatingdirection_c_pyx.pyx:294-386 (W/m^3)."""
    q = np.zeros(shape, dtype="d")
    for idx, src in enumerate(volumetric):
        kind = src[0]
        if kind == IMPULSE_SOURCE:
            if t == src[1]:                                    # exact time match (:297)
                q[volumetric_elements == idx] = src[2] / dt
        elif kind == STEPPED_SOURCE:
            if src[1] <= t <= src[2]:                           # inclusive window (:303)
                q[volumetric_elements == idx] = src[3]
        elif kind == IMPULSE_POINT_SOURCE_JOULES:
            if t == src[1]:
                sel = volumetric_elements == idx
                if np.ndim(volume) > 0:     # per-cell volumes, curved-surface mode (:309-313)
                    q[sel] = src[2] / (volume[sel] * dt)
                else:
                    q[sel] = src[2] / (volume * dt)
        elif kind == SPATIALLY_Z_DECAYING_TEMPORAL_IMPULSE:
            (_, t_imp, direc, offset, zgrid, ddz, jpm2, length) = src
            if t == t_imp:
                sel = volumetric_elements == idx
                center = zgrid * direc[0] - float(offset)
                ddz = abs(float(ddz))
                left = center - ddz / 2.0
                right = center + ddz / 2.0
                use = sel & (right > 0.0)
                r = right[use]
                lft = left[use]
                lft[lft < 0.0] = 0.0
                zint = -np.exp(-r / float(length)) + np.exp(-lft / float(length))
                q[use] = zint * float(jpm2) / (ddz * dt)
    return q


def run_adi_steps(params, steps, t, dt, Tarray, volumetric_elements, volumetric):
    """alternatingdirection_c_pyx.pyx:287-416: returns a new array."""
    T = np.ascontiguousarray(Tarray, dtype="d")
    Q = source_field(params.shape, params.volume_array, t, dt, volumetric_elements, volumetric)
    out = np.empty_like(T)
    rc = lib().oracle_step(params.handle, _p(T), _p(Q), _p(out))
    if rc != 0:
        raise RuntimeError("oracle step failed")
    return out


def insulating_z_min_surface_temperature(T, dz):
    """heatsim2/surface_temperature.py:4-36: the z = 0 surface temperature from layers 0 and 1 of T[z, y, x],
    the mean of the zero-slope quadratic through the layer centres (a, c) and the linear extrapolation, with the
    reference's operations in its order."""
    T = np.asarray(T, dtype="d")
    a = (T[1] - T[0]) / (2.0 * dz ** 2.0)
    c = T[0] - 0.25 * a * dz ** 2.0
    d = T[1] - T[0]
    linear = T[0] - d / 2.0
    return (linear + c) / 2.0
