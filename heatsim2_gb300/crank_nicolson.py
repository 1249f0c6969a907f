"""``setup``: compile a heatsim2 problem (grid, material / boundary / source classes, class arrays) onto the GPU.

Mirrors ``heatsim2.crank_nicolson.setup`` (reference crank_nicolson.pyx:128-498): same arguments, same return
shape ``(ADI_params, ADI_steps)``, same errors where the reference raises.  The reference evaluates a symbolic
heat balance for every voxel in Python and scatters it into sparse matrices; here each boundary class is
evaluated symbolically once per axis into an affine form of the face conductance in the two adjacent
materials' conductivity entries (``compile_boundary_forms``), and the device compiler evaluates those forms
for every face and factorises the per-line tridiagonal systems (libhs2g ``hs2g_create_classes``).
"""
import math
import numbers

import numpy as np

from . import _native
from .expression import linear_expression, ExpressionError

TEMPERATURE_COMPUTE = 0
TEMPERATURE_FIXED = 1

# placeholder names per axis (z, y, x): low / high cell temperatures first, then the tangential neighbours
_T_NAMES = (
    ("Tm55", "Tp55", "Tm45", "Tp45", "Tm65", "Tp65", "Tm54", "Tp54", "Tm56", "Tp56", "Tm46", "Tp46", "Tm64", "Tp64"),
    ("T5m5", "T5p5", "T4m5", "T4p5", "T6m5", "T6p5", "T5m4", "T5p4", "T5m6", "T5p6", "T4m6", "T4p6", "T6m4", "T6p4"),
    ("T55m", "T55p", "T45m", "T45p", "T65m", "T65p", "T54m", "T54p", "T56m", "T56p", "T46m", "T46p", "T64m", "T64p"),
)
_Q_NAMES = ("qz", "qy", "qx")
_K_LO, _K_HI = "kmat_lo", "kmat_hi"


class UnalignedAnisotropyError(AssertionError, NotImplementedError):
    """Raised where the reference asserts: a face flux couples temperatures across axes, which the three-stage
    ADI step cannot solve (alternatingdirection_c_pyx.pyx:570), or ``unaligned_anisotropic=True`` was asked
    for, whose stage-count assertion fails in the reference for every problem (pyx:452)."""


def _form_from_coeffs(coeffs):
    """[(k_name, k_index, coef)] -> affine form vector of length FORM_LEN (see include/hs2g.h)."""
    f = np.zeros(_native.FORM_LEN)
    for kname, kidx, c in coeffs:
        if kname is None:
            f[0] += c
            continue
        base = 1 if kname == _K_LO else 1 + _native.K_ENTRIES
        entry = 0 if kidx is None else 1 + 3 * kidx[0] + kidx[1]
        f[base + entry] += c
    return f


def evaluate_boundary(boundary, axis, dz, dy, dx):
    """Evaluate one boundary class tuple ``(module, *extra)`` on ``axis`` (0=z, 1=y, 2=x).

    Returns (G_form, [(error_code, zero_form), ...]) where G_form is the affine form of the face conductance
    G = -(coefficient of T_hi in q) / d (W/m^3/K) and each zero form must vanish on every face that uses the
    class (otherwise the device compiler raises that error code)."""
    module, extra = boundary[0], tuple(boundary[1:])
    names = _T_NAMES[axis]
    args = [linear_expression(_K_LO), linear_expression(_K_HI), dz, dy, dx] + [linear_expression(n) for n in names]
    try:
        q = getattr(module, _Q_NAMES[axis])(*args, *extra)
    except ExpressionError as e:
        raise ValueError("boundary class %r, %s: %s" % (getattr(module, "__name__", module), _Q_NAMES[axis], e))
    if isinstance(q, numbers.Number):
        q = linear_expression(q)
    if not isinstance(q, linear_expression):
        raise ValueError("boundary class %r returned %r" % (getattr(module, "__name__", module), type(q)))
    lo, hi = names[0], names[1]
    zeros = []
    const = q.constant_terms()
    if const:
        zeros.append((_native.ERR_FORM, _form_from_coeffs(const)))
    terms = q.temperature_terms()
    members = {}
    for (t, g) in terms:
        members.setdefault(g, set()).add(t)
    c_lo = np.zeros(_native.FORM_LEN)
    c_hi = np.zeros(_native.FORM_LEN)
    for (t, g), coeffs in terms.items():
        f = _form_from_coeffs(coeffs)
        if t not in (lo, hi):
            zeros.append((_native.ERR_UNALIGNED, f))
        elif g is None:
            zeros.append((_native.ERR_FORM, f))          # outside any group: explicit-only term
        elif members[g] - {lo, hi}:
            zeros.append((_native.ERR_UNALIGNED, f))     # grouped together with cross-axis terms
        elif t == lo:
            c_lo += f
        else:
            c_hi += f
    if np.any(c_lo + c_hi):
        zeros.append((_native.ERR_FORM, c_lo + c_hi))    # not a two-point difference T_hi - T_lo
    inv_d = 1.0 / (dz, dy, dx)[axis]                     # heat balance divides the flux by the cell size
    G = -c_hi * inv_d
    out = []
    seen = set()
    for code, f in zeros:
        if not np.any(f):
            continue
        key = (code, tuple(f * inv_d))
        if key in seen:
            continue
        seen.add(key)
        out.append((code, f * inv_d))
    return G, out


def compile_boundary_forms(boundaries, dz, dy, dx):
    """ctypes array of FaceForm [nbnd][3]."""
    nb = len(boundaries)
    forms = (_native.FaceForm * (3 * nb))()
    for b, bnd in enumerate(boundaries):
        for axis in range(3):
            G, zeros = evaluate_boundary(bnd, axis, dz, dy, dx)
            if len(zeros) > _native.MAX_ZERO_FORMS:
                raise NotImplementedError("boundary class %d has more than %d independent cross terms"
                                          % (b, _native.MAX_ZERO_FORMS))
            ff = forms[3 * b + axis]
            for e in range(_native.FORM_LEN):
                ff.normal[e] = G[e]
            ff.nzero = len(zeros)
            for z, (code, f) in enumerate(zeros):
                ff.zero_code[z] = code
                for e in range(_native.FORM_LEN):
                    ff.zero[z][e] = f[e]
    return forms


def compile_materials(materials, dt):
    """ctypes array of Material: kind, conductivity entries (NaN where absent), capacity rho*c*(1/dt)."""
    nm = len(materials)
    out = (_native.Material * nm)()
    nan = float("nan")
    for m, mat in enumerate(materials):
        if mat[0] == TEMPERATURE_COMPUTE:
            (_, k, rho, c) = mat
            out[m].kind = TEMPERATURE_COMPUTE
            kk = [nan] * _native.K_ENTRIES
            if isinstance(k, np.ndarray) and k.size == 9:
                kk[1:] = [float(v) for v in np.asarray(k, dtype="d").reshape(9)]
            elif isinstance(k, np.ndarray) and k.size == 1:
                kk[0] = float(k.reshape(()))
            elif isinstance(k, numbers.Number):
                kk[0] = float(k)
            else:
                raise ValueError("material %d: k must be a scalar or a 3x3 array" % m)
            for e in range(_native.K_ENTRIES):
                out[m].k[e] = kk[e]
            out[m].capacity = rho * c * (1.0 / dt)        # crank_nicolson.pyx:378
        elif mat[0] == TEMPERATURE_FIXED:
            out[m].kind = TEMPERATURE_FIXED
            for e in range(_native.K_ENTRIES):
                out[m].k[e] = nan
            out[m].capacity = 1.0
        else:
            raise AssertionError("material %d: first entry must be TEMPERATURE_COMPUTE or TEMPERATURE_FIXED" % m)
    return out


def _u8_array(a, name, shape):
    if not isinstance(a, np.ndarray):
        raise ValueError("%s must be a numpy uint8 array" % name)
    if a.dtype != np.uint8:
        raise ValueError("Buffer dtype mismatch, expected 'uint8_t' but got '%s' (%s)" % (a.dtype, name))
    if a.ndim != 3:
        raise ValueError("Buffer has wrong number of dimensions (expected 3, got %d) (%s)" % (a.ndim, name))
    if tuple(a.shape) != tuple(shape):
        raise ValueError("%s has shape %s, expected %s" % (name, a.shape, tuple(shape)))
    return np.ascontiguousarray(a)


def current_device():
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.current_device()
    except ImportError:
        pass
    return 0


class _Handle(object):
    """Owns one hs2g handle; destroys it when garbage-collected."""

    def __init__(self, ptr, device):
        self.ptr = ptr
        self.device = device

    def __del__(self):
        if self.ptr and _native._lib is not None:
            _native._lib.hs2g_destroy(self.ptr)
            self.ptr = None


class ClassProblem(object):
    """A validated problem packed for the C ABI (hs2g_class_problem); keeps its arrays alive."""

    def __init__(self, z0, y0, x0, dz, dy, dx, nz, ny, nx, dt, materials, boundaries, volumetric,
                 material_elements, boundary_z_elements, boundary_y_elements, boundary_x_elements,
                 volumetric_elements, top_surface_y_curvatures=None, top_surface_x_curvatures=None,
                 unaligned_anisotropic=False):
        self.curvature = None
        if top_surface_y_curvatures is not None or top_surface_x_curvatures is not None:
            # curved-surface mode (pyx:388-457): per-cell curvatures along y and x, zero where not given
            curv = []
            for c in (top_surface_y_curvatures, top_surface_x_curvatures):
                c = np.zeros((int(ny), int(nx))) if c is None else np.asarray(c, dtype="d")
                if c.shape != (int(ny), int(nx)):
                    raise ValueError("surface curvatures must have shape (ny, nx) = %s" % ((int(ny), int(nx)),))
                if not np.isfinite(c).all():
                    raise ValueError("surface curvatures must be finite")
                curv.append(np.ascontiguousarray(c))
            self.curvature = tuple(curv)
        nz, ny, nx = int(nz), int(ny), int(nx)
        if nz < 1 or ny < 1 or nx < 1:
            raise ValueError("grid dimensions must be positive")
        if not (dt > 0 and math.isfinite(dt)):
            raise ValueError("dt must be positive")
        if len(materials) > _native.MAX_CLASSES or len(boundaries) > _native.MAX_CLASSES:
            raise ValueError("at most 256 material and boundary classes (uint8 class arrays)")
        self.shape = (nz, ny, nx)
        self.spacing = (dz, dy, dx)
        self.origin = (z0, y0, x0)
        self.dt = dt
        self.volumetric = volumetric
        self.mat = _u8_array(material_elements, "material_elements", (nz, ny, nx))
        self.bz = _u8_array(boundary_z_elements, "boundary_z_elements", (nz + 1, ny, nx))
        self.by = _u8_array(boundary_y_elements, "boundary_y_elements", (nz, ny + 1, nx))
        self.bx = _u8_array(boundary_x_elements, "boundary_x_elements", (nz, ny, nx + 1))
        self.vol = _u8_array(volumetric_elements, "volumetric_elements", (nz, ny, nx))
        self.mats = compile_materials(materials, dt)
        self.forms = compile_boundary_forms(boundaries, dz, dy, dx)
        self.boundaries = boundaries
        if unaligned_anisotropic:
            # The reference's unaligned-anisotropic mode splits every voxel's heat balance into 15 stages
            # (alternatingdirection_c_pyx.pyx:511-564) but its adi_setup builds three stage matrices
            # (pyx:418-445), so the stage-count assertion of add_equation_to_adi_matrices (pyx:452) fails at
            # the first voxel of every problem, after the classes have been evaluated.  Same error here.
            raise UnalignedAnisotropyError(
                "unaligned_anisotropic=True: the reference's setup fails its stage-count assertion "
                "(alternatingdirection_c_pyx.pyx:452: 15 stage expressions for 3 stage matrices) for every "
                "problem, so this mode has no results to reproduce; anisotropy aligned with the grid axes runs "
                "with unaligned_anisotropic=False")
        self.struct = _native.ClassProblem(nz, ny, nx, len(materials), len(boundaries), self.mats, self.forms,
                                           self.mat.ctypes.data, self.bz.ctypes.data, self.by.ctypes.data,
                                           self.bx.ctypes.data, self.vol.ctypes.data)


def raise_compile_error(rc):
    """Map an hs2g compile error code to the exception the reference raises in that situation."""
    L = _native.load()
    if rc == _native.ERR_UNALIGNED:
        raise UnalignedAnisotropyError(L.hs2g_last_error().decode())
    if rc in (_native.ERR_EXTERIOR, _native.ERR_KTYPE, _native.ERR_FORM, _native.ERR_CAPACITY, _native.ERR_ARG):
        raise ValueError(L.hs2g_last_error().decode())
    _native.check(rc)


def setup(z0, y0, x0, dz, dy, dx, nz, ny, nx, dt, materials, boundaries, volumetric, material_elements,
          boundary_z_elements, boundary_y_elements, boundary_x_elements, volumetric_elements,
          top_surface_y_curvatures=None, top_surface_x_curvatures=None, unaligned_anisotropic=False):
    """Compile the problem; returns ``(ADI_params, ADI_steps)`` for ``run_adi_steps``.

    Arguments as in the reference (crank_nicolson.pyx:128-142).  With surface curvatures the problem compiles
    in the reference's curved-surface mode (heatsim2_gb300.curvature; ``ADI_params.volume_array`` is then the
    per-cell volume).  ``unaligned_anisotropic=True`` raises AssertionError after the classes are validated, as
    the reference's setup does for every problem (alternatingdirection_c_pyx.pyx:452)."""
    from .alternatingdirection import adi_params, adi_step
    cp = ClassProblem(z0, y0, x0, dz, dy, dx, nz, ny, nx, dt, materials, boundaries, volumetric, material_elements,
                      boundary_z_elements, boundary_y_elements, boundary_x_elements, volumetric_elements,
                      top_surface_y_curvatures, top_surface_x_curvatures, unaligned_anisotropic)
    nz, ny, nx = cp.shape
    L = _native.load()
    device = current_device()
    import ctypes
    h = ctypes.c_void_p()
    rc = L.hs2g_create_classes(ctypes.byref(cp.struct), device, ctypes.byref(h))
    if rc != _native.OK:
        raise_compile_error(rc)
    handle = _Handle(h, device)
    volume = dz * dy * dx
    if cp.curvature is not None:
        # the class compile above validated the problem exactly as the flat mode does; the curved problem's
        # rows weigh every face by its cell's own geometry and compile from per-row conductances
        from . import curvature
        r, volume = curvature.rows(cp, boundaries, *cp.curvature)
        rp = _native.RowsProblem(nz, ny, nx, *[r[n].ctypes.data for n in ("zlo", "zhi", "ylo", "yhi", "xlo", "xhi",
                                                                         "capacity", "fixed")],
                                 cp.vol.ctypes.data)
        h2 = ctypes.c_void_p()
        rc = L.hs2g_create_rows(ctypes.byref(rp), device, ctypes.byref(h2))
        if rc != _native.OK:
            raise_compile_error(rc)
        handle = _Handle(h2, device)
    vol = cp.vol
    params = adi_params(shape=(nz, ny, nx), volume_array=volume, dt=dt, handle=handle, device=device,
                        spacing=(dz, dy, dx), origin=(z0, y0, x0), compiled_volumetric=vol.copy())
    steps = tuple(adi_step(params, perm, s) for s, perm in enumerate(((0, 1, 2), (2, 0, 1), (1, 2, 0))))
    return params, steps
