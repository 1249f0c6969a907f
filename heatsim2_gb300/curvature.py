"""Per-row face conductances of the reference's curved-surface mode (crank_nicolson.pyx:388-457).

The reference curves the grid under the top surface: with surface curvatures ky(j,i), kx(j,i) (positive
concave), the cell of layer k at (j,i) has edge lengths

    dy_top = (1 + k ky dz) dy,   dy_bot = (1 + (k+1) ky dz) dy,   dy_mean = (dy_top + dy_bot)/2    (x alike)
    volume = |dx_mean dy_mean dz|

and its heat balance multiplies each face flux by the face's area instead of dividing by the cell size:
the z faces by dx_top dy_top (low) and dx_bot dy_bot (high), the y faces by dx_mean dz, the x faces by
dy_mean dz, with the boundary class's flux evaluated at the cell's own mean edge lengths; the storage term is
rho c volume / dt and the source enters as volume * Q (pyx:397-451).  Divided by its volume, a row is the
flat heat balance with row-specific face conductances

    g = area * F(dz, dy_mean, dx_mean) / volume,

F the flux coefficient of the face's class (W/m^2/K per unit temperature difference).  The two rows of a
face see different values wherever the curvature or the depth differs, so these problems compile through
hs2g_create_rows.

F's dependence on the cell's edge lengths is read off the class symbolically: every entry of a class's flux
form is probed at stretch factors (1,1), (2,1) and (1,2) of (dy, dx), must be a monomial s_y^a s_x^b with
integer a and b (as for every built-in class: 1/d for conducting faces, constant for thin layers), and is
checked against direct evaluation at the problem's own extreme stretches; a class that fails raises
NotImplementedError.
"""
import numpy as np

from . import _native
from .crank_nicolson import evaluate_boundary

TEMPERATURE_FIXED = 1


def geometry(shape, spacing, ky, kx):
    """(dy_top, dy_bot, dy_mean, dx_top, dx_bot, dx_mean, volume), each (nz, ny, nx), as the reference computes
    them per cell (pyx:408-417)."""
    nz, ny, nx = shape
    dz, dy, dx = spacing
    k = np.arange(nz, dtype="d")[:, None, None]
    ky = np.broadcast_to(np.asarray(ky, dtype="d"), (ny, nx))[None]
    kx = np.broadcast_to(np.asarray(kx, dtype="d"), (ny, nx))[None]
    dy_top = (1.0 + k * ky * dz) * dy
    dy_bot = (1.0 + (k + 1) * ky * dz) * dy
    dx_top = (1.0 + k * kx * dz) * dx
    dx_bot = (1.0 + (k + 1) * kx * dz) * dx
    dy_mean = (dy_top + dy_bot) / 2.0
    dx_mean = (dx_top + dx_bot) / 2.0
    volume = np.abs(dx_mean * dy_mean * dz)
    return dy_top, dy_bot, dy_mean, dx_top, dx_bot, dx_mean, volume


def _flux_form(boundary, axis, dz, dy, dx):
    """Affine form (length FORM_LEN) of the face's flux coefficient F = -(coefficient of T_hi in q)."""
    G, _ = evaluate_boundary(boundary, axis, dz, dy, dx)
    return G * (dz, dy, dx)[axis]


def flux_model(boundary, axis, dz, dy, dx, sy_check, sx_check):
    """(F0, a, b): the flux form at the nominal spacing and, per entry, the integer exponents of its
    dependence on the y and x stretch factors.  Verified at the stretch pairs in sy_check / sx_check."""
    F0 = _flux_form(boundary, axis, dz, dy, dx)
    Fy = _flux_form(boundary, axis, dz, 2.0 * dy, dx)
    Fx = _flux_form(boundary, axis, dz, dy, 2.0 * dx)
    a = np.zeros(F0.shape)
    b = np.zeros(F0.shape)
    nz_ = F0 != 0
    bad = (~nz_) & ((Fy != 0) | (Fx != 0))
    with np.errstate(divide="ignore", invalid="ignore"):
        ra = np.where(nz_, Fy / np.where(nz_, F0, 1.0), 1.0)
        rb = np.where(nz_, Fx / np.where(nz_, F0, 1.0), 1.0)
    if bad.any() or (ra <= 0).any() or (rb <= 0).any():
        raise NotImplementedError("curved-surface mode: boundary class %r has a flux that is not a monomial in the "
                                  "cell's edge lengths" % (getattr(boundary[0], "__name__", boundary[0]),))
    a = np.round(np.log2(ra))
    b = np.round(np.log2(rb))
    if np.abs(np.log2(ra) - a).max() > 1e-9 or np.abs(np.log2(rb) - b).max() > 1e-9:
        raise NotImplementedError("curved-surface mode: boundary class %r has a flux that is not a monomial in the "
                                  "cell's edge lengths" % (getattr(boundary[0], "__name__", boundary[0]),))
    for sy, sx in zip(sy_check, sx_check):
        exact = _flux_form(boundary, axis, dz, sy * dy, sx * dx)
        model = F0 * np.power(sy, a) * np.power(sx, b)
        if np.abs(exact - model).max() > 1e-13 * max(np.abs(exact).max(), np.abs(F0).max(), 1e-300):
            raise NotImplementedError("curved-surface mode: boundary class %r has a flux that is not a monomial "
                                      "in the cell's edge lengths" % (getattr(boundary[0], "__name__",
                                                                              boundary[0]),))
    return F0, a, b


def _k_table(mats):
    nm = len(mats)
    kind = np.array([mats[m].kind for m in range(nm)], dtype=np.int32)
    kvec = np.array([[mats[m].k[e] for e in range(_native.K_ENTRIES)] for m in range(nm)], dtype="d")
    cap = np.array([mats[m].capacity for m in range(nm)], dtype="d")
    return kind, kvec, cap


def _apply_form(F, kvec, m_lo, m_hi):
    """F . [1, k_lo, k_hi] per row, with k_lo / k_hi the conductivity entries of materials m_lo / m_hi (index
    arrays); only the entries the form uses are gathered (the others may be NaN: the material lacks them)."""
    K = _native.K_ENTRIES
    out = np.full(m_lo.shape[0], F[0])
    for e in range(K):
        if F[1 + e] != 0.0:
            out = out + F[1 + e] * kvec[m_lo, e]
        if F[1 + K + e] != 0.0:
            out = out + F[1 + K + e] * kvec[m_hi, e]
    return out


def rows(cp, boundaries, ky, kx):
    """Per-row conductances of a validated ClassProblem ``cp`` in curved-surface mode.

    Returns (rows dict with zlo, zhi, ylo, yhi, xlo, xhi, capacity, fixed arrays, volume)."""
    nz, ny, nx = cp.shape
    dz, dy, dx = cp.spacing
    dy_top, dy_bot, dy_m, dx_top, dx_bot, dx_m, volume = geometry(cp.shape, cp.spacing, ky, kx)
    sy = dy_m / dy
    sx = dx_m / dx
    kind, kvec, cap = _k_table(cp.mats)
    mat = cp.mat
    comp_m = kind != TEMPERATURE_FIXED       # per material
    comp = comp_m[mat]                       # per voxel
    # stretch pairs where the monomial models are checked against direct evaluation
    checks_y = [float(sy.min()), float(sy.max()), float(sy.min()), float(sy.max()), 1.0]
    checks_x = [float(sx.min()), float(sx.max()), float(sx.max()), float(sx.min()), 1.0]
    models = {}

    def model(b, axis):
        key = (b, axis)
        if key not in models:
            models[key] = flux_model(boundaries[b], axis, dz, dy, dx, checks_y, checks_x)
        return models[key]

    out = {}
    arrays = ((cp.bz, 0), (cp.by, 1), (cp.bx, 2))
    area = {
        (0, 0): dx_top * dy_top, (0, 1): dx_bot * dy_bot,
        (1, 0): dx_m * dz, (1, 1): dx_m * dz,
        (2, 0): dy_m * dz, (2, 1): dy_m * dz,
    }
    for barr, axis in arrays:
        for side in (0, 1):              # 0: the row's low face, 1: its high face
            # the face's class and the two cells' conductivities with the neighbour fallback (pyx:298-338)
            sl_face = [slice(None)] * 3
            sl_face[axis] = slice(side, side + (nz, ny, nx)[axis])
            cls = barr[tuple(sl_face)]
            nb = np.roll(mat, 1 if side == 0 else -1, axis=axis)
            inside = np.ones(mat.shape, dtype=bool)
            edge = [slice(None)] * 3
            edge[axis] = 0 if side == 0 else -1
            inside[tuple(edge)] = False
            m_nb = np.where(inside & comp_m[nb], nb, mat)   # a fixed or outside neighbour lends the cell's own k
            m_lo = m_nb if side == 0 else mat
            m_hi = mat if side == 0 else m_nb
            g = np.zeros(mat.shape)
            for b in np.unique(cls[comp]):
                sel = comp & (cls == b)
                F0, a, bb = model(int(b), axis)
                lo_s, hi_s = m_lo[sel], m_hi[sel]
                # F(sy, sx) = F0 * sy^a * sx^b entry by entry: group the entries by exponent pair
                Fsel = np.zeros(lo_s.shape[0])
                for ea, eb in sorted(set(zip(a[F0 != 0].tolist(), bb[F0 != 0].tolist()))):
                    part = np.where((a == ea) & (bb == eb), F0, 0.0)
                    val = _apply_form(part, kvec, lo_s, hi_s)
                    Fsel = Fsel + val * np.power(sy[sel], ea) * np.power(sx[sel], eb)
                g[sel] = area[(axis, side)][sel] * Fsel / volume[sel]
            out["zyx"[axis] + ("lo" if side == 0 else "hi")] = np.ascontiguousarray(g)
    out["capacity"] = np.ascontiguousarray(np.where(comp, cap[mat], 1.0))
    out["fixed"] = np.ascontiguousarray((~comp).astype(np.uint8))
    return out, volume
