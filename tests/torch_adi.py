"""A small FP64 PyTorch restatement of the ADI step, differentiable by autograd (test helper, CPU).

Per-voxel conductivity k, volumetric heat capacity C = rho*c and source amplitude q on a box insulating
outside, interior faces conducting with the arithmetic face mean (the reference's boundary_conducting.py:7-71):
G = (k_lo + k_hi) / (2 d^2); or, with face classes and fixed voxels (``faces_general``), the class problem's
faces and the reference's identity rows for fixed voxels.  The step is the Douglas delta form
    r0 = L T + s q,   (M - Lx/2) y0 = r0,   (M - Ly/2) y1 = M y0,   (M - Lz/2) y2 = M y1,   T' = T + y2
with M = C / dt, which is the reference's B/C/D step (alternatingdirection_c_pyx.pyx:287-416) rewritten in
increments; ``test_adjoint_cpu.py`` pins it to the oracle on a multi-material class problem.  The tridiagonal
solves are plain Thomas eliminations written with out-of-place tensor ops so autograd can run through them.
The loss is the sum over steps of the squared misfit of the top layer (k = 0) against observations.
"""
import torch


def faces(k, spacing):
    """Interior face conductances per axis: gz (nz-1, ny, nx), gy (nz, ny-1, nx), gx (nz, ny, nx-1)."""
    dz, dy, dx = spacing
    gz = 0.5 * (k[1:] + k[:-1]) / (dz * dz)
    gy = 0.5 * (k[:, 1:] + k[:, :-1]) / (dy * dy)
    gx = 0.5 * (k[:, :, 1:] + k[:, :, :-1]) / (dx * dx)
    return gz, gy, gx


def laplacian(T, gz, gy, gx):
    """L T: sum over faces of G (T_neighbour - T)."""
    out = torch.zeros_like(T)
    fz = gz * (T[1:] - T[:-1])
    fy = gy * (T[:, 1:] - T[:, :-1])
    fx = gx * (T[:, :, 1:] - T[:, :, :-1])
    out = out + torch.nn.functional.pad(fz, (0, 0, 0, 0, 0, 1)) - torch.nn.functional.pad(fz, (0, 0, 0, 0, 1, 0))
    out = out + torch.nn.functional.pad(fy, (0, 0, 0, 1)) - torch.nn.functional.pad(fy, (0, 0, 1, 0))
    out = out + torch.nn.functional.pad(fx, (0, 1)) - torch.nn.functional.pad(fx, (1, 0))
    return out


def faces_general(k, forms, low, fixed, spacing):
    """Interior face conductances per axis with face classes and fixed voxels, as the reference compiles a
    class problem: a face of class c on axis a conducts f0 + flo k_lo + fhi k_hi (forms[c, a] = (f0, flo, fhi)),
    the k of a fixed side replaced by its computed neighbour's (crank_nicolson.pyx:298-338); nothing between two
    fixed voxels.  low = (low_z, low_y, low_x): the class of each voxel's low face; fixed a bool tensor."""
    f = torch.as_tensor(forms, dtype=k.dtype)
    out = []
    for a in range(3):
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[a] = slice(None, -1)
        hi[a] = slice(1, None)
        lo, hi = tuple(lo), tuple(hi)
        flo, fhi = fixed[lo], fixed[hi]
        klo = torch.where(flo, k[hi], k[lo])
        khi = torch.where(fhi, k[lo], k[hi])
        cls = torch.as_tensor(low[a][hi], dtype=torch.long)
        c = f[cls, a]
        G = c[..., 0] + c[..., 1] * klo + c[..., 2] * khi
        out.append(torch.where(flo & fhi, torch.zeros_like(G), G))
    return tuple(out)


def solve_axis(M, g, rhs, axis, comp=None):
    """Solve (M - L_axis / 2) y = rhs along `axis`, g the interior face conductances of that axis.  comp (bool)
    marks computed voxels; the rows of the others are the identity (the reference's fixed voxels)."""
    Mt = M.movedim(axis, -1)
    b = rhs.movedim(axis, -1)
    gt = g.movedim(axis, -1)
    n = Mt.shape[-1]
    zero = torch.zeros_like(Mt[..., :1])
    glo = torch.cat([zero, gt], dim=-1)      # face below row r
    ghi = torch.cat([gt, zero], dim=-1)      # face above row r
    diag = Mt + 0.5 * (glo + ghi)
    sub = -0.5 * glo
    sup = -0.5 * ghi
    if comp is not None:
        ct = comp.movedim(axis, -1)
        diag = torch.where(ct, diag, torch.ones_like(diag))
        sub = torch.where(ct, sub, torch.zeros_like(sub))
        sup = torch.where(ct, sup, torch.zeros_like(sup))
    cp, dp = [], []
    for r in range(n):
        if r == 0:
            den = diag[..., 0]
            cp.append(sup[..., 0] / den)
            dp.append(b[..., 0] / den)
        else:
            den = diag[..., r] - sub[..., r] * cp[r - 1]
            cp.append(sup[..., r] / den)
            dp.append((b[..., r] - sub[..., r] * dp[r - 1]) / den)
    x = [None] * n
    x[n - 1] = dp[n - 1]
    for r in range(n - 2, -1, -1):
        x[r] = dp[r] - cp[r] * x[r + 1]
    return torch.stack(x, dim=-1).movedim(-1, axis)


def step(T, k, C, q, s, dt, spacing, faces_=None, comp=None):
    """One step; comp (bool, or None for all) marks computed voxels: the others keep their temperature, take
    no source and couple to their computed neighbours only through those neighbours' rows."""
    gz, gy, gx = faces(k, spacing) if faces_ is None else faces_
    M = C / dt
    r0 = laplacian(T, gz, gy, gx) + s * q
    if comp is not None:
        r0 = torch.where(comp, r0, torch.zeros_like(r0))
    y0 = solve_axis(M, gx, r0, 2, comp)
    y1 = solve_axis(M, gy, M * y0, 1, comp)
    y2 = solve_axis(M, gz, M * y1, 0, comp)
    return T + y2


def run(T0, k, C, q, schedule, dt, spacing, qfields=None, forms=None, low=None, fixed=None):
    """Temperatures after each step (list).  qfields (per-step source arrays) replaces s * q when given;
    forms / low / fixed give face classes and fixed voxels (faces_general), else every face conducts."""
    comp = None
    if forms is not None:
        fx = torch.zeros(k.shape, dtype=torch.bool) if fixed is None else torch.as_tensor(fixed, dtype=torch.bool)
        fc = faces_general(k, forms, low, fx, spacing)
        comp = ~fx
    else:
        fc = faces(k, spacing)
    T = T0
    out = []
    for n, s in enumerate(schedule):
        if qfields is not None:
            T = step(T, k, C, qfields[n], 1.0, dt, spacing, fc, comp)
        else:
            T = step(T, k, C, q, s, dt, spacing, fc, comp)
        out.append(T)
    return out


def misfit(T0, k, C, q, schedule, obs, dt, spacing, forms=None, low=None, fixed=None):
    """sum_n sum_{top layer} (T_{n+1} - obs[n])^2."""
    J = torch.zeros((), dtype=T0.dtype)
    for n, T in enumerate(run(T0, k, C, q, schedule, dt, spacing, forms=forms, low=low, fixed=fixed)):
        J = J + ((T[0] - obs[n]) ** 2).sum()
    return J
