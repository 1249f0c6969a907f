"""A numpy model of the CUDA step's arithmetic (test helper, CPU only).

It repeats, operation for operation, what libhs2g's device compiler and sweep kernels compute -- face
conductances from the compiled boundary forms (hs2g_compile.cu faces_kernel), the per-line factorisations and
scaled delta-form coefficients (factor_{z,y,x}_kernel) and the three sweeps (hs2g_sweep.cu) -- so the
formulation can be checked against the oracle on machines without a GPU.  It is never used by the product.
"""
import numpy as np

from heatsim2_gb300 import _native
from heatsim2_gb300.crank_nicolson import compile_boundary_forms, compile_materials


def faces_from_classes(shape, materials, boundaries, dz, dy, dx, dt, mat, bz, by, bx):
    nz, ny, nx = shape
    mats = compile_materials(materials, dt)
    forms = compile_boundary_forms(boundaries, dz, dy, dx)
    kind = np.array([m.kind for m in mats])
    kvec = np.array([list(m.k) for m in mats])
    cap = np.array([m.capacity for m in mats])
    comp = kind[mat] == 0
    M = np.where(comp, cap[mat], 1.0)
    out = []
    for axis, barr in enumerate((bz, by, bx)):
        G = np.zeros(barr.shape)
        fz, fy, fx = barr.shape
        for f_k in range(fz):
            for f_j in range(fy):
                for f_i in range(fx):
                    c = (f_k, f_j, f_i)[axis]
                    n_axis = shape[axis]
                    lo_in, hi_in = c > 0, c < n_axis
                    lo = list((f_k, f_j, f_i))
                    lo[axis] -= 1
                    mlo = mat[tuple(lo)] if lo_in else -1
                    mhi = mat[f_k, f_j, f_i] if hi_in else -1
                    lo_c = lo_in and kind[mlo] == 0
                    hi_c = hi_in and kind[mhi] == 0
                    if not (lo_c or hi_c):
                        continue
                    klo = kvec[mlo] if lo_c else kvec[mhi]
                    khi = kvec[mhi] if hi_c else kvec[mlo]
                    f = np.array(forms[3 * barr[f_k, f_j, f_i] + axis].normal)
                    g = f[0]
                    for e in range(_native.K_ENTRIES):
                        if f[1 + e] != 0.0:
                            g += f[1 + e] * klo[e]
                        if f[1 + _native.K_ENTRIES + e] != 0.0:
                            g += f[1 + _native.K_ENTRIES + e] * khi[e]
                    G[f_k, f_j, f_i] = g
        out.append(G)
    return out[0], out[1], out[2], M, comp


def factor(Gz, Gy, Gx, M, comp):
    """Coefficients from shared face conductances (class and dense problems)."""
    return factor_rows(Gz[:-1], Gz[1:], Gy[:, :-1], Gy[:, 1:], Gx[:, :, :-1], Gx[:, :, 1:], M, comp)


def factor_rows(gzl, gzh, gyl, gyh, gxl, gxh, M, comp):
    """Coefficients from per-row face conductances (hs2g_compile.cu factor kernels with RowFaces)."""
    nz, ny, nx = M.shape
    c = {}

    def row(gl, gh):
        d = np.where(comp, M + 0.5 * (gl + gh), 1.0)
        lo = np.where(comp, -(0.5 * gl), 0.0)
        hi = np.where(comp, -(0.5 * gh), 0.0)
        return d, lo, hi

    z = lambda a: np.where(comp, a, 0.0)
    gzl, gzh, gyl, gyh, gxl, gxh = (z(a) for a in (gzl, gzh, gyl, gyh, gxl, gxh))
    # z lines
    d, lo, hi = row(gzl, gzh)
    a2 = np.zeros_like(M); b2 = np.zeros_like(M); s2 = np.zeros_like(M)
    u_prev = np.zeros((ny, nx))
    for k in range(nz):
        piv = d[k] - u_prev * lo[k]
        u = hi[k] / piv
        a2[k] = lo[k] / piv; b2[k] = u; s2[k] = M[k] / piv
        u_prev = u
    # y lines
    d, lo, hi = row(gyl, gyh)
    a1 = np.zeros_like(M); b1 = np.zeros_like(M); sg = np.zeros_like(M)
    u_prev = np.zeros((nz, nx)); s2_prev = np.ones((nz, nx))
    for j in range(ny):
        piv = d[:, j] - u_prev * lo[:, j]
        u = hi[:, j] / piv
        sg[:, j] = s2[:, j] * M[:, j] / piv
        a1[:, j] = s2[:, j] * lo[:, j] / (piv * s2_prev) if j > 0 else 0.0
        b1[:, j] = s2[:, j] * u / s2[:, j + 1] if j + 1 < ny else 0.0
        u_prev = u; s2_prev = s2[:, j]
    # x lines
    d, lo, hi = row(gxl, gxh)
    names = ("wc", "wxl", "wxh", "wyl", "wyh", "wzl", "wzh", "wq", "a0", "b0")
    for nme in names:
        c[nme] = np.zeros_like(M)
    u_prev = np.zeros((nz, ny)); sg_prev = np.ones((nz, ny))
    for i in range(nx):
        piv = d[:, :, i] - u_prev * lo[:, :, i]
        u = hi[:, :, i] / piv
        f0 = sg[:, :, i] / piv
        center = -(((gxl[:, :, i] + gxh[:, :, i]) + (gyl[:, :, i] + gyh[:, :, i])) + (gzl[:, :, i] + gzh[:, :, i]))
        c["wc"][:, :, i] = f0 * center
        for nme, g in (("wxl", gxl), ("wxh", gxh), ("wyl", gyl), ("wyh", gyh), ("wzl", gzl), ("wzh", gzh)):
            c[nme][:, :, i] = f0 * g[:, :, i]
        c["wq"][:, :, i] = np.where(comp[:, :, i], f0, 0.0)
        c["a0"][:, :, i] = sg[:, :, i] * lo[:, :, i] / (piv * sg_prev) if i > 0 else 0.0
        c["b0"][:, :, i] = sg[:, :, i] * u / sg[:, :, i + 1] if i + 1 < nx else 0.0
        u_prev = u; sg_prev = sg[:, :, i]
    c.update(a1=a1, b1=b1, a2=a2, b2=b2)
    return c


def step(c, T, Q):
    nz, ny, nx = T.shape
    pad = np.pad(T, 1, mode="edge")
    r = c["wc"] * T
    r = r + c["wxl"] * pad[1:-1, 1:-1, :-2] + c["wxh"] * pad[1:-1, 1:-1, 2:]
    r = r + c["wyl"] * pad[1:-1, :-2, 1:-1] + c["wyh"] * pad[1:-1, 2:, 1:-1]
    r = r + c["wzl"] * pad[:-2, 1:-1, 1:-1] + c["wzh"] * pad[2:, 1:-1, 1:-1]
    r = r + c["wq"] * Q
    W0 = np.zeros_like(T)
    z = np.zeros((nz, ny))
    for i in range(nx):
        z = r[:, :, i] - c["a0"][:, :, i] * z
        W0[:, :, i] = z
    x = np.zeros((nz, ny))
    for i in range(nx - 1, -1, -1):
        x = W0[:, :, i] - c["b0"][:, :, i] * x
        W0[:, :, i] = x
    W1 = np.zeros_like(T)
    z = np.zeros((nz, nx))
    for j in range(ny):
        z = W0[:, j] - c["a1"][:, j] * z
        W1[:, j] = z
    x = np.zeros((nz, nx))
    for j in range(ny - 1, -1, -1):
        x = W1[:, j] - c["b1"][:, j] * x
        W1[:, j] = x
    Z = np.zeros_like(T)
    z = np.zeros((ny, nx))
    for k in range(nz):
        z = W1[k] - c["a2"][k] * z
        Z[k] = z
    out = np.empty_like(T)
    x = np.zeros((ny, nx))
    for k in range(nz - 1, -1, -1):
        x = Z[k] - c["b2"][k] * x
        out[k] = T[k] + x
    return out
