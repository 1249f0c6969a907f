"""A numpy model of libhs2g's adjoint kernels (hs2g_adjoint.cu), operation for operation (test helper, CPU).

It repeats the forward step in the LU form the device uses (per-line factors lo/pivot, u, 1/pivot), the
checkpointed forward pass, the segment-by-segment recompute and the reverse sweep -- solves with the
transposed line operators (equal to the forward ones, A being symmetric) in the order z, y, x, then
lambda += L mu0, the face / capacity / source gradient accumulation and the chain to k and C -- so the
adjoint's derivation and its checkpoint bookkeeping can be checked against autograd through ``torch_adi`` on
machines without a GPU.  It is never used by the product.
"""
import numpy as np


def low_faces(k, spacing):
    """Per-voxel low-face conductances of each axis (zero on the exterior), as adj_setup_kernel."""
    dz, dy, dx = spacing
    gz = np.zeros_like(k)
    gy = np.zeros_like(k)
    gx = np.zeros_like(k)
    gz[1:] = 0.5 * (k[:-1] + k[1:]) * (1.0 / (dz * dz))
    gy[:, 1:] = 0.5 * (k[:, :-1] + k[:, 1:]) * (1.0 / (dy * dy))
    gx[:, :, 1:] = 0.5 * (k[:, :, :-1] + k[:, :, 1:]) * (1.0 / (dx * dx))
    return gz, gy, gx


FIXED_CAPACITY = 1e300   # kFixedCapacity of hs2g_adjoint.cu


def low_faces_general(k, forms, low, fixed):
    """Low-face conductances with face classes and fixed voxels, as adj_setup_faces_kernel: the class's form
    f0 + flo k_lo + fhi k_hi, a fixed side's k replaced by its neighbour's, 0 between two fixed voxels."""
    out = []
    for a in range(3):
        g = np.zeros_like(k)
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[a] = slice(None, -1)
        hi[a] = slice(1, None)
        lo, hi = tuple(lo), tuple(hi)
        flo, fhi = fixed[lo], fixed[hi]
        klo = np.where(flo, k[hi], k[lo])
        khi = np.where(fhi, k[lo], k[hi])
        c = forms[low[a][hi].astype(np.int64), a]
        G = c[..., 0] + c[..., 1] * klo + c[..., 2] * khi
        g[hi] = np.where(flo & fhi, 0.0, G)
        out.append(g)
    return tuple(out)


def factor(M, g, axis):
    """(e, u, ip) of M - L_axis/2 along `axis`, as adj_factor_kernel: e = lo / piv, u = super / piv, ip = 1/piv."""
    Mt = np.moveaxis(M, axis, -1)
    gt = np.moveaxis(g, axis, -1)
    n = Mt.shape[-1]
    e = np.zeros_like(Mt)
    u = np.zeros_like(Mt)
    ip = np.zeros_like(Mt)
    u_prev = np.zeros(Mt.shape[:-1])
    for r in range(n):
        gl = gt[..., r]
        gh = gt[..., r + 1] if r + 1 < n else np.zeros_like(gl)
        l = -(0.5 * gl)
        piv = Mt[..., r] + 0.5 * (gl + gh) - u_prev * l
        uu = -(0.5 * gh) / piv
        inv = 1.0 / piv
        e[..., r] = l * inv
        u[..., r] = uu
        ip[..., r] = inv
        u_prev = uu
    return tuple(np.moveaxis(a, -1, axis) for a in (e, u, ip))


def solve(f, b, axis, M=None):
    """A^-1 b along `axis` in the two one-FMA passes of the device's line solves:
    z_r = c_r - e_r z_{r-1} with c_r = b_r ip_r (ascending), y_r = z_r - u_r y_{r+1} (descending).
    With M: A^-1 (M b), c_r = b_r (M_r ip_r), M / piv formed once as adj_factor_kernel's mip.
    A is symmetric, so the adjoint's transposed solves are this solve too."""
    e, u, ip = (np.moveaxis(a, axis, -1) for a in f)
    if M is not None:
        ip = np.moveaxis(M, axis, -1) * ip
    bt = np.moveaxis(b, axis, -1)
    n = bt.shape[-1]
    y = np.zeros_like(bt)
    z = np.zeros(bt.shape[:-1])
    for r in range(n):
        z = bt[..., r] * ip[..., r] - e[..., r] * z
        y[..., r] = z
    x = np.zeros(bt.shape[:-1])
    for r in range(n - 1, -1, -1):
        x = y[..., r] - u[..., r] * x
        y[..., r] = x
    return np.moveaxis(y, -1, axis)


def lap(T, gz, gy, gx):
    """(L T)_p = sum over the six faces of G (T_neighbour - T_p), low-face arrays."""
    out = np.zeros_like(T)
    out[:, :, 1:] += gx[:, :, 1:] * (T[:, :, :-1] - T[:, :, 1:])
    out[:, :, :-1] += gx[:, :, 1:] * (T[:, :, 1:] - T[:, :, :-1])
    out[:, 1:] += gy[:, 1:] * (T[:, :-1] - T[:, 1:])
    out[:, :-1] += gy[:, 1:] * (T[:, 1:] - T[:, :-1])
    out[1:] += gz[1:] * (T[:-1] - T[1:])
    out[:-1] += gz[1:] * (T[1:] - T[:-1])
    return out


def residual(T, q, s, gz, gy, gx, D):
    """s q - D T + sum over faces of G T_nbr, the forward x stage's residual (residual_at in hs2g_adjoint.cu)."""
    r = s * q - D * T
    r[:, :, 1:] += gx[:, :, 1:] * T[:, :, :-1]
    r[:, :, :-1] += gx[:, :, 1:] * T[:, :, 1:]
    r[:, 1:] += gy[:, 1:] * T[:, :-1]
    r[:, :-1] += gy[:, 1:] * T[:, 1:]
    r[1:] += gz[1:] * T[:-1]
    r[:-1] += gz[1:] * T[1:]
    return r


def diagonal(gz, gy, gx):
    D = gz + gy + gx
    D[:, :, :-1] += gx[:, :, 1:]
    D[:, :-1] += gy[:, 1:]
    D[:-1] += gz[1:]
    return D


class Model(object):
    """forms / low / fixed: face classes and fixed voxels (hs2g_adjoint_set_faces), else every face conducts."""

    def __init__(self, k, C, q, dt, spacing, forms=None, low=None, fixed=None):
        self.k, self.C, self.q, self.dt, self.spacing = k, C, q, dt, spacing
        self.forms, self.low = forms, low
        self.fixed = np.zeros(k.shape, dtype=bool) if fixed is None else np.asarray(fixed, dtype=bool)
        self.g = low_faces(k, spacing) if forms is None else low_faces_general(k, forms, low, self.fixed)
        self.D = diagonal(*self.g)
        self.M = np.where(self.fixed, FIXED_CAPACITY, C * (1.0 / dt))
        gz, gy, gx = self.g
        self.f = [factor(self.M, gx, 2), factor(self.M, gy, 1), factor(self.M, gz, 0)]

    def fwd_step(self, T, s):
        gz, gy, gx = self.g
        y0 = solve(self.f[0], residual(T, self.q, s, gz, gy, gx, self.D), 2)
        y1 = solve(self.f[1], y0, 1, self.M)
        y2 = solve(self.f[2], y1, 0, self.M)
        return T + y2, y0, y1, y2

    def forward(self, T0, schedule, obs, ckpt):
        self.schedule, self.obs, self.ckpt = list(schedule), obs, min(ckpt, len(schedule))
        self.ckpts = []
        T = T0.copy()
        J = 0.0
        for s, sv in enumerate(self.schedule):
            if s % self.ckpt == 0:
                self.ckpts.append(T.copy())
            T = self.fwd_step(T, sv)[0]
            J += float(((T[0] - obs[s]) ** 2).sum())
        self.T_end = T
        return J

    def backward(self):
        gz, gy, gx = self.g
        N, Cp = len(self.schedule), self.ckpt
        gg = [np.zeros_like(self.k) for _ in range(3)]       # x, y, z low-face gradients
        gM = np.zeros_like(self.k)
        gq = np.zeros_like(self.k)
        lam = np.zeros_like(self.k)
        lam[0] = 2.0 * (self.T_end[0] - self.obs[N - 1])
        for sg in range((N + Cp - 1) // Cp - 1, -1, -1):
            s0, s1 = sg * Cp, min(N, sg * Cp + Cp)
            slots = []
            T = self.ckpts[sg]
            for s in range(s0, s1):
                Tn, y0, y1, y2 = self.fwd_step(T, self.schedule[s])
                slots.append((T, y0, y1, y2))
                T = Tn
            for s in range(s1 - 1, s0 - 1, -1):
                Tn, y0, y1, y2 = slots[s - s0]
                mu2 = solve(self.f[2], lam, 0)
                mu1 = solve(self.f[1], mu2, 1, self.M)
                mu0 = solve(self.f[0], mu1, 2, self.M)
                lam = lam + lap(mu0, gz, gy, gx)
                if s >= 1:
                    lam[0] += 2.0 * (Tn[0] - self.obs[s - 1])
                d0 = mu0[:, :, 1:] - mu0[:, :, :-1]
                gg[0][:, :, 1:] += -d0 * (Tn[:, :, 1:] - Tn[:, :, :-1]) - 0.5 * d0 * (y0[:, :, 1:] - y0[:, :, :-1])
                gg[1][:, 1:] += (-(mu0[:, 1:] - mu0[:, :-1]) * (Tn[:, 1:] - Tn[:, :-1])
                                 - 0.5 * (mu1[:, 1:] - mu1[:, :-1]) * (y1[:, 1:] - y1[:, :-1]))
                gg[2][1:] += (-(mu0[1:] - mu0[:-1]) * (Tn[1:] - Tn[:-1])
                              - 0.5 * (mu2[1:] - mu2[:-1]) * (y2[1:] - y2[:-1]))
                gM += mu2 * y1 + mu1 * y0 - mu0 * y0 - mu1 * y1 - mu2 * y2
                gq += self.schedule[s] * mu0
        dz, dy, dx = self.spacing
        gk = np.zeros_like(self.k)
        if self.forms is None:
            for a, (gf, d) in enumerate(zip(gg, (dx, dy, dz))):
                ax = 2 - a
                sl_hi = [slice(None)] * 3
                sl_lo = [slice(None)] * 3
                sl_hi[ax] = slice(1, None)
                sl_lo[ax] = slice(None, -1)
                face = gf[tuple(sl_hi)] * (0.5 / (d * d))
                gk[tuple(sl_hi)] += face
                gk[tuple(sl_lo)] += face
            return gk, gM / self.dt, gq, lam
        # adj_chain_faces_kernel: each face's gradient times dG/dk of its two sides (both coefficients to the
        # computed side when the other is fixed); fixed voxels' k, C and q get none
        fx = self.fixed
        for ax in range(3):
            gf = gg[2 - ax]                       # gg holds x, y, z
            lo = [slice(None)] * 3
            hi = [slice(None)] * 3
            lo[ax] = slice(None, -1)
            hi[ax] = slice(1, None)
            lo, hi = tuple(lo), tuple(hi)
            c = self.forms[self.low[ax][hi].astype(np.int64), ax]
            face = gf[hi]
            gk[hi] += face * np.where(fx[lo], c[..., 1] + c[..., 2], c[..., 2])
            gk[lo] += face * np.where(fx[hi], c[..., 1] + c[..., 2], c[..., 1])
        gk[fx] = 0.0
        gC = np.where(fx, 0.0, gM / self.dt)
        gq = np.where(fx, 0.0, gq)
        return gk, gC, gq, lam
