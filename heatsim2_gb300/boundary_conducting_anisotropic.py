"""Conducting face between materials with a 3x3 conductivity tensor K (z,y,x order), using the face mean
K_f = (K_lo + K_hi)/2 and q_a = -sum_b K_f[a,b] dT/db (reference heatsim2/boundary_conducting_anisotropic.py:7-67).

The tangential gradients are central differences averaged over the two cells that share the face.  Only the
normal term survives for tensors aligned with the grid axes, which is the case the three-stage ADI step
solves; a non-zero off-diagonal entry is rejected when the problem is compiled."""
from heatsim2_gb300.expression import group


def qz(kmatm55, kmatp55, dz, dy, dx, Tm55, Tp55, Tm45, Tp45, Tm65, Tp65, Tm54, Tp54, Tm56, Tp56, Tm46, Tp46,
       Tm64, Tp64):
    dTdz = group((Tp55 - Tm55) * (1.0 / dz))
    dTdy = group((Tp65 - Tp45) * (0.25 / dy)) + group((Tm65 - Tm45) * (0.25 / dy))
    dTdx = group((Tp56 - Tp54) * (0.25 / dx)) + group((Tm56 - Tm54) * (0.25 / dx))
    K = (kmatm55 + kmatp55) * 0.5
    return -K[0, 0] * dTdz - K[0, 1] * dTdy - K[0, 2] * dTdx


def qy(kmat5m5, kmat5p5, dz, dy, dx, T5m5, T5p5, T4m5, T4p5, T6m5, T6p5, T5m4, T5p4, T5m6, T5p6, T4m6, T4p6,
       T6m4, T6p4):
    dTdz = group((T6p5 - T4p5) * (0.25 / dz)) + group((T6m5 - T4m5) * (0.25 / dz))
    dTdy = group((T5p5 - T5m5) * (1.0 / dy))
    dTdx = group((T5p6 - T5p4) * (0.25 / dx)) + group((T5m6 - T5m4) * (0.25 / dx))
    K = (kmat5m5 + kmat5p5) * 0.5
    return -K[1, 0] * dTdz - K[1, 1] * dTdy - K[1, 2] * dTdx


def qx(kmat55m, kmat55p, dz, dy, dx, T55m, T55p, T45m, T45p, T65m, T65p, T54m, T54p, T56m, T56p, T46m, T46p,
       T64m, T64p):
    dTdz = group((T65p - T45p) * (0.25 / dz)) + group((T65m - T45m) * (0.25 / dz))
    dTdy = group((T56p - T54p) * (0.25 / dy)) + group((T56m - T54m) * (0.25 / dy))
    dTdx = group((T55p - T55m) * (1.0 / dx))
    K = (kmat55m + kmat55p) * 0.5
    return -K[2, 0] * dTdz - K[2, 1] * dTdy - K[2, 2] * dTdx
