"""Conducting face between isotropic materials (scalar k): Fourier's law with the arithmetic mean of the two
conductivities, q = -(k_lo + k_hi)/2 * (T_hi - T_lo)/d (reference heatsim2/boundary_conducting.py:7-71).

The temperature difference is wrapped in ``group`` so the ADI stage split averages it in time as one unit."""
from heatsim2_gb300.expression import group


def qz(kmatm55, kmatp55, dz, dy, dx, Tm55, Tp55, Tm45, Tp45, Tm65, Tp65, Tm54, Tp54, Tm56, Tp56, Tm46, Tp46,
       Tm64, Tp64):
    k_face = (kmatm55 + kmatp55) * 0.5
    return -k_face * group((Tp55 - Tm55) * (1.0 / dz))


def qy(kmat5m5, kmat5p5, dz, dy, dx, T5m5, T5p5, T4m5, T4p5, T6m5, T6p5, T5m4, T5p4, T5m6, T5p6, T4m6, T4p6,
       T6m4, T6p4):
    k_face = (kmat5m5 + kmat5p5) * 0.5
    return -k_face * group((T5p5 - T5m5) * (1.0 / dy))


def qx(kmat55m, kmat55p, dz, dy, dx, T55m, T55p, T45m, T45p, T65m, T65p, T54m, T54p, T56m, T56p, T46m, T46p,
       T64m, T64p):
    k_face = (kmat55m + kmat55p) * 0.5
    return -k_face * group((T55p - T55m) * (1.0 / dx))
