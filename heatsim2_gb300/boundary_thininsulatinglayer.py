"""Thin insulating layer on a face: a contact conductance h (W/m^2/K) in series with nothing else,
q = -h * (T_hi - T_lo), independent of the materials' k (reference heatsim2/boundary_thininsulatinglayer.py:9-59).

Use as ``(boundary_thininsulatinglayer, h)``: the extra tuple entry is passed as ``conductioncoefficient``."""
from heatsim2_gb300.expression import group


def qz(kmatm55, kmatp55, dz, dy, dx, Tm55, Tp55, Tm45, Tp45, Tm65, Tp65, Tm54, Tp54, Tm56, Tp56, Tm46, Tp46,
       Tm64, Tp64, conductioncoefficient):
    return -conductioncoefficient * group(Tp55 - Tm55)


def qy(kmat5m5, kmat5p5, dz, dy, dx, T5m5, T5p5, T4m5, T4p5, T6m5, T6p5, T5m4, T5p4, T5m6, T5p6, T4m6, T4p6,
       T6m4, T6p4, conductioncoefficient):
    return -conductioncoefficient * group(T5p5 - T5m5)


def qx(kmat55m, kmat55p, dz, dy, dx, T55m, T55p, T45m, T45p, T65m, T65p, T54m, T54p, T56m, T56p, T46m, T46p,
       T64m, T64p, conductioncoefficient):
    return -conductioncoefficient * group(T55p - T55m)
