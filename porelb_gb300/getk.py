"""Analytic permeability of a body-centred-cubic sphere array (getK.c).

getK.c (getK.c:39-95) estimates the permeability of a BCC array of spheres
of radius a = sqrt(3) L chi / 4 (chi in (0, 1]; chi = 1 when neighbours
touch) with L = nx - 1:

* K1 (getK.c:67-70): Stokes drag of the array, K = 2/9 a^2 / (d* (1 - eps)),
  with d*(chi) = sum_i q_i chi^i the drag-coefficient series of Sangani &
  Acrivos (1982) for BCC arrays (31 coefficients, getK.c:5-36).
* K2 (getK.c:61-64,72): Kozeny-Carman, eps^3 / (C S^2), C = 5,
  S = 2 * 4 pi a^2 / L^3.
eps = 1 - 8/3 pi a^3 / L^3 is the porosity of two spheres per cell.
The TABLE build (getK.c:74-92) multiplies K1 by eps.

These are the reference's validation numbers for the half-way bounce-back
mode: they are not computed from simulation output.
"""
import math

# drag-coefficient series for BCC arrays, the table of getK.c:5-36
QS_BCC = [
    0.1000000e+01, 0.1575834e+01, 0.2483254e+01, 0.3233022e+01,
    0.4022864e+01, 0.4650320e+01, 0.5281412e+01, 0.5826374e+01,
    0.6258376e+01, 0.6544504e+01, 0.6878396e+01, 0.7190839e+01,
    0.7268068e+01, 0.7304025e+01, 0.7301217e+01, 0.7236410e+01,
    0.7298014e+01, 0.7369849e+01, 0.7109497e+01, 0.6228418e+01,
    0.5235796e+01, 0.4476874e+01, 0.3541982e+01, 0.2939353e+01,
    0.3935484e+01, 0.5179097e+01, 0.3959872e+01, 0.2227627e+01,
    0.3393390e+01, 0.4491369e+01, 0.2200686e+01,
]


def bcc_k(chi, L, table_variant=False):
    """(K1, K2, a, eps) for packing fraction parameter chi and cell size L."""
    a = math.sqrt(3.0) * L * chi / 4.0
    eps = 1.0 - 8.0 / 3 * math.pi * a * a * a / L / L / L
    C = 5
    S = 2 * 4 * math.pi * a * a / L / L / L
    d_star = 0.0
    for i in range(31):
        d_star += QS_BCC[i] * math.pow(chi, i)
    K1 = 2.0 / 9 * a * a / d_star / (1 - eps)
    if table_variant:
        K1 *= eps
    K2 = eps * eps * eps / C / S / S
    return K1, K2, a, eps


def getk(chi, nx):
    """getK.c's command-line result for `getK Chi nx` (L = nx - 1)."""
    return bcc_k(chi, float(nx - 1))


def bcc_flag(n, chi):
    """Periodic BCC array on an n^3 grid (cell size n): spheres of radius
    sqrt(3) n chi / 4 centred at (0,0,0) and (n/2,n/2,n/2); 1 fluid, 0 solid."""
    import numpy as np
    a = math.sqrt(3.0) * n * chi / 4.0
    x = np.arange(n, dtype=np.float64)
    flag = np.ones((n, n, n), np.uint8)
    for c in (0.0, n / 2.0):
        d = np.abs(x - c)
        d = np.minimum(d, n - d)
        d2 = d[:, None, None] ** 2 + d[None, :, None] ** 2 + d[None, None, :] ** 2
        flag[d2 <= a * a] = 0
    return flag.reshape(-1)
