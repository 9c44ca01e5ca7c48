"""Mie series for a homogeneous sphere (physics anchor for the tests).

Written from the published Bohren & Huffman formulation (Absorption and
Scattering of Light by Small Particles, 1983, ch. 4): a_n, b_n from the
Riccati-Bessel functions, with the logarithmic derivative D_n(mx) computed by
downward recurrence.  Returns efficiencies Qext, Qsca (and Qabs = Qext - Qsca).
"""
import numpy as np


def mie_q(m: complex, x: float):
    nstop = int(x + 4.05 * x ** (1.0 / 3.0) + 2.0)
    y = m * x
    nmx = int(max(nstop, abs(y))) + 16
    D = np.zeros(nmx + 1, dtype=complex)
    for n in range(nmx, 0, -1):
        D[n - 1] = n / y - 1.0 / (D[n] + n / y)
    psi0, psi1 = np.cos(x), np.sin(x)
    chi0, chi1 = -np.sin(x), np.cos(x)
    xi1 = complex(psi1, -chi1)
    qext = qsca = 0.0
    for n in range(1, nstop + 1):
        psi = (2 * n - 1) * psi1 / x - psi0
        chi = (2 * n - 1) * chi1 / x - chi0
        xi = complex(psi, -chi)
        an = ((D[n] / m + n / x) * psi - psi1) / ((D[n] / m + n / x) * xi - xi1)
        bn = ((m * D[n] + n / x) * psi - psi1) / ((m * D[n] + n / x) * xi - xi1)
        qext += (2 * n + 1) * (an + bn).real
        qsca += (2 * n + 1) * (abs(an) ** 2 + abs(bn) ** 2)
        psi0, psi1 = psi1, psi
        chi0, chi1 = chi1, chi
        xi1 = complex(psi1, -chi1)
    return 2.0 / x ** 2 * qext, 2.0 / x ** 2 * qsca
