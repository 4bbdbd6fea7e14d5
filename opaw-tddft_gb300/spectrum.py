"""Absorption spectrum of a delta-kick run (post-processing of d_dip(t)).

The reference writes the dipole signal d_dip(t) = (dip'(t) - dip(t)) / gamma
of a kick psi' = exp(-i gamma r_ipol) psi (tddft_excite.f90:1-16,
tddft_plot.f90:40-57) and leaves the spectrum to the user.  Here the dipole
strength function

    S(w) = -(2 w / pi) Im  int_0^T d_dip(t) exp(i w t) D(t) dt

with a damping window D (exponential exp(-t/tau) or Gaussian exp(-t^2/2 tau^2))
is evaluated by direct quadrature on a frequency grid (atomic units).  With
the reference's sign conventions (density dipole, kick exp(-i gamma x)) a
resonance at w0 gives a positive peak and S integrates to the electron count
(Thomas-Reiche-Kuhn sum rule) in the limit of a long, lightly damped signal.
`first_peak` returns the energy of the lowest clear maximum: the
"first-peak energy" whose mixed-vs-FP64 error the tetracene run reports.
"""
from __future__ import annotations

import numpy as np


def strength_function(d_dip, dt, omega, tau=None, window="exp", t0=None):
    """S(omega) of the sampled signal d_dip[k] at t_k = t0 + k dt (t0
    defaults to dt: the reference records the dipole after each step)."""
    d = np.asarray(d_dip, np.float64).reshape(-1)
    w = np.asarray(omega, np.float64).reshape(-1)
    t = (dt if t0 is None else t0) + dt * np.arange(d.size)
    T = t[-1] if d.size else 0.0
    if tau is None:
        tau = T / 5.0 if T > 0 else 1.0
    if window == "exp":
        D = np.exp(-t / tau)
    elif window == "gauss":
        D = np.exp(-0.5 * (t / tau) ** 2)
    else:
        raise ValueError("window must be 'exp' or 'gauss'")
    f = d * D * dt
    S = np.empty(w.size)
    for j0 in range(0, w.size, 512):  # blocks of frequencies: bounded memory
        wj = w[j0:j0 + 512]
        F = np.exp(1j * np.outer(wj, t)) @ f
        S[j0:j0 + 512] = -(2.0 * wj / np.pi) * F.imag
    return S


def first_peak(omega, S, rel=0.05):
    """Energy of the first local maximum of S above rel * max(S), refined by a
    parabola through the three samples around it."""
    w = np.asarray(omega, np.float64)
    s = np.asarray(S, np.float64)
    thr = rel * np.max(s)
    for j in range(1, s.size - 1):
        if s[j] > thr and s[j] >= s[j - 1] and s[j] > s[j + 1]:
            a, b, c = s[j - 1], s[j], s[j + 1]
            den = a - 2.0 * b + c
            off = 0.5 * (a - c) / den if den != 0.0 else 0.0
            return float(w[j] + off * (w[j + 1] - w[j - 1]) / 2.0)
    raise ValueError("no peak above the threshold")
