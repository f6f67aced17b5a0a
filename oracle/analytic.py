"""Analytic nested-sphere solutions (test infrastructure, CPU, numpy).

This module is part of the oracle: only the tests, ``__graft_entry__.smoke``
and the bench's CPU leg may use it, as a checker of the GPU results.  It
restates published closed forms, not reference code:

* EEG: potential on the outer surface of a piecewise-homogeneous, isotropic
  concentric-sphere conductor for a current dipole in the innermost layer,
  as a Legendre series whose radial factors come from the interface
  conditions (continuity of the potential and of the normal current, no
  current through the outer surface) -- the layered-sphere solution of
  de Munck & Peters, IEEE Trans. Biomed. Eng. 40(11), 1993, written here
  with per-layer ratios B_k / A_k propagated inward from the outer
  surface, then amplitudes propagated outward.
* MEG: Sarvas's formula for the magnetic field outside a spherically
  symmetric conductor (Phys. Med. Biol. 32(1), 1987), with
  mu0 / (4 pi) = 1e-7 (OpenMEEG/include/constants.h:22).
* RDM / MAG: the column-wise comparison measures of the reference's test
  tool (tests/test_compare_matrix.cpp:305-380): columns are centred (average
  reference), RDM = || u/|u| - v/|v| ||, MAG = | 1 - |u|/|v| |.

The reference ships analytic values for its sample head Head3 (computed
elsewhere); ``tests/golden/make_golden.py`` stores them with the sample's
dipoles and sensors, and ``tests/test_cpu_oracle.py`` pins this module to
them.
"""
from __future__ import annotations

import numpy as np

MAG_FACTOR = 1e-7


def _radial_factors(radii, sigmas, nmax):
    """g[n] (n = 1..nmax): potential at the outer radius of the n-th harmonic
    whose source part in the innermost layer is r^-(n+1) (unit coefficient)."""
    radii = np.asarray(radii, np.float64)
    sig = np.asarray(sigmas, np.float64)
    L = len(radii)
    g = np.zeros(nmax + 1)
    for n in range(1, nmax + 1):
        # t_k = rho_k / r_k^(2n+1) for the layer inside interface k; outer layer: no normal current
        rho_over_u = [0.0] * L                          # rho_{k} / r_k^{2n+1}, k = layer index
        t_out = n / (n + 1.0)                           # rho_L / r_L^{2n+1}
        rho_over_u[L - 1] = t_out
        # propagate inward: layer k (inside radius r_k) from layer k+1
        t_next = t_out                                  # rho_{k+1} / r_{k+1}^{2n+1}
        for k in range(L - 2, -1, -1):
            # rho_{k+1} / r_k^{2n+1}
            t = t_next * (radii[k + 1] / radii[k]) ** (2 * n + 1)
            # rho_k / r_k^{2n+1} = (n - F) / (F + n + 1) with F = sr (n - (n+1) t) / (1 + t),
            # expanded so that no difference of nearly equal terms is formed
            sr = sig[k + 1] / sig[k]
            if t <= 1.0:
                num = n * (1.0 - sr) + t * (n + sr * (n + 1))
                den = sr * n + (n + 1) + (n + 1) * (1.0 - sr) * t
            else:
                u = 1.0 / t
                num = n * (1.0 - sr) * u + (n + sr * (n + 1))
                den = (sr * n + n + 1) * u + (n + 1) * (1.0 - sr)
            rho_over_u[k] = num / den
            t_next = rho_over_u[k]
        # amplitudes: B_1 = 1, A_1 = 1 / rho_1; outward through the interfaces
        logA = -np.log(abs(rho_over_u[0])) - (2 * n + 1) * np.log(radii[0])
        signA = np.sign(rho_over_u[0])
        for k in range(L - 1):
            # A_{k+1} / A_k = (1 + rho_k / u_k) / (1 + rho_{k+1} / u_k), u_k = r_k^{2n+1}
            num = 1.0 + rho_over_u[k]
            den = 1.0 + (rho_over_u[k + 1] * (radii[k + 1] / radii[k]) ** (2 * n + 1))
            logA += np.log(abs(num)) - np.log(abs(den))
            signA *= np.sign(num) * np.sign(den)
        rN = radii[-1]
        # V(r_N) = A_L r_N^n (1 + rho_L / r_N^{2n+1}) = A_L r_N^n (2n+1)/(n+1)
        g[n] = signA * np.exp(logA + n * np.log(rN)) * (2 * n + 1.0) / (n + 1.0)
    return g


def eeg_sphere(radii, sigmas, dipoles, electrodes, tol=1e-14, nmax=6000):
    """Potentials (n_electrodes x n_dipoles) on the outer sphere.

    radii: interface radii, innermost first (the last is the outer surface);
    sigmas: conductivity of each layer, innermost first; dipoles (n, 6) in the
    innermost layer; electrodes (m, 3), projected onto the outer sphere.
    """
    dip = np.asarray(dipoles, np.float64)
    el = np.asarray(electrodes, np.float64)[:, :3]
    r0 = dip[:, :3]
    q = dip[:, 3:6]
    b = np.linalg.norm(r0, axis=1)
    rN = float(radii[-1])
    if np.any(b >= radii[0]):
        raise ValueError("dipoles must lie inside the innermost sphere")
    ratio = max(float(b.max()) / float(radii[0]), 1e-3)
    n_need = int(np.ceil(np.log(tol) / np.log(ratio))) + 10
    # (r_N / r_1)^(2n+1) (the ratios accumulated over the interfaces) must stay inside the double range
    span = float(np.log(float(radii[-1]) / float(radii[0])))
    n_safe = int(600.0 / (2.0 * span)) if span > 0 else nmax
    if n_need > min(nmax, n_safe):
        raise ValueError("a dipole is too close to the innermost sphere for the series in double precision")
    N = max(n_need, 20)
    g = _radial_factors(radii, sigmas, N)
    rh = el / np.linalg.norm(el, axis=1, keepdims=True)
    bs = np.where(b > 0, b, 1.0)
    r0h = r0 / bs[:, None]
    qr = np.sum(q * r0h, axis=1)                                    # (nd,)
    x = np.clip(rh @ r0h.T, -1.0, 1.0)                              # cos gamma (ne, nd)
    qdotr = rh @ q.T                                                # q . r_hat (ne, nd)
    # sum_n b^(n-1) g_n [ n q_r P_n(x) + (q.r - q_r x) P_n'(x) ]
    V = np.zeros_like(x)
    P_prev, P = np.ones_like(x), x.copy()                            # P_0, P_1
    dP_prev, dP = np.zeros_like(x), np.ones_like(x)                  # P_0', P_1'
    bpow = np.ones_like(b)                                           # b^(n-1)
    for n in range(1, N + 1):
        V += (bpow * g[n])[None, :] * (n * qr[None, :] * P + (qdotr - qr[None, :] * x) * dP)
        # P_{n+1} = ((2n+1) x P_n - n P_{n-1}) / (n+1); P'_{n+1} = P'_{n-1} + (2n+1) P_n
        P_next = ((2 * n + 1) * x * P - n * P_prev) / (n + 1)
        dP_next = dP_prev + (2 * n + 1) * P
        P_prev, P, dP_prev, dP = P, P_next, dP, dP_next
        bpow = bpow * b
    return V / (4.0 * np.pi * float(sigmas[0]))


def sarvas(dipoles, squids):
    """Magnetic field component along each sensor's (normalised) orientation,
    n_squids x n_dipoles, for dipoles in a spherically symmetric conductor
    centred at the origin."""
    dip = np.asarray(dipoles, np.float64)
    sq = np.asarray(squids, np.float64)
    r = sq[:, None, :3]
    o = sq[:, 3:6] / np.linalg.norm(sq[:, 3:6], axis=1, keepdims=True)
    rq = dip[None, :, :3]
    Q = dip[None, :, 3:6]
    a = r - rq
    an = np.linalg.norm(a, axis=2)
    rn = np.linalg.norm(r, axis=2)
    adotr = np.sum(a * r, axis=2)
    F = an * (rn * an + rn ** 2 - np.sum(rq * r, axis=2))
    gF = (an ** 2 / rn + adotr / an + 2 * an + 2 * rn)[..., None] * r - (an + 2 * rn + adotr / an)[..., None] * rq
    Qxrq = np.cross(Q, rq)
    B = MAG_FACTOR / F[..., None] ** 2 * (F[..., None] * Qxrq - np.sum(Qxrq * r, axis=2)[..., None] * gF)
    return np.sum(B * o[:, None, :], axis=2)


def rdm(u, v):
    """Column-wise relative difference measure of centred columns."""
    u = np.asarray(u, np.float64) - np.mean(u, axis=0)
    v = np.asarray(v, np.float64) - np.mean(v, axis=0)
    return np.linalg.norm(u / np.linalg.norm(u, axis=0) - v / np.linalg.norm(v, axis=0), axis=0)


def mag(u, v):
    """Column-wise magnification error of centred columns."""
    u = np.asarray(u, np.float64) - np.mean(u, axis=0)
    v = np.asarray(v, np.float64) - np.mean(v, axis=0)
    return np.abs(1.0 - np.linalg.norm(u, axis=0) / np.linalg.norm(v, axis=0))
