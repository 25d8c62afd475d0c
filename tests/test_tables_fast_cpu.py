"""CPU: the algebra of the fast phase tables, restated in numpy.

The fast pdf kernel evaluates S1 and S2 at mu and at -mu from one Legendre recurrence, using
pi_n(-mu) = (-1)^(n-1) pi_n(mu) and tau_n(-mu) = (-1)^n tau_n(mu) and sums split by the parity of n:
S1(mu) = Po+Qo+Pe+Qe, S1(-mu) = Po-Qo-Pe+Qe, S2(mu) = Ro+To+Re+Te, S2(-mu) = -Ro+To+Re-Te with
P = c a pi, Q = c b tau, R = c a tau, T = c b pi. This checks those identities against direct sums at both
angles for random coefficients, and the symmetry of the reference's theta grid they rely on.
"""
from __future__ import annotations

import numpy as np


def _pi_tau(mu: float, nmax: int):
    pi = np.zeros(nmax + 2)
    tau = np.zeros(nmax + 1)
    pi[1] = 1.0
    for n in range(1, nmax + 1):
        tau[n] = n * mu * pi[n] - (n + 1) * pi[n - 1]
        pi[n + 1] = ((2 * n + 1) / n) * mu * pi[n] - ((n + 1) / n) * pi[n - 1]
    return pi[1:nmax + 1], tau[1:nmax + 1]


def _direct(mu, a, b):
    n = np.arange(1, a.size + 1)
    c = (2 * n + 1) / (n * (n + 1.0))
    pi, tau = _pi_tau(mu, a.size)
    return np.sum(c * (a * pi + b * tau)), np.sum(c * (a * tau + b * pi))


def _mirrored(mu, a, b):
    n = np.arange(1, a.size + 1)
    c = (2 * n + 1) / (n * (n + 1.0))
    A, B = c * a, c * b
    pi, tau = _pi_tau(mu, a.size)
    odd = (n % 2) == 1
    P, Q, R, T = A * pi, B * tau, A * tau, B * pi
    Po, Qo, Ro, To = (x[odd].sum() for x in (P, Q, R, T))
    Pe, Qe, Re, Te = (x[~odd].sum() for x in (P, Q, R, T))
    return (Po + Qo + Pe + Qe, Ro + To + Re + Te), (Po - Qo - Pe + Qe, -Ro + To + Re - Te)


def test_mirrored_sums_equal_direct_sums():
    rng = np.random.default_rng(7)
    for nmax in (3, 40, 400):
        a = rng.normal(size=nmax) + 1j * rng.normal(size=nmax)
        b = rng.normal(size=nmax) + 1j * rng.normal(size=nmax)
        for mu in (1.0, 0.93, 0.31, 0.0, 1e-3):
            (s1p, s2p), (s1m, s2m) = _mirrored(mu, a, b)
            d1p, d2p = _direct(mu, a, b)
            d1m, d2m = _direct(-mu, a, b)
            scale = np.sum(np.abs(a) + np.abs(b)) * nmax ** 2
            for x, y in ((s1p, d1p), (s2p, d2p), (s1m, d1m), (s2m, d2m)):
                assert abs(x - y) <= 1e-12 * scale


def test_reference_theta_grid_is_mirror_symmetric():
    # theta_j = pi/2 (1 - cos(pi j/(nt-1))) (CLARITAS/CLARITAS.py:3488-3493): theta_{nt-1-j} = pi - theta_j to
    # rounding, for odd and even grid sizes
    for nt in (257, 1801, 2048):
        j = np.arange(nt)
        th = 0.5 * np.pi * (1.0 - np.cos(np.pi * j / (nt - 1)))
        th[0], th[-1] = 0.0, np.pi
        assert np.max(np.abs(th[::-1] - (np.pi - th))) < 2e-15  # a few ulps of pi
        assert np.max(np.abs(np.cos(th[::-1]) + np.cos(th))) < 2e-15
