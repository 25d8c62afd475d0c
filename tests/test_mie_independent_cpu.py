"""CPU: the oracle's Mie tables against an independent Mie computation.

The oracle restates the reference's Mie kernels (CLARITAS/CLARITAS.py:3495-3592: logarithmic-derivative
recurrences, truncation at nstop, phase pdf on the reference's theta grid, trapezoid CDF) and equals the
reference's own code bit for bit. Here the same quantities come from a separate route: the Lorenz-Mie
coefficients from the Riccati-Bessel functions of scipy's spherical Bessel functions, the efficiencies and
asymmetry from the series of Bohren & Huffman, "Absorption and Scattering of Light by Small Particles"
(1983, sections 4.4-4.5), and the amplitude functions S1, S2 from the angular functions pi_n, tau_n.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_harness as H
from tardiis_and_claritas_gb300 import scene as S

special = pytest.importorskip("scipy.special")


def mie_coefficients(m: complex, x: float, nmax: int):
    n = np.arange(1, nmax + 1)
    mx = m * x
    jx, djx = special.spherical_jn(n, x), special.spherical_jn(n, x, derivative=True)
    yx, dyx = special.spherical_yn(n, x), special.spherical_yn(n, x, derivative=True)
    jm, djm = special.spherical_jn(n, mx), special.spherical_jn(n, mx, derivative=True)
    psi_x, dpsi_x = x * jx, jx + x * djx
    xi_x, dxi_x = x * (jx + 1j * yx), (jx + 1j * yx) + x * (djx + 1j * dyx)
    psi_m, dpsi_m = mx * jm, jm + mx * djm
    a = (m * psi_m * dpsi_x - psi_x * dpsi_m) / (m * psi_m * dxi_x - xi_x * dpsi_m)
    b = (psi_m * dpsi_x - m * psi_x * dpsi_m) / (psi_m * dxi_x - m * xi_x * dpsi_m)
    return n, a, b


def efficiencies(a, b, n, x):
    qext = 2.0 / x ** 2 * np.sum((2 * n + 1) * (a + b).real)
    qsca = 2.0 / x ** 2 * np.sum((2 * n + 1) * (np.abs(a) ** 2 + np.abs(b) ** 2))
    g1 = np.sum(n[:-1] * (n[:-1] + 2) / (n[:-1] + 1) * (a[:-1] * np.conj(a[1:]) + b[:-1] * np.conj(b[1:])).real)
    g2 = np.sum((2 * n + 1) / (n * (n + 1)) * (a * np.conj(b)).real)
    g = 4.0 / (x ** 2 * qsca) * (g1 + g2)
    qback = np.abs(np.sum((2 * n + 1) * (-1.0) ** n * (a - b))) ** 2 / x ** 2
    return qext, qsca, g, qback


def phase_pdf(a, b, n, theta):
    """0.5 (|S1|^2 + |S2|^2) sin(theta) with S1, S2 from the angular functions pi_n, tau_n."""
    mu = np.cos(theta)
    s1 = np.zeros(theta.shape, complex)
    s2 = np.zeros(theta.shape, complex)
    pi_prev, pi_cur = np.zeros_like(mu), np.ones_like(mu)
    for k, nn in enumerate(n):
        tau = nn * mu * pi_cur - (nn + 1) * pi_prev
        c = (2 * nn + 1) / (nn * (nn + 1))
        s1 += c * (a[k] * pi_cur + b[k] * tau)
        s2 += c * (a[k] * tau + b[k] * pi_cur)
        pi_prev, pi_cur = pi_cur, ((2 * nn + 1) * mu * pi_cur - (nn + 1) * pi_prev) / nn
    return 0.5 * (np.abs(s1) ** 2 + np.abs(s2) ** 2) * np.sin(theta)


@pytest.mark.parametrize("k_imag", [0.0, 1e-3])
@pytest.mark.parametrize("d_range", [(0.1e-6, 12e-6), (20e-6, 200e-6)])  # size parameters ~0.5-60, ~97-972
def test_oracle_mie_matches_independent_series(k_imag, d_range):
    cfg = S.small_cell_config(particle_surface_rms_slope_deg=0.0, wave_surface_rms_height_m=0.0)
    d = np.geomspace(*d_range, 6)
    parts = S.Particles(d, np.ones(d.size), np.full(d.size, 1.54), np.full(d.size, k_imag), 0.1, 2650.0)
    orc = H.OracleRun("port", cfg, parts)
    ph = orc.physics()
    orc.close()
    n_med = float(cfg.n_water)
    m = complex(1.54, k_imag) / n_med
    theta = ph["theta"]
    for i in range(d.size):
        x = float(ph["size_parameter"][i])
        assert x == pytest.approx(np.pi * d[i] * n_med / cfg.particle_wavelength_m, rel=1e-12)
        nstop = int(ph["nstop"][i])
        n, a, b = mie_coefficients(m, x, nstop)
        qext, qsca, g, qback = efficiencies(a, b, n, x)
        np.testing.assert_allclose([ph["qext"][i], ph["qsca"][i], ph["asym_g"][i]], [qext, qsca, g], rtol=1e-9)
        np.testing.assert_allclose(ph["qback"][i], qback, rtol=1e-8, atol=1e-14)
        # the truncation at nstop (x + 4 x^(1/3) + 2) leaves out less than 1e-8 of the series
        n2, a2, b2 = mie_coefficients(m, x, nstop + 15)
        np.testing.assert_allclose(efficiencies(a2, b2, n2, x)[:2], [qext, qsca], rtol=1e-8)
        # the phase CDF: trapezoid integral of the pdf on the oracle's angle grid, normalised
        pdf = phase_pdf(a, b, n, theta)
        cdf = np.concatenate([[0.0], np.cumsum(0.5 * (pdf[1:] + pdf[:-1]) * np.diff(theta))])
        cdf /= cdf[-1]
        np.testing.assert_allclose(ph["phase_cdf"][i], cdf, rtol=1e-8, atol=1e-12)
