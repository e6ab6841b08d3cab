"""Blocking analysis (hande_gb300.analysis) on data with known statistics."""

import numpy as np

from hande_gb300 import analysis


def _ar1(n, phi, rng):
    x = np.empty(n)
    x[0] = rng.normal()
    e = rng.normal(size=n) * np.sqrt(1 - phi * phi)
    for i in range(1, n):
        x[i] = phi * x[i - 1] + e[i]
    return x


def test_reblock_recovers_correlated_error():
    rng = np.random.default_rng(3)
    phi, n = 0.9, 1 << 16
    x = _ar1(n, phi, rng)
    mean, err, opt = analysis.mean_error(x)
    exact = np.sqrt((1 + phi) / (1 - phi) / n)  # unit-variance AR(1)
    assert opt > 2
    assert abs(err / exact - 1) < 0.25
    naive = x.std(ddof=1) / np.sqrt(n)
    assert err > 3 * naive


def test_projected_energy_ratio():
    rng = np.random.default_rng(5)
    n = 1 << 14
    d0 = 100 + 5 * _ar1(n, 0.5, rng)
    num = -0.25 * d0 + 0.5 * _ar1(n, 0.5, rng)
    e, err, opt = analysis.projected_energy(num, d0)
    assert abs(e + 0.25) < 5 * err
    assert 0 < err < 1e-3
