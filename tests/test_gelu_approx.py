"""The pair MLP's GELU uses erfc from Abramowitz & Stegun eq. 7.1.26 (|erf error| <= 1.5e-7);
this restates the formula in float64 and checks that bound and the resulting GELU error against
the exact (erf) GELU over the range the pair MLP sees. No GPU."""
import numpy as np
import pytest

special = pytest.importorskip("scipy.special")


def gelu_as(x):
    z = np.abs(x) / np.sqrt(2.0)
    t = 1.0 / (1.0 + 0.3275911 * z)
    poly = t * (0.254829592 + t * (-0.284496736 + t * (1.421413741 + t * (-1.453152027 + t * 1.061405429))))
    ec = poly * np.exp(-z * z)
    return 0.5 * x * np.where(x >= 0, 2.0 - ec, ec)


def test_published_erf_bound_and_gelu_error():
    x = np.linspace(-12.0, 12.0, 2_000_001)
    z = np.abs(x) / np.sqrt(2.0)
    t = 1.0 / (1.0 + 0.3275911 * z)
    poly = t * (0.254829592 + t * (-0.284496736 + t * (1.421413741 + t * (-1.453152027 + t * 1.061405429))))
    erf_as = 1.0 - poly * np.exp(-z * z)
    assert np.abs(erf_as - special.erf(z)).max() <= 1.5e-7
    exact = 0.5 * x * (1.0 + special.erf(x / np.sqrt(2.0)))
    err = np.abs(gelu_as(x) - exact)
    assert np.all(err <= 0.5 * np.abs(x) * 1.5e-7 + 1e-12)
