"""Plain PM is the fallback and the yardstick: the monitor's revert logic on synthetic series (CPU)."""
import math

from augur_gb300.learned import FallbackMonitor


def test_stays_enabled_under_threshold():
    m = FallbackMonitor(drift_max=0.05, corr_max=0.5)
    for e in [-1.0, -1.01, -0.99, -1.03, -0.97]:
        assert m.observe(energy=e, corr_ratio=0.1)
    assert not m.reverted


def test_reverts_on_energy_drift_and_stays_reverted():
    m = FallbackMonitor(drift_max=0.05)
    series = [-2.0, -2.02, -2.05, -2.2, -2.0]
    states = [m.observe(energy=e) for e in series]
    assert states == [True, True, True, False, False]
    assert "energy drift" in m.reason


def test_reverts_on_large_correction_and_on_nonfinite_values():
    m = FallbackMonitor(corr_max=0.5)
    assert m.observe(corr_ratio=0.49)
    assert not m.observe(corr_ratio=0.51)
    m2 = FallbackMonitor()
    m2.observe(energy=-1.0)
    assert not m2.observe(energy=math.nan)
