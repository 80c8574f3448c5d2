"""The bench's force statistics on synthetic drag and lift series (CPU): the
spectral peak of a Hann-windowed FFT refined by a parabola recovers a
frequency between FFT bins, and shedding_stats returns the coefficients,
Strouhal number and periods the signals were built with."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


@pytest.mark.parametrize("period", [7946.0, 1234.5, 333.3])
def test_spectral_peak_between_bins(period):
    rng = np.random.default_rng(5)
    t = np.arange(100_000)
    x = 0.3 * np.sin(2 * np.pi * t / period + 0.4) + 0.01 * rng.standard_normal(t.size) + 2.0
    f = bench.spectral_peak(x)
    assert abs(1.0 / f - period) <= 2e-3 * period


def test_shedding_stats_recovers_the_built_signal():
    T, D, U = 200_000, 64.0, 0.05
    q = 0.5 * U * U * D
    t = np.arange(T)
    rng = np.random.default_rng(7)
    # the shedding (lift at the shedding frequency) and an acoustic mode in the drag
    St, cd, cl_amp, p_drag = 0.161, 1.369, 0.325, 14_396.7
    f = St * U / D
    lift = cl_amp * np.sin(2 * np.pi * f * t) + 1e-3 * rng.standard_normal(T)
    drag = cd + 0.3 * np.sqrt(2) * np.sin(2 * np.pi * t / p_drag) + 1e-3 * rng.standard_normal(T)
    s = bench.shedding_stats(np.stack([drag * q, lift * q], axis=1), q, D, U)
    assert abs(s["strouhal"] - St) <= 2e-3 * St
    assert abs(s["C_D_mean"] - cd) <= 2e-3
    assert abs(s["C_L_amplitude"] - cl_amp) <= 5e-3 * cl_amp
    assert abs(s["C_D_period_steps"] - p_drag) <= 5e-3 * p_drag
    # a stationary lift: the quarters hold 6.3 periods each, so their RMS
    # differs by the partial period only
    assert abs(s["C_L_rms_change_q3_to_q4"]) < 0.05
