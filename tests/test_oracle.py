"""CPU checks of the oracle (the restatement of the reference step).

The reference ships no test vectors; its results are pinned by the analytic
validators each scenario carries (taylorGreenFunctors.cuh:57-98,
poiseuilleFunctors.cuh:63-87), which these tests apply to the oracle, and by
the golden dumps of the patched reference build in tests/golden/ where
present (test_golden.py).
"""
import numpy as np
import pytest

import cases as C
import oracle as O


def test_taylor_green_decay_matches_analytic():
    nu = 0.01
    c = C.taylor_green(64, 64, op=C.BGK, nu=nu)
    o = C.make_oracle(c)
    u0 = np.asarray(c["u"])
    k = 2 * np.pi / 64
    o.step(400)
    _, u, _ = o.moments()
    amp = np.sqrt((u ** 2).sum() / (u0 ** 2).sum())
    assert abs(amp - np.exp(-2 * nu * k * k * 400)) < 3e-3


@pytest.mark.parametrize("op", [C.BGK, C.MRT, C.CM])
def test_poiseuille_profile(op):
    nu, umax, ny = 1.0 / 6.0, 0.05, 16
    c = C.poiseuille(8, ny, op=op, nu=nu, u_max=umax)
    o = C.make_oracle(c)
    o.step(3000)
    _, u, _ = o.moments()
    prof = u[0].mean(axis=1)
    # on-node bounce-back walls at y = 0 and ny-1 leave the no-slip planes on
    # the wall rows: u(y) = F/(2 nu) y (ny-1-y), the parabola of the
    # reference's validator with NY-1 as the channel width
    F = 8 * nu * umax / ny ** 2
    y = np.arange(1, ny - 1)
    ana = F / (2 * nu) * y * (ny - 1.0 - y)
    err = np.abs(prof[1:-1] - ana).max() / ana.max()
    assert err < 0.05, err


def test_mass_conserved_periodic_and_closed():
    for c in (C.taylor_green(32, 32, op=C.MRT), C.cavity_moving_wall(32, 24, op=C.BGK)):
        o = C.make_oracle(c)
        o.step(1)
        m0 = o.sums()[0]
        o.step(200)
        assert abs(o.sums()[0] - m0) / m0 < 1e-12


def test_mrt_with_uniform_rates_is_bgk():
    om = 1.3
    c = C.random_state(C.taylor_green(24, 20, op=C.BGK, nu=(1 / om - 0.5) / 3), seed=1)
    c2 = dict(c, op=C.MRT, S=[om] * 9)
    a, b = C.make_oracle(c), C.make_oracle(c2)
    a.step(10)
    b.step(10)
    assert np.abs(a.populations() - b.populations()).max() < 1e-12


def test_f32_oracle_close_to_f64():
    c = C.cavity_regularized(32, 32, op=C.MRT, quirks=C.QUIRKS_REFERENCE)
    a, b = C.make_oracle(c, "f64"), C.make_oracle(c, "f32")
    a.step(200)
    b.step(200)
    _, ua, _ = a.moments()
    _, ub, _ = b.moments()
    assert np.abs(ua - ub).max() < 2e-5


def test_rest_population_quirk_lags_two_steps():
    # with the quirk, f0 after step t is the collision output of step t-2's f0 slot
    c = C.random_state(C.taylor_green(16, 16, op=C.BGK), seed=2)
    q = C.make_oracle(dict(c, quirks=O.QUIRK_REST_LAG))
    n = C.make_oracle(c)
    q.step(1)
    n.step(1)
    # first step: both start from f_eq and collide identical inputs except f0
    # which is the init value in both cases, so populations agree
    assert np.abs(q.populations() - n.populations()).max() < 1e-14
    q.step(1)
    n.step(1)
    assert np.abs(q.populations()[0] - n.populations()[0]).max() > 1e-8


def test_zouhe_left_quirk_changes_inlet_density():
    c = C.channel(32, 16)
    a = C.make_oracle(dict(c, quirks=O.QUIRK_ZOUHE_LEFT))
    b = C.make_oracle(c)
    a.step(20)
    b.step(20)
    ra, _, _ = a.moments()
    rb, _, _ = b.moments()
    assert np.abs(ra[:, 0] - rb[:, 0]).max() > 1e-6


def test_ibm_force_opposes_flow():
    mk = C.cylinder_markers(16.0, 12.0, 3.0, 16)
    c = C.channel(48, 24, markers=mk)
    o = C.make_oracle(c)
    o.step(200)
    _, _, F = o.markers()
    assert F[0].sum() < 0  # drag on the fluid points upstream


def test_oracle_brinkman_term():
    # gamma = 0 is the plain step bit for bit; a solid fraction slows the channel
    c = C.channel_brinkman(32, 16, op=C.BGK, sigma=2.0, gamma_scale=0.5)
    assert 0.0 <= c["gamma"].min() and c["gamma"].max() <= 0.5 + 1e-7
    o1 = C.make_oracle(c)
    o1.step(40)
    _, u1, _ = o1.moments()
    o0 = C.make_oracle(c)
    o0.set_gamma(np.zeros_like(c["gamma"]))
    o0.step(40)
    _, u0, _ = o0.moments()
    np.testing.assert_array_equal(u0, u1)
    o2 = C.make_oracle(c)
    o2.set_gamma(c["gamma"])
    o2.step(40)
    _, u2, _ = o2.moments()
    assert u2[0].mean() < 0.9 * u1[0].mean()
