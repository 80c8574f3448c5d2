"""Stochastic rounding of the 16-bit storage forms.

Rounding to nearest gives a steady flow the same rounding error at every node
every step, a persistent source term that the slow viscous modes amplify
with the lattice size; stochastic rounding (the default) makes every store
unbiased.  Checked on the lid-driven cavity at Re 1000 run towards steady
state: against the engine's FP32 run, against the FP64 oracle's field after
its steady state (tests/golden/steady_cavity256_mrt.npz, made by
make_steady_cavity.py in that folder), and for bitwise reproducibility.
"""
import os

import numpy as np
import pytest

import cases as C
import lbmx

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "steady_cavity256_mrt.npz")
F32, F16, BF16 = 0, 1, 2


def cavity(n, storage, options=0):
    c = C.cavity_moving_wall(n, n, op=C.MRT, nu=0.1 * n / 1000.0, u_lid=0.1)
    return C.make_lattice(c, storage=storage, options=options)


def velocity(n, storage, steps, options=0):
    L = cavity(n, storage, options)
    L.step(steps)
    _, u, _ = L.moments()
    return u.astype(np.float64)


def l2(u, ref):
    return float(np.sqrt(((u - ref) ** 2).sum() / (ref ** 2).sum()))


def test_stochastic_rounding_removes_the_steady_state_bias():
    n, steps = 256, 20000
    u32 = velocity(n, F32, steps)
    e16 = l2(velocity(n, F16, steps), u32)
    e16_nearest = l2(velocity(n, F16, steps, lbmx.OPTION_ROUND_NEAREST), u32)
    ebf = l2(velocity(n, BF16, steps), u32)
    ebf_nearest = l2(velocity(n, BF16, steps, lbmx.OPTION_ROUND_NEAREST), u32)
    assert e16 < 1.5e-3, e16
    assert ebf < 1e-2, ebf
    # round to nearest drifts an order of magnitude further
    assert e16_nearest > 5 * e16 and ebf_nearest > 5 * ebf, (e16_nearest, ebf_nearest)


def test_steady_state_against_the_fp64_oracle():
    """At steady state (the FP64 field changes by at most 1e-6 over its last
    1000 steps) FP16 offset storage with stochastic rounding is as close to
    FP64 as FP32 storage is (both about 1.1e-3: FP32 stores f itself, whose
    rounding the slow modes amplify as well); BF16 within 1e-2."""
    import json
    g = np.load(GOLDEN)
    meta = json.loads(str(g["meta"]))
    assert meta["residual_last_1000_steps"] <= 1e-6
    ref = g["u"]
    err = {}
    for storage in (F32, F16, BF16):
        u = velocity(256, storage, meta["steps"])
        err[storage] = l2(u[:, ::4, ::4], ref)
    print("steady-state L2 error vs FP64 after %d steps: FP32 %.2e FP16 %.2e BF16 %.2e"
          % (meta["steps"], err[F32], err[F16], err[BF16]))
    assert err[F32] < 1.5e-3, err
    assert err[F16] < 1.2 * err[F32], err
    assert err[BF16] < 1e-2, err


def test_stochastic_rounding_is_reproducible():
    runs = []
    for _ in range(2):
        L = cavity(96, F16)
        L.step(301)
        runs.append(L.populations())
    np.testing.assert_array_equal(runs[0], runs[1])
