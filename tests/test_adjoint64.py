"""The FP64 host adjoint (oracle/adjoint64.py), pinned to the oracle.

Its forward model must give the FP64 oracle's objective to 1e-12 relative
for every operator the engine's adjoint supports, and its reverse-mode
gradient must agree with central differences of the oracle.  The engine's
adjoint is then held to it on the GPU (tests/test_adjoint_gpu.py).
"""
import numpy as np
import pytest

import adjoint64 as A
import cases as C
import test_adjoint_gpu as T


def model(c, drag=False):
    return A.Model(c["nx"], c["ny"], c["op"], c["S"], c["omega"], c["flags"], c["periodic"], c["rho"], c["u"],
                   T.weights(c), T.FIRST, T.T, drag=drag)


@pytest.mark.parametrize("op", [C.BGK, C.MRT, C.CM, C.CM_OPT])
def test_host_adjoint_forward_is_the_oracles(op):
    c = T.case(op)
    fx = float(c["force"][0].flat[0])
    gam = c["gamma"].astype(np.float64)
    J, g, gw, gfx, gfy = model(c).gradient(gam, c["omega"], fx, 0.0)
    assert abs(J - T.oracle_J(c, gam, c["omega"], fx, 0.0)) <= 1e-12 * abs(J)
    # omega and a smooth gamma direction against FP64 central differences
    h = 1e-4
    fd = (T.oracle_J(c, gam, c["omega"] + h, fx, 0.0) - T.oracle_J(c, gam, c["omega"] - h, fx, 0.0)) / (2 * h)
    assert abs(gw - fd) <= 1e-6 * abs(fd)
    d = C.brinkman_field(T.NX, T.NY, sigma=2.0, seed=7).astype(np.float64) - 0.5
    h = 1e-6
    fd = (T.oracle_J(c, gam + h * d, c["omega"], fx, 0.0) - T.oracle_J(c, gam - h * d, c["omega"], fx, 0.0)) / (2 * h)
    assert abs((g * d).sum() - fd) <= 1e-6 * abs(fd) + 1e-12


def test_host_adjoint_rejects_open_edges():
    c = T.case(C.BGK)
    fl = c["flags"].copy()
    fl[0, :] = C.FLUID
    with pytest.raises(ValueError):
        A.Model(c["nx"], c["ny"], C.BGK, c["S"], c["omega"], fl, c["periodic"], c["rho"], c["u"], T.weights(c),
                T.FIRST, T.T)
