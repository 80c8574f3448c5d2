"""Tangent-linear model (lbmx_tangent_*): derivatives of a run with respect to
one scalar parameter.

The forward values must match the engine's own step; the derivatives of the
time-averaged drag and lift on an IBM cylinder (inlet velocity, omega), of
the cavity's velocity field (lid velocity) and of a forced channel's velocity
(body force) must match central finite differences of the FP64 oracle to
1e-3 relative.
"""
import numpy as np
import pytest

import cases as C
import lbmx

pytestmark = pytest.mark.gpu

RTOL = 1e-3


def cylinder(op=C.BGK, u_in=0.05):
    # off-centre cylinder (so the lift is not zero by symmetry) in a channel
    # with a parabolic Zou-He inlet and a Zou-He pressure outlet
    mk = C.cylinder_markers(30.3, 21.7, 6.0, 36)
    return C.channel(112, 44, op=op, nu=0.04, u_in=u_in, inlet="parabolic", outlet="zouhe_p", markers=mk)


def tangent_of(c, parameter, **over):
    kw = dict(op=c["op"], omega=c["omega"], S=c["S"], periodic=c["periodic"], flags=c["flags"], quirks=c["quirks"],
              u_bc=c["u_bc"], wall_u=c["wall_u"], rho_out=c["rho_out"])
    if c["force"] is not None:
        kw["body_force"] = (float(np.asarray(c["force"])[0].flat[0]), float(np.asarray(c["force"])[1].flat[0]))
    kw.update(over)
    t = lbmx.Tangent(c["nx"], c["ny"], parameter, **kw)
    t.set_state(np.asarray(c["rho"], np.float32), np.asarray(c["u"], np.float32))
    if c["markers"] is not None:
        t.set_markers(c["markers"])
    return t


def oracle_run(c, steps, **over):
    """FP64 oracle run; returns (per-step drag and lift [steps, 2] or None, final u)."""
    import oracle as O
    p = dict(op=c["op"], omega=c["omega"], S=c["S"], periodic=c["periodic"], quirks=c["quirks"], u_bc=c["u_bc"],
             wall_u=c["wall_u"], rho_out=c["rho_out"])
    force = c["force"]
    if "omega" in over:
        p["S"] = C.S_for(c["op"], over["omega"])
    if "body_fx" in over:
        force = np.zeros((2, c["ny"], c["nx"]))
        force[0] = over.pop("body_fx")
    p.update(over)
    o = O.Oracle(c["nx"], c["ny"], precision="f64", **p)
    o.set_flags(c["flags"])
    o.init(c["rho"], c["u"], force)
    dl = None
    if c["markers"] is not None:
        o.set_markers(c["markers"])
        dl = np.zeros((steps, 2))
        for s in range(steps):
            o.step(1)
            _, _, F = o.markers()
            dl[s] = -F.sum(axis=1)
    else:
        o.step(steps)
    _, u, _ = o.moments()
    return dl, u


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-30)


@pytest.mark.parametrize("op", [C.BGK, C.MRT, C.CM])
def test_tangent_forward_matches_engine(op):
    c = cylinder(op)
    t = tangent_of(c, lbmx.TANGENT_U_BC)
    series = t.run(100)
    rho_t, u_t, _, _ = t.moments()
    L = C.make_lattice(c)
    L.step(100)
    rho_e, u_e, _ = L.moments()
    _, dl = L.marker_forces()
    assert np.abs(rho_t - rho_e).max() < 5e-6 and np.abs(u_t - u_e).max() < 5e-6
    assert rel(series[-1, 0], dl[0]) < 1e-4 and abs(series[-1, 1] - dl[1]) < 1e-4 * abs(dl[0])
    assert t.t_steps == 100


@pytest.mark.parametrize("op,parameter", [(C.BGK, lbmx.TANGENT_U_BC), (C.MRT, lbmx.TANGENT_U_BC),
                                          (C.CM, lbmx.TANGENT_U_BC), (C.BGK, lbmx.TANGENT_OMEGA),
                                          (C.MRT, lbmx.TANGENT_OMEGA)])
def test_mean_drag_derivative_matches_fp64_finite_differences(op, parameter):
    T, first = 400, 200  # mean over steps 201..400
    c = cylinder(op)
    t = tangent_of(c, parameter)
    s = t.run(T)
    d_drag, d_lift = s[first:, 2].mean(), s[first:, 3].mean()
    if parameter == lbmx.TANGENT_U_BC:
        h, key, x0 = 1e-4, "u_bc", c["u_bc"]
    else:
        h, key, x0 = 1e-4, "omega", c["omega"]
    dp, _ = oracle_run(c, T, **{key: x0 + h})
    dm, _ = oracle_run(c, T, **{key: x0 - h})
    fd = (dp[first:].mean(axis=0) - dm[first:].mean(axis=0)) / (2 * h)
    assert rel(d_drag, fd[0]) < RTOL, (d_drag, fd[0])
    assert abs(d_lift - fd[1]) < RTOL * max(abs(fd[1]), 1e-2 * abs(fd[0])), (d_lift, fd[1])


def test_lid_velocity_derivative_of_the_cavity_field():
    c = C.cavity_moving_wall(48, 40, op=C.MRT, nu=0.02, u_lid=0.1)
    t = tangent_of(c, lbmx.TANGENT_WALL_UX)
    t.run(150)
    _, _, _, du = t.moments()
    h = 1e-4
    _, up = oracle_run(c, 150, wall_u=(0.1 + h, 0.0))
    _, um = oracle_run(c, 150, wall_u=(0.1 - h, 0.0))
    fd = (up - um) / (2 * h)
    assert np.linalg.norm(du - fd) < RTOL * np.linalg.norm(fd)


def test_body_force_derivative_of_the_channel_field():
    c = C.poiseuille(48, 24, op=C.BGK, nu=0.05, u_max=0.05)
    F0 = float(np.asarray(c["force"])[0].flat[0])
    t = tangent_of(c, lbmx.TANGENT_BODY_FX)
    t.run(300)
    _, _, _, du = t.moments()
    h = 1e-3 * F0
    _, up = oracle_run(c, 300, body_fx=F0 + h)
    _, um = oracle_run(c, 300, body_fx=F0 - h)
    fd = (up - um) / (2 * h)
    assert np.linalg.norm(du - fd) < RTOL * np.linalg.norm(fd)


def test_tangent_rejects_what_it_does_not_differentiate():
    c = cylinder()
    with pytest.raises(lbmx.LbmxError) as e:
        lbmx.Tangent(c["nx"], c["ny"], lbmx.TANGENT_U_BC, op=C.CM_OPT, flags=c["flags"])
    assert e.value.code == 6
    zg = C.channel(64, 32, outlet="zg")
    with pytest.raises(lbmx.LbmxError) as e:
        lbmx.Tangent(64, 32, lbmx.TANGENT_U_BC, flags=zg["flags"])
    assert e.value.code == 6
    with pytest.raises(lbmx.LbmxError) as e:
        lbmx.Tangent(64, 32, 7)
    assert e.value.code == 1
    t = lbmx.Tangent(64, 32, lbmx.TANGENT_OMEGA)
    with pytest.raises(lbmx.LbmxError) as e:
        t.run(1)  # no state yet
    assert e.value.code == 5
