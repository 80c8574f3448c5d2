"""Discrete adjoint (lbmx_adjoint_*): gradients of the outlet mass flux with
respect to the Brinkman field, omega and the body force.

The gradient is checked against central finite differences of the FP64
oracle's objective (the oracle restates the same step, Brinkman term
included) to 1e-3 relative, and against the FP64 host adjoint
(oracle/adjoint64.py: reverse-mode gradient of an FP64 restatement of the
oracle's step) node by node; the Brinkman-drag objective likewise; the
adjoint's forward model against the engine;
the checkpoint interval must not change the gradient; the autograd wrapper
must return the adjoint's gradient.
"""
import numpy as np
import pytest

import cases as C
import lbmx

pytestmark = pytest.mark.gpu

NX, NY, T, FIRST = 40, 20, 80, 41
RTOL = 1e-3


def case(op, gamma_scale=None):
    # starts from the developed Poiseuille profile (half-way walls half a link
    # outside rows 0 and NY-1), which the Brinkman field then slows down.
    # CM_OPT runs at gamma = 0: with drag, the OptimalAdapter's rate (a
    # regression in the node's |j| over the grid average, clamped where it
    # turns negative) makes this flow ill-conditioned -- FP32 and FP64 runs
    # part by 1e-4..1e-3 within 80 steps -- and a finite difference would
    # measure that, not the derivative.  The gamma gradient is still taken
    # (at gamma = 0).
    if gamma_scale is None:
        gamma_scale = 0.0 if op == C.CM_OPT else 0.3
    c = C.channel_brinkman(NX, NY, op=op, nu=0.02, u_max=0.05, sigma=3.0, gamma_scale=gamma_scale, seed=1)
    y = np.arange(NY) + 0.5
    c["u"] = c["u"].copy()
    c["u"][0] = (4.0 * 0.05 * y * (NY - y) / (NY * NY))[:, None]
    return c


def weights(c):
    # mass flux through the outlet column, averaged over steps FIRST..T
    w = np.zeros((3, c["ny"], c["nx"]), np.float32)
    w[1, :, c["nx"] - 1] = 1.0 / (T - FIRST + 1)
    return w


def make_adjoint(c, every=10):
    fx, fy = float(c["force"][0].flat[0]), float(c["force"][1].flat[0])
    a = lbmx.Adjoint(c["nx"], c["ny"], op=c["op"], omega=c["omega"], S=c["S"], periodic=c["periodic"],
                     flags=c["flags"], checkpoint_every=every, body_force=(fx, fy))
    a.set_state(np.asarray(c["rho"], np.float32), np.asarray(c["u"], np.float32))
    a.set_gamma(c["gamma"])
    a.set_objective(weights(c), FIRST)
    return a


def oracle_J(c, gamma, omega, fx, fy):
    import oracle as O
    o = O.Oracle(c["nx"], c["ny"], op=c["op"], omega=omega, S=C.S_for(c["op"], omega), periodic=c["periodic"],
                 precision="f64")
    o.set_flags(c["flags"])
    o.set_gamma(gamma)
    F = np.zeros((2, c["ny"], c["nx"]))
    F[0], F[1] = fx, fy
    o.init(c["rho"], c["u"], F)
    w = weights(c).astype(np.float64)
    J = 0.0
    for t in range(1, T + 1):
        o.step(1)
        if t >= FIRST:
            r, u, _ = o.moments()
            J += float((w[0] * r + w[1] * r * u[0] + w[2] * r * u[1]).sum())
    return J


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-30)


@pytest.mark.parametrize("op", [C.BGK, C.MRT, C.CM, C.CM_OPT])
def test_adjoint_forward_matches_engine_and_oracle(op):
    c = case(op, gamma_scale=0.3 if op != C.CM_OPT else 0.0)
    a = make_adjoint(c)
    J = a.forward(T)
    ra, ua = a.moments()
    o = C.make_oracle(c, precision="f32")
    o.set_gamma(c["gamma"])
    o.step(T)
    ro, uo, _ = o.moments()
    assert np.abs(ra - ro).max() < 2e-5 and np.abs(ua - uo).max() < 2e-5
    fx = float(c["force"][0].flat[0])
    # FP32 vs FP64 of a drag-damped flow: the flux has fallen to ~1% of its
    # start, so the bound is relative to the starting flux (~0.66)
    assert abs(J - oracle_J(c, c["gamma"].astype(np.float64), c["omega"], fx, 0.0)) < 1e-6
    # the engine's production step on the same case (20 steps: CM_OPT's
    # clamped rate lets rounding differences of the two paths grow later)
    a20 = make_adjoint(c)
    a20.forward(20)
    r20, u20 = a20.moments()
    L = C.make_lattice(c)
    L.set_brinkman(c["gamma"])
    L.step(20)
    rl, ul, _ = L.moments()
    assert np.abs(r20 - rl).max() < 2e-6 and np.abs(u20 - ul).max() < 2e-6


@pytest.mark.parametrize("op", [C.BGK, C.MRT, C.CM, C.CM_OPT])
def test_adjoint_gradient_matches_fp64_finite_differences(op):
    c = case(op)
    a = make_adjoint(c)
    a.forward(T)
    g_gamma, (g_om, g_fx, g_fy) = a.backward()
    om, fx = c["omega"], float(c["force"][0].flat[0])
    gam = c["gamma"].astype(np.float64)
    # omega
    h = 1e-4
    fd = (oracle_J(c, gam, om + h, fx, 0.0) - oracle_J(c, gam, om - h, fx, 0.0)) / (2 * h)
    assert rel(g_om, fd) < RTOL, (g_om, fd)
    # body force
    h = 1e-3 * fx
    fd = (oracle_J(c, gam, om, fx + h, 0.0) - oracle_J(c, gam, om, fx - h, 0.0)) / (2 * h)
    assert rel(g_fx, fd) < RTOL, (g_fx, fd)
    # Brinkman field along a smooth random direction; h = 1e-6 (FP64 keeps
    # ~1e-10 there): CM_OPT's clamped rate puts kinks in J close to the base
    # point, which a wider difference straddles
    d = C.brinkman_field(NX, NY, sigma=2.0, seed=7).astype(np.float64) - 0.5
    h = 1e-6
    fd = (oracle_J(c, gam + h * d, om, fx, 0.0) - oracle_J(c, gam - h * d, om, fx, 0.0)) / (2 * h)
    assert rel(float((g_gamma.astype(np.float64) * d).sum()), fd) < RTOL
    # and at single nodes (one inside the flow, one next to the wall)
    for (y, x) in ((NY // 2, NX // 3), (1, NX - 2)):
        e = np.zeros_like(gam)
        e[y, x] = 1.0
        fd = (oracle_J(c, gam + h * e, om, fx, 0.0) - oracle_J(c, gam - h * e, om, fx, 0.0)) / (2 * h)
        assert abs(g_gamma[y, x] - fd) < RTOL * max(abs(fd), 1e-3 * np.abs(g_gamma).max()), (y, x, g_gamma[y, x], fd)


def test_checkpoint_interval_leaves_the_gradient_unchanged():
    c = case(C.MRT)
    out = []
    for every in (1, 7, T):
        a = make_adjoint(c, every=every)
        a.forward(T)
        g, s = a.backward()
        out.append((g, s))
    for g, s in out[1:]:
        np.testing.assert_array_equal(g, out[0][0])
        assert s == out[0][1]


def test_autograd_wrapper_returns_the_adjoint_gradient():
    torch = pytest.importorskip("torch")
    import lbmx_autograd
    c = case(C.CM_OPT)
    a = make_adjoint(c)
    gamma = torch.tensor(c["gamma"], device="cuda", requires_grad=True)
    omega = torch.tensor(c["omega"], dtype=torch.float64, requires_grad=True)
    force = torch.tensor([float(c["force"][0].flat[0]), 0.0], dtype=torch.float64, requires_grad=True)
    J = lbmx_autograd.objective(gamma, omega, force, a, T)
    J.backward()
    b = make_adjoint(c)
    Jb = b.forward(T)
    g, (gw, gfx, gfy) = b.backward()
    assert abs(J.item() - Jb) <= 1e-12 * abs(Jb)
    np.testing.assert_array_equal(gamma.grad.cpu().numpy(), g)
    assert omega.grad.item() == gw and force.grad[0].item() == gfx and force.grad[1].item() == gfy


def test_adjoint_rejects_what_it_does_not_differentiate():
    c = case(C.BGK)
    bb = c["flags"].copy()
    bb[0, :] = C.BOUNCE_BACK  # reads populations from outside the domain at x = 0 and nx - 1
    with pytest.raises(lbmx.LbmxError) as e:
        lbmx.Adjoint(NX, NY, op=C.BGK, omega=c["omega"], periodic=(True, False), flags=bb)
    assert e.value.code == 6
    open_edge = c["flags"].copy()
    open_edge[0, :] = C.FLUID
    with pytest.raises(lbmx.LbmxError):
        lbmx.Adjoint(NX, NY, op=C.BGK, omega=c["omega"], periodic=(True, False), flags=open_edge)
    zg = c["flags"].copy()
    zg[:, 0] = C.ZG_OUTFLOW
    with pytest.raises(lbmx.LbmxError):
        lbmx.Adjoint(NX, NY, op=C.BGK, omega=c["omega"], periodic=(True, False), flags=zg)


def host_adjoint(c, drag=False):
    import adjoint64 as A
    m = A.Model(c["nx"], c["ny"], c["op"], c["S"], c["omega"], c["flags"], c["periodic"], c["rho"], c["u"],
                weights(c), FIRST, T, drag=drag)
    return m.gradient(c["gamma"].astype(np.float64), c["omega"], float(c["force"][0].flat[0]), 0.0)


# FP32 gradient against the FP64 one: per scalar, and over the gamma field
# as a whole (a component's error relative to the field's norm)
HOST_RTOL = {C.BGK: 2e-5, C.MRT: 2e-5, C.CM: 2e-5, C.CM_OPT: 1e-4}


@pytest.mark.parametrize("op", [C.BGK, C.MRT, C.CM, C.CM_OPT])
@pytest.mark.parametrize("drag", [False, True])
def test_adjoint_gradient_matches_the_fp64_host_adjoint(op, drag):
    c = case(op)
    a = make_adjoint(c)
    if drag:
        a.set_objective(weights(c), FIRST, kind=lbmx.OBJECTIVE_BRINKMAN_DRAG)
    J = a.forward(T)
    g, (g_om, g_fx, g_fy) = a.backward()
    J64, g64, om64, fx64, fy64 = host_adjoint(c, drag)
    tol = HOST_RTOL[op]
    print("op %d drag %d: J %.9e / %.9e, omega %.6e / %.6e, Fx %.6e / %.6e, |dg|/|g| %.2e" % (
        op, drag, J, J64, g_om, om64, g_fx, fx64, np.linalg.norm(g - g64) / np.linalg.norm(g64)))
    assert abs(J - J64) <= 1e-6 + 1e-5 * abs(J64)
    assert rel(g_om, om64) < tol and rel(g_fx, fx64) < tol
    assert abs(g_fy - fy64) <= tol * (abs(fy64) + abs(fx64))
    assert np.abs(g - g64).max() <= tol * np.linalg.norm(g64)
    assert np.linalg.norm(g - g64) <= tol * np.linalg.norm(g64)


def test_brinkman_drag_gradient_matches_fp64_finite_differences():
    """The drag objective's gamma gradient, explicit term included, against
    central differences of the FP64 oracle's drag sum gamma rho u_x."""
    import oracle as O
    c = case(C.MRT, gamma_scale=0.3)
    a = make_adjoint(c)
    a.set_objective(weights(c), FIRST, kind=lbmx.OBJECTIVE_BRINKMAN_DRAG)
    a.forward(T)
    g, _ = a.backward()
    w = weights(c).astype(np.float64)
    fx = float(c["force"][0].flat[0])

    def J(gam):
        o = O.Oracle(c["nx"], c["ny"], op=c["op"], omega=c["omega"], S=c["S"], periodic=c["periodic"],
                     precision="f64")
        o.set_flags(c["flags"])
        o.set_gamma(gam)
        F = np.zeros((2, c["ny"], c["nx"]))
        F[0] = fx
        o.init(c["rho"], c["u"], F)
        tot = 0.0
        for t in range(1, T + 1):
            o.step(1)
            if t >= FIRST:
                r, u, _ = o.moments()
                tot += float((gam * (w[0] * r + w[1] * r * u[0] + w[2] * r * u[1])).sum())
        return tot

    gam = c["gamma"].astype(np.float64)
    for (y, x) in ((NY // 2, NX - 1), (3, NX - 1), (NY // 2, 5)):
        e = np.zeros_like(gam)
        e[y, x] = 1.0
        h = 1e-6
        fd = (J(gam + h * e) - J(gam - h * e)) / (2 * h)
        assert abs(g[y, x] - fd) < RTOL * max(abs(fd), 1e-3 * np.abs(g).max()), (y, x, g[y, x], fd)
