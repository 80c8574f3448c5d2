"""Seeded test cases shared by the parity tests, smoke() and bench.py.

Each builder returns a dict with the lattice parameters (the same keys the
engine binding and the oracle take), the boundary flags and the initial
fields.  The configurations restate the reference's 2-D scenarios
(src/scenarios/{taylorGreen,lidDrivenCavity,poiseuille,flowPastCylinder})
at sizes the CPU oracle runs in seconds.
"""
import numpy as np

BGK, MRT, CM, CM_OPT = 0, 1, 2, 3
FLUID, BOUNCE_BACK, ZOU_HE_TOP, ZOU_HE_LEFT = 0, 1, 2, 3
CYLINDER, ZG_OUTFLOW, PRESSURE_OUTLET, REGULARIZED_INLET_TOP = 6, 7, 8, 9
REGULARIZED_BOUNCE_BACK, REGULARIZED_BOUNCE_BACK_CORNER = 11, 12
MOVING_WALL_BB, ZOU_HE_PRESSURE_RIGHT, ZOU_HE_PARABOLIC_LEFT, HALFWAY_BB = 32, 33, 34, 35
CORNER_TOP_LEFT, CORNER_BOTTOM_LEFT = 36, 37
QUIRKS_REFERENCE = 0x1F


def omega_of(nu):
    """tau = 3 nu + 1/2 (viscosity_to_tau, src/core/lbm_constants.cuh:364-366)."""
    return 1.0 / (3.0 * nu + 0.5)


def mrt_S(omega):
    """The reference's MRT rate set (taylorGreenScenario.cuh:32-42, lidDrivenCavityScenario.cuh:62-72)."""
    return [0.0, 1.0, 1.4, 0.0, 1.2, 0.0, 1.9, omega, omega]


def cm_S(omega):
    """Central-moment rates of the reference scenarios (lidDrivenCavityScenario.cuh:50-60)."""
    return [0.0, 0.0, 0.0, 1.0, omega, omega, 1.0, 1.0, 1.0]


def S_for(op, omega):
    return mrt_S(omega) if op == MRT else (cm_S(omega) if op in (CM, CM_OPT) else [omega] * 9)


def base(nx, ny, op, nu, **kw):
    om = omega_of(nu)
    c = dict(nx=nx, ny=ny, op=op, omega=om, S=S_for(op, om), periodic=(False, False), quirks=0,
             u_bc=0.0, wall_u=(0.0, 0.0), rho_out=1.0, flags=np.zeros((ny, nx), np.uint8),
             rho=np.ones((ny, nx)), u=np.zeros((2, ny, nx)), force=None, markers=None)
    c.update(kw)
    return c


def taylor_green(nx=64, ny=48, op=BGK, nu=0.01, u0=0.04, **kw):
    """Decaying vortex, fully periodic: u = u0 sin kx cos ky, v = -u0 cos kx sin ky."""
    kx, ky = 2 * np.pi / nx, 2 * np.pi / ny
    X, Y = np.meshgrid(np.arange(nx), np.arange(ny))
    ux = u0 * np.sin(kx * X) * np.cos(ky * Y)
    uy = -u0 * (kx / ky) * np.cos(kx * X) * np.sin(ky * Y)
    rho = 1.0 - 3.0 * (u0 ** 2 / 4.0) * (np.cos(2 * kx * X) + np.cos(2 * ky * Y))
    return base(nx, ny, op, nu, periodic=(True, True), rho=rho, u=np.stack([ux, uy]), **kw)


def cavity_regularized(nx=48, ny=40, op=BGK, nu=0.02, u_lid=0.1, **kw):
    """The reference's lid-driven cavity flags (lidDrivenCavityFunctors.cuh:41-56)."""
    fl = np.zeros((ny, nx), np.uint8)
    fl[0, :] = REGULARIZED_BOUNCE_BACK
    fl[:, 0] = REGULARIZED_BOUNCE_BACK
    fl[:, -1] = REGULARIZED_BOUNCE_BACK
    fl[-1, :] = REGULARIZED_INLET_TOP
    for y, x in ((0, 0), (0, nx - 1), (ny - 1, 0), (ny - 1, nx - 1)):
        fl[y, x] = REGULARIZED_BOUNCE_BACK_CORNER
    return base(nx, ny, op, nu, flags=fl, u_bc=u_lid, **kw)


def cavity_moving_wall(nx=48, ny=40, op=MRT, nu=0.02, u_lid=0.1, **kw):
    """Cavity with a half-way moving-wall lid and half-way bounce-back walls."""
    fl = np.full((ny, nx), FLUID, np.uint8)
    fl[0, :] = HALFWAY_BB
    fl[:, 0] = HALFWAY_BB
    fl[:, -1] = HALFWAY_BB
    fl[-1, 1:-1] = MOVING_WALL_BB
    return base(nx, ny, op, nu, flags=fl, wall_u=(u_lid, 0.0), **kw)


def cavity_zouhe(nx=40, ny=32, op=BGK, nu=0.05, u_lid=0.05, **kw):
    fl = np.zeros((ny, nx), np.uint8)
    fl[0, :] = BOUNCE_BACK
    fl[:, 0] = BOUNCE_BACK
    fl[:, -1] = BOUNCE_BACK
    fl[-1, 1:-1] = ZOU_HE_TOP
    return base(nx, ny, op, nu, flags=fl, u_bc=u_lid, **kw)


def poiseuille(nx=64, ny=32, op=BGK, nu=1.0 / 6.0, u_max=0.05, **kw):
    """Body-force channel, periodic x, bounce-back walls (poiseuilleFunctors.cuh:34-57)."""
    fl = np.zeros((ny, nx), np.uint8)
    fl[0, :] = BOUNCE_BACK
    fl[-1, :] = BOUNCE_BACK
    F = np.zeros((2, ny, nx))
    F[0] = 8.0 * nu * u_max / (ny * ny)
    return base(nx, ny, op, nu, periodic=(True, False), flags=fl, force=F, **kw)


def cylinder_markers(cx, cy, r, n):
    """create_cylinder (src/IBM/IBM_generators.cu:5-25): n evenly spaced ring markers."""
    a = 2 * np.pi / n
    i = np.arange(n)
    return np.stack([cx + r * np.cos(i * a), cy + r * np.sin(i * a)], axis=1).astype(np.float32)


def channel(nx=96, ny=48, op=BGK, nu=0.04, u_in=0.05, inlet="zouhe", outlet="zg", markers=None, **kw):
    """Flow past a cylinder channel (flowPastCylinderFunctors.cuh:62-93)."""
    fl = np.zeros((ny, nx), np.uint8)
    fl[:, 0] = {"zouhe": ZOU_HE_LEFT, "parabolic": ZOU_HE_PARABOLIC_LEFT}[inlet]
    fl[:, -1] = {"zg": ZG_OUTFLOW, "pressure": PRESSURE_OUTLET, "zouhe_p": ZOU_HE_PRESSURE_RIGHT}[outlet]
    fl[0, :] = BOUNCE_BACK
    fl[-1, :] = BOUNCE_BACK
    return base(nx, ny, op, nu, flags=fl, u_bc=u_in, markers=markers, **kw)


def random_state(c, seed=0, amp=0.02):
    """Perturb the initial velocity with seeded noise (exercises every population)."""
    rng = np.random.default_rng(seed)
    c = dict(c)
    c["u"] = c["u"] + amp * rng.standard_normal(c["u"].shape)
    c["rho"] = c["rho"] * (1.0 + 0.01 * rng.standard_normal(c["rho"].shape))
    return c


def make_oracle(c, precision="f64"):
    import oracle as O
    o = O.Oracle(c["nx"], c["ny"], op=c["op"], omega=c["omega"], S=c["S"], periodic=c["periodic"],
                 quirks=c["quirks"], u_bc=c["u_bc"], wall_u=c["wall_u"], rho_out=c["rho_out"],
                 precision=precision)
    o.set_flags(c["flags"])
    n = c["nx"] * c["ny"]
    F = np.zeros(2 * n) if c["force"] is None else c["force"]
    o.init(c["rho"], c["u"], F)
    if c["markers"] is not None:
        o.set_markers(c["markers"])
    return o


def make_lattice(c, storage=0, options=0, stream=None):
    import lbmx
    L = lbmx.Lattice(c["nx"], c["ny"], op=c["op"], omega=c["omega"], S=c["S"], periodic=c["periodic"],
                     storage=storage, quirks=c["quirks"], options=options, u_bc=c["u_bc"],
                     wall_u=c["wall_u"], rho_out=c["rho_out"], stream=stream)
    L.set_flags(c["flags"])
    L.init(np.asarray(c["rho"], np.float32), np.asarray(c["u"], np.float32),
           None if c["force"] is None else np.asarray(c["force"], np.float32))
    if c["markers"] is not None:
        L.set_markers(c["markers"])
    return L


def ensemble(count=512, seed=0, sides=tuple(range(64, 769, 32)), re_range=(100.0, 5000.0), u_lid=0.1):
    """The batched-ensemble workload: `count` lid-driven cavities, side lengths
    drawn uniformly from {64, 96, ..., 768} and Reynolds numbers log-uniform in
    [100, 5000] (numpy PCG64, seed 0); nu = u_lid * side / Re."""
    rng = np.random.default_rng(seed)
    s = rng.choice(np.asarray(sides), size=count)
    re = np.exp(rng.uniform(np.log(re_range[0]), np.log(re_range[1]), size=count))
    return [(int(a), float(b), u_lid * float(a) / float(b)) for a, b in zip(s, re)]


def ensemble_cavity(side, nu, op=MRT, u_lid=0.1):
    """One cavity of the ensemble: rho = 1, u = 0, half-way walls, moving lid."""
    return cavity_moving_wall(side, side, op=op, nu=nu, u_lid=u_lid)


def splitmix64(z):
    """splitmix64 finaliser on a uint64 array (counter-based normal noise)."""
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def brinkman_field(nx, ny, sigma=16.0, seed=0):
    """Per-node solid fraction in [0, 1]: i.i.d. N(0, 1) per node from a
    splitmix64 counter hash (Box-Muller), Gaussian-blurred with sigma nodes
    (periodic in x, reflected in y), min-max scaled."""
    from scipy.ndimage import gaussian_filter
    i = np.arange(nx * ny, dtype=np.uint64) + np.uint64(seed) * np.uint64(2 * nx * ny)
    a = splitmix64(np.uint64(2) * i)
    b = splitmix64(np.uint64(2) * i + np.uint64(1))
    u1 = ((a >> np.uint64(11)).astype(np.float64) + 0.5) * 2.0 ** -53
    u2 = (b >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    z = (np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)).reshape(ny, nx)
    s = gaussian_filter(z, sigma, mode=("reflect", "wrap"))
    return ((s - s.min()) / (s.max() - s.min())).astype(np.float32)


def channel_brinkman(nx=64, ny=32, op=CM_OPT, nu=0.02, u_max=0.05, sigma=16.0, gamma_scale=1.0, seed=0, **kw):
    """Body-force Poiseuille channel with a Brinkman field: periodic x,
    half-way bounce-back walls at y = 0 and y = ny - 1 (the walls half a link
    outside), F_x = 8 nu u_max / ny^2 (poiseuilleFunctors.cuh:37)."""
    fl = np.zeros((ny, nx), np.uint8)
    fl[0, :] = HALFWAY_BB
    fl[-1, :] = HALFWAY_BB
    F = np.zeros((2, ny, nx))
    F[0] = 8.0 * nu * u_max / (ny * ny)
    c = base(nx, ny, op, nu, periodic=(True, False), flags=fl, force=F, **kw)
    c["gamma"] = gamma_scale * brinkman_field(nx, ny, sigma=sigma, seed=seed)
    return c
