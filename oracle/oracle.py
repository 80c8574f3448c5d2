"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle restates the reference D2Q9 step on the CPU (see lbm_oracle.h for
the file:line map).  Only tests/, __graft_entry__.smoke() and the CPU-baseline
leg of bench.py import this module; the product path never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")

BGK, MRT, CM, CM_OPT = 0, 1, 2, 3
QUIRK_REST_LAG, QUIRK_ZOUHE_LEFT, QUIRK_MRT_FORCE, QUIRK_IBM_2X2, QUIRK_IBM_CLAMP = 1, 2, 4, 8, 16
QUIRKS_REFERENCE = 0x1F


class Params(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("periodic_x", ctypes.c_int), ("periodic_y", ctypes.c_int),
        ("op", ctypes.c_int), ("quirks", ctypes.c_int),
        ("ibm_iters", ctypes.c_int), ("threads", ctypes.c_int),
        ("omega", ctypes.c_double), ("S", ctypes.c_double * 9),
        ("u_bc", ctypes.c_double), ("wall_ux", ctypes.c_double), ("wall_uy", ctypes.c_double),
        ("rho_out", ctypes.c_double), ("ibm_ds", ctypes.c_double),
    ]


def build():
    """Compile both oracle variants with the committed Makefile."""
    subprocess.check_call(["make", "-s", "-C", HERE], stdout=subprocess.DEVNULL)


_LIBS = {}


def _lib(precision):
    if precision not in _LIBS:
        path = os.path.join(BUILD, "liboracle%d.so" % (64 if precision == "f64" else 32))
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        P = ctypes.POINTER
        dp = P(ctypes.c_double)
        lib.lbo_create.restype = ctypes.c_void_p
        lib.lbo_create.argtypes = [P(Params)]
        lib.lbo_destroy.argtypes = [ctypes.c_void_p]
        lib.lbo_set_flags.argtypes = [ctypes.c_void_p, P(ctypes.c_uint8)]
        lib.lbo_init.argtypes = [ctypes.c_void_p, dp, dp, dp]
        lib.lbo_set_markers.argtypes = [ctypes.c_void_p, dp, ctypes.c_int]
        lib.lbo_set_gamma.argtypes = [ctypes.c_void_p, dp]
        lib.lbo_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.lbo_time.restype = ctypes.c_long
        lib.lbo_time.argtypes = [ctypes.c_void_p]
        lib.lbo_get_f.argtypes = [ctypes.c_void_p, dp]
        lib.lbo_get_moments.argtypes = [ctypes.c_void_p, dp, dp, dp]
        lib.lbo_get_avg.argtypes = [ctypes.c_void_p, dp]
        lib.lbo_get_marker.argtypes = [ctypes.c_void_p, dp, dp, dp]
        lib.lbo_get_sums.argtypes = [ctypes.c_void_p, dp]
        _LIBS[precision] = lib
    return _LIBS[precision]


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """One lattice advanced by the CPU restatement of the reference step."""

    def __init__(self, nx, ny, op=BGK, omega=1.0, S=None, periodic=(False, False), quirks=0,
                 u_bc=0.0, wall_u=(0.0, 0.0), rho_out=1.0, ibm_iters=3, ibm_ds=1.0,
                 precision="f64", threads=0):
        self.lib = _lib(precision)
        self.nx, self.ny, self.n = nx, ny, nx * ny
        p = Params()
        p.nx, p.ny = nx, ny
        p.periodic_x, p.periodic_y = int(periodic[0]), int(periodic[1])
        p.op, p.quirks, p.ibm_iters, p.threads = op, quirks, ibm_iters, threads
        p.omega = omega
        S = [omega] * 9 if S is None else S
        for i in range(9):
            p.S[i] = S[i]
        p.u_bc, p.wall_ux, p.wall_uy, p.rho_out, p.ibm_ds = u_bc, wall_u[0], wall_u[1], rho_out, ibm_ds
        self.h = self.lib.lbo_create(ctypes.byref(p))
        if not self.h:
            raise ValueError("oracle: invalid parameters")
        self.nm = 0

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.lbo_destroy(self.h)
            self.h = None

    def set_flags(self, flags):
        fl = np.ascontiguousarray(flags, dtype=np.uint8).reshape(-1)
        assert fl.size == self.n
        self.lib.lbo_set_flags(self.h, fl.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))

    def init(self, rho, u, force=None):
        rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(-1)
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        force = np.zeros(2 * self.n) if force is None else np.ascontiguousarray(force, dtype=np.float64).reshape(-1)
        self.lib.lbo_init(self.h, _dp(rho), _dp(u), _dp(force))

    def set_markers(self, xy):
        xy = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1)
        self.nm = xy.size // 2
        self.lib.lbo_set_markers(self.h, _dp(xy), self.nm)

    def set_gamma(self, gamma):
        if gamma is None:
            self.lib.lbo_set_gamma(self.h, None)
            return
        g = np.ascontiguousarray(gamma, dtype=np.float64).reshape(-1)
        assert g.size == self.n
        self.lib.lbo_set_gamma(self.h, _dp(g))

    def step(self, n=1):
        self.lib.lbo_step(self.h, int(n))

    @property
    def t(self):
        return self.lib.lbo_time(self.h)

    def populations(self):
        f = np.empty(9 * self.n)
        self.lib.lbo_get_f(self.h, _dp(f))
        return f.reshape(9, self.ny, self.nx)

    def moments(self):
        rho, u, F = np.empty(self.n), np.empty(2 * self.n), np.empty(2 * self.n)
        self.lib.lbo_get_moments(self.h, _dp(rho), _dp(u), _dp(F))
        return rho.reshape(self.ny, self.nx), u.reshape(2, self.ny, self.nx), F.reshape(2, self.ny, self.nx)

    def averages(self):
        a = np.empty(3)
        self.lib.lbo_get_avg(self.h, _dp(a))
        return a

    def sums(self):
        a = np.empty(3)
        self.lib.lbo_get_sums(self.h, _dp(a))
        return a

    def markers(self):
        u, r, F = np.empty(2 * self.nm), np.empty(self.nm), np.empty(2 * self.nm)
        self.lib.lbo_get_marker(self.h, _dp(u), _dp(r), _dp(F))
        return u.reshape(2, self.nm), r, F.reshape(2, self.nm)
