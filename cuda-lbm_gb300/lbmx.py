"""Python binding of liblbmx.so (the engine's C-ABI, include/lbmx.h).

A thin ctypes layer: it loads the in-tree shared library (built by
build.py) and mirrors the C entry points one to one.  Field arguments may be
numpy arrays (host memory) or torch tensors (host or CUDA memory); the
library copies with cudaMemcpyDefault either way.  There is no fallback:
if the library cannot be loaded, importing fails loudly.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("LBMX_LIBRARY") or os.path.join(HERE, "liblbmx.so")

# operators, storage, flags and quirks: the values of include/lbmx.h
BGK, MRT, CM, CM_OPT = 0, 1, 2, 3
F32, F16_OFFSET, BF16_OFFSET = 0, 1, 2
FLUID, BOUNCE_BACK, ZOU_HE_TOP, ZOU_HE_LEFT = 0, 1, 2, 3
CYLINDER, ZG_OUTFLOW, PRESSURE_OUTLET, REGULARIZED_INLET_TOP = 6, 7, 8, 9
REGULARIZED_INLET_LEFT, REGULARIZED_BOUNCE_BACK, REGULARIZED_BOUNCE_BACK_CORNER = 10, 11, 12
MOVING_WALL_BB, ZOU_HE_PRESSURE_RIGHT, ZOU_HE_PARABOLIC_LEFT, HALFWAY_BB = 32, 33, 34, 35
CORNER_TOP_LEFT, CORNER_BOTTOM_LEFT = 36, 37
QUIRK_REST_LAG, QUIRK_ZOUHE_LEFT, QUIRK_MRT_FORCE, QUIRK_IBM_2X2, QUIRK_IBM_CLAMP = 1, 2, 4, 8, 16
QUIRKS_REFERENCE = 0x1F
OPTION_LAGGED_AVERAGES = 1
OPTION_ROUND_NEAREST = 2
STEP_STORE_MOMENTS, STEP_CHECK_FINITE, STEP_SUMS, STEP_KINETIC_ENERGY = 1, 2, 4, 8

STATUS = {0: "OK", 1: "INVALID_ARGUMENT", 2: "OUT_OF_MEMORY", 3: "CUDA", 4: "INVALID_FLAGS",
          5: "NOT_INITIALIZED", 6: "UNSUPPORTED", 7: "NONFINITE", 8: "TOO_LARGE"}

EXPORTED = ["lbmx_version", "lbmx_params_default", "lbmx_create", "lbmx_destroy", "lbmx_set_flags",
            "lbmx_init_from_fields", "lbmx_set_force_field", "lbmx_set_brinkman", "lbmx_step", "lbmx_step_ex", "lbmx_moments", "lbmx_moment_sums_async", "lbmx_step_sums", "lbmx_step_forces", "lbmx_kinetic_energy",
            "lbmx_get_populations", "lbmx_averages", "lbmx_ibm_set_markers", "lbmx_ibm_forces", "lbmx_time",
            "lbmx_synchronize", "lbmx_last_error", "lbmx_moment_sums_noalloc", "lbmx_checkpoint_save",
            "lbmx_checkpoint_load", "lbmx_write_vti", "lbmx_batch_create", "lbmx_batch_destroy",
            "lbmx_batch_set_config", "lbmx_batch_get_config", "lbmx_batch_autotune", "lbmx_batch_step",
            "lbmx_batch_synchronize", "lbmx_batch_last_error", "lbmx_adjoint_create", "lbmx_adjoint_destroy",
            "lbmx_adjoint_set_state", "lbmx_adjoint_set_gamma", "lbmx_adjoint_set_scalars",
            "lbmx_adjoint_set_objective", "lbmx_adjoint_set_objective_ex", "lbmx_adjoint_forward", "lbmx_adjoint_backward", "lbmx_adjoint_moments",
            "lbmx_adjoint_last_error", "lbmx_tangent_create", "lbmx_tangent_destroy", "lbmx_tangent_set_state",
            "lbmx_tangent_set_markers", "lbmx_tangent_run", "lbmx_tangent_moments", "lbmx_tangent_time",
            "lbmx_tangent_last_error", "lbmx_set_slab", "lbmx_halo_get", "lbmx_halo_put",
            "lbmx_opt_partials", "lbmx_set_averages"]
# lbmx_adjoint_set_objective_ex kinds
OBJECTIVE_MOMENTS, OBJECTIVE_BRINKMAN_DRAG = 0, 1
# lbmx_tangent_create parameters
TANGENT_U_BC, TANGENT_OMEGA, TANGENT_BODY_FX, TANGENT_WALL_UX = 0, 1, 2, 3


class Params(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
        ("periodic_x", ctypes.c_int32), ("periodic_y", ctypes.c_int32),
        ("op", ctypes.c_int32), ("storage", ctypes.c_int32),
        ("quirks", ctypes.c_uint32), ("options", ctypes.c_uint32),
        ("ibm_iters", ctypes.c_int32), ("device", ctypes.c_int32),
        ("omega", ctypes.c_float), ("S", ctypes.c_float * 9),
        ("u_bc", ctypes.c_float), ("wall_ux", ctypes.c_float), ("wall_uy", ctypes.c_float),
        ("rho_out", ctypes.c_float), ("ibm_ds", ctypes.c_float),
        ("body_fx", ctypes.c_float), ("body_fy", ctypes.c_float),
        ("stream", ctypes.c_void_p),
    ]


class BatchConfig(ctypes.Structure):
    _fields_ = [("tile_w", ctypes.c_int32), ("tile_h", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32),
                ("chunk", ctypes.c_int32),
                ("graph_steps", ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class LbmxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("lbmx error %d (%s): %s" % (code, STATUS.get(code, "?"), msg))
        self.code = code


def load_library(path=LIB_PATH):
    """Load liblbmx.so and declare its signatures; raises OSError if absent."""
    lib = ctypes.CDLL(path)
    P, vp = ctypes.POINTER, ctypes.c_void_p
    fp, dp = P(ctypes.c_float), P(ctypes.c_double)
    lib.lbmx_version.restype = ctypes.c_int32
    lib.lbmx_params_default.argtypes = [P(Params)]
    lib.lbmx_create.argtypes = [P(Params), P(vp)]
    lib.lbmx_destroy.argtypes = [vp]
    lib.lbmx_set_flags.argtypes = [vp, vp]
    lib.lbmx_init_from_fields.argtypes = [vp, vp, vp, vp]
    lib.lbmx_set_force_field.argtypes = [vp, vp]
    lib.lbmx_set_brinkman.argtypes = [vp, vp]
    lib.lbmx_set_brinkman.restype = ctypes.c_int32
    lib.lbmx_step.argtypes = [vp, ctypes.c_int32]
    lib.lbmx_step_ex.argtypes = [vp, ctypes.c_int32, ctypes.c_uint32]
    lib.lbmx_moments.argtypes = [vp, vp, vp, dp]
    lib.lbmx_moment_sums_async.argtypes = [vp, vp]
    lib.lbmx_moment_sums_async.restype = ctypes.c_int32
    lib.lbmx_step_sums.argtypes = [vp, ctypes.c_int32, ctypes.c_uint32, vp]
    lib.lbmx_step_sums.restype = ctypes.c_int32
    lib.lbmx_set_slab.argtypes = [vp, ctypes.c_uint32, ctypes.c_int64, ctypes.c_int32]
    lib.lbmx_halo_get.argtypes = [vp, ctypes.c_int32, ctypes.c_uint32, vp]
    lib.lbmx_halo_put.argtypes = [vp, ctypes.c_int32, ctypes.c_uint32, vp]
    lib.lbmx_opt_partials.argtypes = [vp, P(ctypes.c_int64)]
    lib.lbmx_set_averages.argtypes = [vp, fp]
    for name in ("lbmx_set_slab", "lbmx_halo_get", "lbmx_halo_put", "lbmx_opt_partials", "lbmx_set_averages"):
        getattr(lib, name).restype = ctypes.c_int32
    lib.lbmx_step_forces.argtypes = [vp, ctypes.c_int32, ctypes.c_uint32, vp]
    lib.lbmx_step_forces.restype = ctypes.c_int32
    lib.lbmx_kinetic_energy.argtypes = [vp, vp]
    lib.lbmx_kinetic_energy.restype = ctypes.c_int32
    lib.lbmx_get_populations.argtypes = [vp, vp]
    lib.lbmx_averages.argtypes = [vp, fp]
    lib.lbmx_ibm_set_markers.argtypes = [vp, vp, ctypes.c_int32]
    lib.lbmx_ibm_forces.argtypes = [vp, fp, dp]
    lib.lbmx_time.restype = ctypes.c_int64
    lib.lbmx_time.argtypes = [vp]
    lib.lbmx_synchronize.argtypes = [vp]
    lib.lbmx_last_error.restype = ctypes.c_char_p
    lib.lbmx_last_error.argtypes = [vp]
    for name in ("lbmx_checkpoint_save", "lbmx_checkpoint_load", "lbmx_write_vti"):
        getattr(lib, name).restype = ctypes.c_int32
        getattr(lib, name).argtypes = [vp, ctypes.c_char_p]
    lib.lbmx_batch_create.argtypes = [P(vp), ctypes.c_int32, P(vp)]
    lib.lbmx_batch_destroy.argtypes = [vp]
    lib.lbmx_batch_set_config.argtypes = [vp, P(BatchConfig)]
    lib.lbmx_batch_get_config.argtypes = [vp, P(BatchConfig)]
    lib.lbmx_batch_autotune.argtypes = [vp, ctypes.c_int32, P(BatchConfig)]
    lib.lbmx_batch_step.argtypes = [vp, ctypes.c_int32, ctypes.c_uint32]
    lib.lbmx_batch_synchronize.argtypes = [vp]
    lib.lbmx_batch_last_error.restype = ctypes.c_char_p
    lib.lbmx_batch_last_error.argtypes = [vp]
    for name in ("lbmx_batch_create", "lbmx_batch_set_config", "lbmx_batch_get_config", "lbmx_batch_autotune",
                 "lbmx_batch_step", "lbmx_batch_synchronize"):
        getattr(lib, name).restype = ctypes.c_int32
    lib.lbmx_adjoint_create.argtypes = [P(Params), vp, ctypes.c_int32, P(vp)]
    lib.lbmx_adjoint_destroy.argtypes = [vp]
    lib.lbmx_adjoint_set_state.argtypes = [vp, vp, vp]
    lib.lbmx_adjoint_set_gamma.argtypes = [vp, vp]
    lib.lbmx_adjoint_set_scalars.argtypes = [vp, ctypes.c_float, ctypes.c_float, ctypes.c_float]
    lib.lbmx_adjoint_set_objective.argtypes = [vp, vp, ctypes.c_int32]
    lib.lbmx_adjoint_set_objective_ex.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_int32]
    lib.lbmx_adjoint_forward.argtypes = [vp, ctypes.c_int32, dp]
    lib.lbmx_adjoint_backward.argtypes = [vp, vp, dp]
    lib.lbmx_adjoint_moments.argtypes = [vp, vp, vp]
    lib.lbmx_adjoint_last_error.restype = ctypes.c_char_p
    lib.lbmx_adjoint_last_error.argtypes = [vp]
    lib.lbmx_tangent_create.argtypes = [P(Params), vp, ctypes.c_int32, P(vp)]
    lib.lbmx_tangent_destroy.argtypes = [vp]
    lib.lbmx_tangent_set_state.argtypes = [vp, vp, vp]
    lib.lbmx_tangent_set_markers.argtypes = [vp, vp, ctypes.c_int32]
    lib.lbmx_tangent_run.argtypes = [vp, ctypes.c_int32, vp]
    lib.lbmx_tangent_moments.argtypes = [vp, vp, vp, vp, vp]
    lib.lbmx_tangent_time.restype = ctypes.c_int64
    lib.lbmx_tangent_time.argtypes = [vp]
    lib.lbmx_tangent_last_error.restype = ctypes.c_char_p
    lib.lbmx_tangent_last_error.argtypes = [vp]
    for name in ("lbmx_adjoint_create", "lbmx_adjoint_set_state", "lbmx_adjoint_set_gamma", "lbmx_adjoint_set_scalars",
                 "lbmx_adjoint_set_objective", "lbmx_adjoint_set_objective_ex", "lbmx_adjoint_forward", "lbmx_adjoint_backward",
                 "lbmx_adjoint_moments"):
        getattr(lib, name).restype = ctypes.c_int32
    lib.lbmx_moment_sums_noalloc.restype = ctypes.c_int32
    lib.lbmx_moment_sums_noalloc.argtypes = [vp, vp, ctypes.c_int64, vp, vp]
    for name in ("lbmx_create", "lbmx_set_flags", "lbmx_init_from_fields", "lbmx_set_force_field",
                 "lbmx_step", "lbmx_step_ex", "lbmx_moments", "lbmx_get_populations", "lbmx_averages",
                 "lbmx_ibm_set_markers", "lbmx_ibm_forces", "lbmx_synchronize"):
        getattr(lib, name).restype = ctypes.c_int32
    return lib


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        _LIB = load_library()
    return _LIB


def _ptr(a, dtype):
    """Data pointer of a numpy array or torch tensor (host or CUDA), checked."""
    if a is None:
        return None, None
    if hasattr(a, "data_ptr"):  # torch tensor
        import torch
        want = {np.float32: torch.float32, np.uint8: torch.uint8, np.float64: torch.float64}[dtype]
        if a.dtype != want or not a.is_contiguous():
            a = a.to(want).contiguous()
        return a.data_ptr(), a
    a = np.ascontiguousarray(a, dtype=dtype)
    return a.ctypes.data, a


class Lattice:
    """One D2Q9 lattice on the GPU, driven through the C-ABI."""

    def __init__(self, nx, ny, op=BGK, omega=1.0, S=None, periodic=(False, False), storage=F32,
                 quirks=0, options=0, u_bc=0.0, wall_u=(0.0, 0.0), rho_out=1.0, ibm_iters=3, ibm_ds=1.0,
                 body_force=(0.0, 0.0), device=0, stream=None):
        self.lib = lib()
        p = Params()
        self.lib.lbmx_params_default(ctypes.byref(p))
        p.nx, p.ny = nx, ny
        p.periodic_x, p.periodic_y = int(bool(periodic[0])), int(bool(periodic[1]))
        p.op, p.storage, p.quirks, p.options = op, storage, quirks, options
        p.ibm_iters, p.device = ibm_iters, device
        p.omega = omega
        S = [omega] * 9 if S is None else S
        for i in range(9):
            p.S[i] = S[i]
        p.u_bc, p.wall_ux, p.wall_uy, p.rho_out, p.ibm_ds = u_bc, wall_u[0], wall_u[1], rho_out, ibm_ds
        p.body_fx, p.body_fy = body_force
        p.stream = stream
        self.params = p
        h = ctypes.c_void_p()
        rc = self.lib.lbmx_create(ctypes.byref(p), ctypes.byref(h))
        if rc != 0:
            raise LbmxError(rc, self.lib.lbmx_last_error(None).decode())
        self.h = h
        self.nx, self.ny, self.n = nx, ny, nx * ny
        self.nm = 0
        self.op = op
        self.elem_size = 4 if storage == F32 else 2

    def close(self):
        if getattr(self, "h", None):
            self.lib.lbmx_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc):
        if rc != 0:
            raise LbmxError(rc, self.lib.lbmx_last_error(self.h).decode())

    def set_flags(self, flags):
        p, keep = _ptr(flags, np.uint8)
        self._check(self.lib.lbmx_set_flags(self.h, p))

    def init(self, rho, u, force=None):
        pr, k1 = _ptr(rho, np.float32)
        pu, k2 = _ptr(u, np.float32)
        pf, k3 = _ptr(force, np.float32)
        self._check(self.lib.lbmx_init_from_fields(self.h, pr, pu, pf))

    def set_brinkman(self, gamma):
        pg, k = _ptr(gamma, np.float32)
        self._check(self.lib.lbmx_set_brinkman(self.h, pg))

    def set_force_field(self, force):
        pf, k = _ptr(force, np.float32)
        self._check(self.lib.lbmx_set_force_field(self.h, pf))

    def step(self, n=1, flags=STEP_STORE_MOMENTS):
        self._check(self.lib.lbmx_step_ex(self.h, int(n), int(flags)))

    # --- y-slabs (lbmx_set_slab, lbmx_halo_*, lbmx_opt_partials, lbmx_set_averages)
    def set_slab(self, ghost_mask, row_origin, whole_ny=0):
        self._check(self.lib.lbmx_set_slab(self.h, int(ghost_mask), int(row_origin), int(whole_ny)))

    def halo_get(self, row, plane_mask, buf):
        """Copy the stored slots of `row`, planes in plane_mask, into buf (a
        contiguous numpy array or torch tensor of the storage's element size)."""
        ptr = buf.data_ptr() if hasattr(buf, "data_ptr") else buf.ctypes.data
        self._check(self.lib.lbmx_halo_get(self.h, int(row), int(plane_mask), ptr))
        return buf

    def halo_put(self, row, plane_mask, buf):
        ptr = buf.data_ptr() if hasattr(buf, "data_ptr") else buf.ctypes.data
        self._check(self.lib.lbmx_halo_put(self.h, int(row), int(plane_mask), ptr))

    def opt_partials(self):
        out = (ctypes.c_int64 * 3)()
        self._check(self.lib.lbmx_opt_partials(self.h, out))
        return np.array(list(out), np.int64)

    def set_averages(self, avg3):
        a = (ctypes.c_float * 3)(*[float(v) for v in avg3])
        self._check(self.lib.lbmx_set_averages(self.h, a))

    def step_forces(self, n, flags=0, out=None):
        """n steps recording each step's drag and lift (lbmx_step_forces):
        an (n, 2) FP64 array.  `out` may be a pinned-host or CUDA torch
        tensor of n*2 doubles, which the IBM kernel writes directly; then
        the call returns without waiting and `out` is returned."""
        if out is None:
            res = np.zeros((int(n), 2), np.float64)
            self._check(self.lib.lbmx_step_forces(self.h, int(n), int(flags), res.ctypes.data))
            return res
        self._check(self.lib.lbmx_step_forces(self.h, int(n), int(flags), out.data_ptr()))
        return out

    def step_sums(self, n, flags=0):
        """n steps that reduce the FP64 sums of every step: an [n, 3] array of
        {rho, rho ux, rho uy}, [n, 4] with the kinetic energy when flags has
        STEP_KINETIC_ENERGY (lbmx_step_sums into pageable host memory)."""
        width = 4 if flags & STEP_KINETIC_ENERGY else 3
        out = np.zeros((int(n), width), np.float64)
        self._check(self.lib.lbmx_step_sums(self.h, int(n), int(flags), out.ctypes.data))
        self.synchronize()
        return out

    def kinetic_energy(self):
        """1/2 sum rho |u|^2 of the last step that reduced it (lbmx_kinetic_energy)."""
        v = ctypes.c_double()
        self._check(self.lib.lbmx_kinetic_energy(self.h, ctypes.byref(v)))
        return v.value

    def moments(self, rho=None, u=None):
        """(rho[ny,nx], u[2,ny,nx], sums[3]) of the last stored step, as numpy."""
        rho = np.empty((self.ny, self.nx), np.float32) if rho is None else rho
        u = np.empty((2, self.ny, self.nx), np.float32) if u is None else u
        s = (ctypes.c_double * 3)()
        pr, _ = _ptr(rho, np.float32) if not isinstance(rho, np.ndarray) else (rho.ctypes.data, rho)
        pu, _ = _ptr(u, np.float32) if not isinstance(u, np.ndarray) else (u.ctypes.data, u)
        self._check(self.lib.lbmx_moments(self.h, pr, pu, s))
        return rho, u, np.array(list(s))

    def populations(self):
        out = np.empty((9, self.ny, self.nx), np.float32)
        self._check(self.lib.lbmx_get_populations(self.h, out.ctypes.data))
        return out

    def averages(self):
        a = (ctypes.c_float * 3)()
        self._check(self.lib.lbmx_averages(self.h, a))
        return np.array(list(a))

    def set_markers(self, xy):
        p, k = _ptr(xy, np.float32)
        n = int(np.asarray(xy).size // 2) if not hasattr(xy, "numel") else int(xy.numel() // 2)
        self._check(self.lib.lbmx_ibm_set_markers(self.h, p, n))
        self.nm = n

    def marker_forces(self):
        F = np.zeros(2 * max(self.nm, 1), np.float32)
        dl = (ctypes.c_double * 2)()
        self._check(self.lib.lbmx_ibm_forces(self.h, F.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), dl))
        return F[: 2 * self.nm].reshape(2, self.nm), np.array(list(dl))

    def save(self, path):
        self._check(self.lib.lbmx_checkpoint_save(self.h, os.fsencode(path)))

    def load(self, path):
        self._check(self.lib.lbmx_checkpoint_load(self.h, os.fsencode(path)))

    def write_vti(self, path):
        self._check(self.lib.lbmx_write_vti(self.h, os.fsencode(path)))

    @property
    def t(self):
        return self.lib.lbmx_time(self.h)

    def synchronize(self):
        self._check(self.lib.lbmx_synchronize(self.h))


class Batch:
    """Many lattices advanced by one persistent launch per step (lbmx_batch_*).

    The lattices stay ordinary Lattice objects (read them as usual); they
    must outlive the batch."""

    def __init__(self, lattices):
        self.lib = lib()
        self.lattices = list(lattices)
        arr = (ctypes.c_void_p * len(self.lattices))(*[L.h.value for L in self.lattices])
        b = ctypes.c_void_p()
        rc = self.lib.lbmx_batch_create(arr, len(self.lattices), ctypes.byref(b))
        if rc != 0:
            raise LbmxError(rc, self.lib.lbmx_batch_last_error(None).decode())
        self.b = b

    def _check(self, rc):
        if rc != 0:
            raise LbmxError(rc, self.lib.lbmx_batch_last_error(self.b).decode())

    def close(self):
        if getattr(self, "b", None):
            self.lib.lbmx_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        self.close()

    @property
    def config(self):
        c = BatchConfig()
        self._check(self.lib.lbmx_batch_get_config(self.b, ctypes.byref(c)))
        return c.as_dict()

    def set_config(self, tile_w=128, tile_h=4, ctas_per_sm=3, chunk=1, graph_steps=16):
        c = BatchConfig(tile_w, tile_h, ctas_per_sm, chunk, graph_steps)
        self._check(self.lib.lbmx_batch_set_config(self.b, ctypes.byref(c)))

    def autotune(self, trial_steps=8):
        c = BatchConfig()
        self._check(self.lib.lbmx_batch_autotune(self.b, int(trial_steps), ctypes.byref(c)))
        return c.as_dict()

    def step(self, n=1, flags=STEP_STORE_MOMENTS):
        self._check(self.lib.lbmx_batch_step(self.b, int(n), int(flags)))

    def synchronize(self):
        self._check(self.lib.lbmx_batch_synchronize(self.b))


class Adjoint:
    """Discrete adjoint of the step (lbmx_adjoint_*): J over steps >= first of
    w_rho rho + w_x rho u_x + w_y rho u_y, and its gradient with respect to
    the Brinkman field gamma, omega and the body force."""

    def __init__(self, nx, ny, op=BGK, omega=1.0, S=None, periodic=(False, False), flags=None, checkpoint_every=1,
                 quirks=0, wall_u=(0.0, 0.0), body_force=(0.0, 0.0), device=0, stream=None):
        self.lib = lib()
        p = Params()
        self.lib.lbmx_params_default(ctypes.byref(p))
        p.nx, p.ny = nx, ny
        p.periodic_x, p.periodic_y = int(bool(periodic[0])), int(bool(periodic[1]))
        p.op, p.quirks, p.device, p.omega = op, quirks, device, omega
        S = [omega] * 9 if S is None else S
        for i in range(9):
            p.S[i] = S[i]
        p.wall_ux, p.wall_uy = wall_u
        p.body_fx, p.body_fy = body_force
        p.stream = stream
        fl = np.zeros((ny, nx), np.uint8) if flags is None else np.ascontiguousarray(flags, np.uint8)
        a = ctypes.c_void_p()
        rc = self.lib.lbmx_adjoint_create(ctypes.byref(p), fl.ctypes.data, int(checkpoint_every), ctypes.byref(a))
        if rc != 0:
            raise LbmxError(rc, self.lib.lbmx_adjoint_last_error(None).decode())
        self.a = a
        self.nx, self.ny, self.n = nx, ny, nx * ny

    def _check(self, rc):
        if rc != 0:
            raise LbmxError(rc, self.lib.lbmx_adjoint_last_error(self.a).decode())

    def close(self):
        if getattr(self, "a", None):
            self.lib.lbmx_adjoint_destroy(self.a)
            self.a = None

    def __del__(self):
        self.close()

    def set_state(self, rho, u):
        pr, k1 = _ptr(rho, np.float32)
        pu, k2 = _ptr(u, np.float32)
        self._check(self.lib.lbmx_adjoint_set_state(self.a, pr, pu))

    def set_gamma(self, gamma):
        pg, k = _ptr(gamma, np.float32)
        self._check(self.lib.lbmx_adjoint_set_gamma(self.a, pg))

    def set_scalars(self, omega, fx, fy):
        self._check(self.lib.lbmx_adjoint_set_scalars(self.a, float(omega), float(fx), float(fy)))

    def set_objective(self, weights, first_step, kind=OBJECTIVE_MOMENTS):
        pw, k = _ptr(weights, np.float32)
        if kind == OBJECTIVE_MOMENTS:
            self._check(self.lib.lbmx_adjoint_set_objective(self.a, pw, int(first_step)))
        else:
            self._check(self.lib.lbmx_adjoint_set_objective_ex(self.a, pw, int(first_step), int(kind)))

    def forward(self, nsteps):
        J = ctypes.c_double()
        self._check(self.lib.lbmx_adjoint_forward(self.a, int(nsteps), ctypes.byref(J)))
        return J.value

    def backward(self, grad_gamma=None):
        """(dJ/dgamma [ny, nx], (dJ/domega, dJ/dFx, dJ/dFy)); grad_gamma may be a
        float32 CUDA tensor to receive dJ/dgamma in place."""
        g3 = (ctypes.c_double * 3)()
        if grad_gamma is None:
            out = np.empty((self.ny, self.nx), np.float32)
            self._check(self.lib.lbmx_adjoint_backward(self.a, out.ctypes.data, g3))
        else:
            out = grad_gamma
            self._check(self.lib.lbmx_adjoint_backward(self.a, out.data_ptr(), g3))
        return out, tuple(g3)

    def moments(self):
        rho = np.empty((self.ny, self.nx), np.float32)
        u = np.empty((2, self.ny, self.nx), np.float32)
        self._check(self.lib.lbmx_adjoint_moments(self.a, rho.ctypes.data, u.ctypes.data))
        return rho, u


class Tangent:
    """Tangent-linear derivative of a run with respect to one scalar parameter
    (lbmx_tangent_*): TANGENT_U_BC, TANGENT_OMEGA, TANGENT_BODY_FX or
    TANGENT_WALL_UX.  run() returns per step (drag, lift, d drag, d lift)."""

    def __init__(self, nx, ny, parameter=TANGENT_U_BC, op=BGK, omega=1.0, S=None, periodic=(False, False),
                 flags=None, quirks=0, u_bc=0.0, wall_u=(0.0, 0.0), rho_out=1.0, body_force=(0.0, 0.0),
                 ibm_iters=3, device=0, stream=None):
        self.lib = lib()
        p = Params()
        self.lib.lbmx_params_default(ctypes.byref(p))
        p.nx, p.ny = nx, ny
        p.periodic_x, p.periodic_y = int(bool(periodic[0])), int(bool(periodic[1]))
        p.op, p.quirks, p.device, p.omega = op, quirks, device, omega
        S = [omega] * 9 if S is None else S
        for i in range(9):
            p.S[i] = S[i]
        p.u_bc, p.rho_out, p.ibm_iters = u_bc, rho_out, ibm_iters
        p.wall_ux, p.wall_uy = wall_u
        p.body_fx, p.body_fy = body_force
        p.stream = stream
        fl = np.zeros((ny, nx), np.uint8) if flags is None else np.ascontiguousarray(flags, np.uint8)
        t = ctypes.c_void_p()
        rc = self.lib.lbmx_tangent_create(ctypes.byref(p), fl.ctypes.data, int(parameter), ctypes.byref(t))
        if rc != 0:
            raise LbmxError(rc, self.lib.lbmx_tangent_last_error(None).decode())
        self.t = t
        self.nx, self.ny, self.n = nx, ny, nx * ny

    def _check(self, rc):
        if rc != 0:
            raise LbmxError(rc, self.lib.lbmx_tangent_last_error(self.t).decode())

    def close(self):
        if getattr(self, "t", None):
            self.lib.lbmx_tangent_destroy(self.t)
            self.t = None

    def __del__(self):
        self.close()

    def set_state(self, rho, u):
        pr, k1 = _ptr(rho, np.float32)
        pu, k2 = _ptr(u, np.float32)
        self._check(self.lib.lbmx_tangent_set_state(self.t, pr, pu))

    def set_markers(self, xy):
        xy = np.ascontiguousarray(xy, np.float32).reshape(-1, 2)
        self._check(self.lib.lbmx_tangent_set_markers(self.t, xy.ctypes.data, xy.shape[0]))

    def run(self, nsteps):
        series = np.zeros((int(nsteps), 4), np.float64)
        self._check(self.lib.lbmx_tangent_run(self.t, int(nsteps), series.ctypes.data))
        return series

    def moments(self):
        """(rho, u, drho, du) of the last step."""
        rho = np.empty((self.ny, self.nx), np.float32)
        u = np.empty((2, self.ny, self.nx), np.float32)
        drho = np.empty_like(rho)
        du = np.empty_like(u)
        self._check(self.lib.lbmx_tangent_moments(self.t, rho.ctypes.data, u.ctypes.data, drho.ctypes.data,
                                                  du.ctypes.data))
        return rho, u, drho, du

    @property
    def t_steps(self):
        return int(self.lib.lbmx_tangent_time(self.t))
