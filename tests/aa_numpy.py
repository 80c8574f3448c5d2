"""A numpy lattice with the engine's in-place (AA) slot layout, for testing
the y-slab exchange protocol (cuda-lbm_gb300/lbmx_slabs.py) on CPU ranks.

Test infrastructure.  It stores one buffer of slots F[q][y][x] exactly as the
engine does: after an even step (and after init) slot OPP(q) of node x holds
f*_q(x); an odd step reads slot OPP(q) of the upstream node x - c_q and
writes f*_q into slot q of the downstream node x + c_q; an even step reads
slot q of x and writes slot OPP(q) of x.  Collision is BGK in FP64, periodic
in x; rows are periodic in y unless the lattice is a slab with ghost rows,
which are never stepped.  In `averaged` mode the relaxation rate depends on
the grid-average density, summed in the engine's 2^-30 fixed point, so the
slabs must fold their integer partial sums exactly (lbmx_opt_partials /
lbmx_set_averages play that part on the engine).
"""
import numpy as np

CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1])
OPP = np.array([0, 3, 4, 1, 2, 7, 8, 5, 6])
W = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)


def equilibrium(rho, ux, uy):
    cu = CX[:, None, None] * ux + CY[:, None, None] * uy
    usq = ux * ux + uy * uy
    return W[:, None, None] * rho * (1 + 3 * cu + 4.5 * cu * cu - 1.5 * usq)


class AALattice:
    op = 0

    def __init__(self, rho, u, omega, ghost_mask=0, averaged=False, whole_nodes=None):
        ny, nx = rho.shape
        self.nx, self.ny, self.omega = nx, ny, omega
        self.elem_size = 8
        self.t = 0
        self.ghost_mask = ghost_mask
        self.owned = np.ones((ny, nx), bool)
        if ghost_mask & 1:
            self.owned[0] = False
        if ghost_mask & 2:
            self.owned[-1] = False
        self.averaged = averaged
        self.op = 3 if averaged else 0
        self.whole_nodes = whole_nodes if whole_nodes is not None else nx * ny
        self.ext_avg = None
        feq = equilibrium(np.asarray(rho, np.float64), np.asarray(u[0], np.float64), np.asarray(u[1], np.float64))
        self.F = np.empty((9, ny, nx))
        for q in range(9):
            self.F[OPP[q]] = feq[q]

    def _post_stream(self, parity):
        if parity:
            return np.stack([np.roll(self.F[OPP[q]], (CY[q], CX[q]), axis=(0, 1)) for q in range(9)])
        return self.F.copy()

    def _fixed_sum_rho(self, fin):
        rho = fin.sum(axis=0)
        return int(np.rint(rho[self.owned] * 2.0 ** 30).astype(np.int64).sum())

    def opt_partials(self):
        fin = self._post_stream((self.t + 1) & 1)
        return np.array([self._fixed_sum_rho(fin), 0, 0], np.int64)

    def set_averages(self, avg3):
        self.ext_avg = np.float32(avg3[0])

    def step(self, n=1, flags=None):
        for _ in range(int(n)):
            parity = (self.t + 1) & 1
            fin = self._post_stream(parity)
            rho = fin.sum(axis=0)
            ux = (CX[:, None, None] * fin).sum(axis=0) / rho
            uy = (CY[:, None, None] * fin).sum(axis=0) / rho
            om = self.omega
            if self.averaged:
                if self.ext_avg is not None:
                    avg = self.ext_avg
                else:
                    s = np.float64(self._fixed_sum_rho(fin)) * 2.0 ** -30
                    avg = np.float32(s / np.float64(self.whole_nodes))
                self.ext_avg = None
                om = self.omega * (1.0 + 0.5 * (np.float64(avg) - 1.0))
            fout = fin - om * (fin - equilibrium(rho, ux, uy))
            for q in range(9):
                if parity:
                    dst = np.roll(self.owned, (CY[q], CX[q]), axis=(0, 1))
                    self.F[q][dst] = np.roll(fout[q], (CY[q], CX[q]), axis=(0, 1))[dst]
                else:
                    self.F[OPP[q]][self.owned] = fout[q][self.owned]
            self.t += 1

    def _view(self, buf, count):
        a = buf.numpy() if hasattr(buf, "numpy") else np.asarray(buf)
        return a.view(np.float64)[:count]

    def halo_get(self, row, plane_mask, buf):
        qs = [q for q in range(9) if (plane_mask >> q) & 1]
        v = self._view(buf, len(qs) * self.nx)
        for i, q in enumerate(qs):
            v[i * self.nx:(i + 1) * self.nx] = self.F[q, row]
        return buf

    def halo_put(self, row, plane_mask, buf):
        qs = [q for q in range(9) if (plane_mask >> q) & 1]
        v = self._view(buf, len(qs) * self.nx)
        for i, q in enumerate(qs):
            self.F[q, row] = v[i * self.nx:(i + 1) * self.nx]

    def synchronize(self):
        pass
