"""FP64 host adjoint of the D2Q9 step (test infrastructure only).

The engine's discrete adjoint (lbmx_adjoint_*) is checked against this: the
same objective and the same step, restated in FP64 on the host and
differentiated in reverse mode by torch autograd (CPU, float64), so the
whole gradient -- dJ/dgamma at every node, dJ/domega, dJ/dF -- comes from
one backward pass of an FP64 model, with no difference quotient.

The forward model restates oracle/lbm_oracle.c's one_step (the oracle's
own FP64 arithmetic forms) for the configuration the engine's adjoint
supports: BGK, MRT, CM<NoAdapter> and CM<OptimalAdapter>; a uniform body
force and the Brinkman term; periodic edges or half-way (moving) bounce-back
walls on the non-periodic ones, so every slot is written every step.  The
objective is J = sum over steps t >= first of sum_x w . (rho, rho ux, rho uy)
with the force-corrected velocity -- or, for the Brinkman-drag objective,
the same weights times the node's gamma.  tests/ pin the model to the
oracle: its J equals the oracle's to 1e-12 relative.

Follows (oracle file:line): streaming and half-way walls lbm_oracle.c
one_step; collide_bgk, collide_mrt, collide_cm; the reference files they
cite (BGK.cuh:13-51, MRT.cu:4-76, CM.cuh:27-138, adapters.cuh:48-111,
macroscopics.cu:4-38, 98-110, equilibrium.cu:3-39).
"""
import numpy as np

BGK, MRT, CM, CM_OPT = 0, 1, 2, 3
FLUID, MOVING_WALL_BB, HALFWAY_BB = 0, 32, 35
CX = [0, 1, 0, -1, 0, 1, -1, -1, 1]
CY = [0, 0, 1, 0, -1, 1, 1, -1, -1]
OPP = [0, 3, 4, 1, 2, 7, 8, 5, 6]
W = [4.0 / 9.0] + [1.0 / 9.0] * 4 + [1.0 / 36.0] * 4
MM = [[1, 1, 1, 1, 1, 1, 1, 1, 1],
      [-4, -1, -1, -1, -1, 2, 2, 2, 2],
      [4, -2, -2, -2, -2, 1, 1, 1, 1],
      [0, 1, 0, -1, 0, 1, -1, -1, 1],
      [0, -2, 0, 2, 0, 1, -1, -1, 1],
      [0, 0, 1, 0, -1, 1, 1, -1, -1],
      [0, 0, -2, 0, 2, 1, 1, -1, -1],
      [0, 1, -1, 1, -1, 0, 0, 0, 0],
      [0, 0, 0, 0, 0, 1, -1, 1, -1]]


def _feq(torch, rho, ux, uy):
    out = []
    uu = ux * ux + uy * uy
    for q in range(9):
        cu = CX[q] * ux + CY[q] * uy
        out.append((W[q] * rho) * (1.0 + 4.5 * cu * cu - 1.5 * uu + 3.0 * cu))
    return torch.stack(out)


class Model:
    """The step of one configuration; `objective(gamma, omega, fx, fy)` runs
    `steps` steps from the initial state and returns J as a float64 tensor
    (differentiable in every argument)."""

    def __init__(self, nx, ny, op, S, omega, flags, periodic, rho0, u0, weights, first, steps,
                 wall_u=(0.0, 0.0), drag=False):
        import torch
        self.torch = torch
        self.nx, self.ny, self.op = nx, ny, op
        self.S0 = [float(s) for s in S]
        self.omega0 = float(omega)
        # S entries equal to omega move with it (lbmx_adjoint's omega_mask)
        self.tied = [op != BGK and np.float32(s) == np.float32(omega) for s in S]
        self.periodic = periodic
        fl = np.asarray(flags)
        self.halfway = torch.tensor(np.isin(fl, (MOVING_WALL_BB, HALFWAY_BB)))
        self.moving = torch.tensor(fl == MOVING_WALL_BB)
        for q in range(1, 9):
            bad = self._outside(q) & ~self.halfway
            if bool(bad.any()):
                raise ValueError("a fluid node reads population %d from outside the lattice" % q)
        self.rho0 = torch.tensor(np.asarray(rho0, np.float64))
        self.u0 = torch.tensor(np.asarray(u0, np.float64))
        self.w = torch.tensor(np.asarray(weights, np.float64))
        self.first, self.steps = int(first), int(steps)
        self.wall_u = wall_u
        self.drag = drag
        self.M = torch.tensor(np.array(MM, np.float64))
        nrm = (self.M * self.M).sum(dim=1)
        self.Minv = (self.M / nrm[:, None]).T.contiguous()

    def _outside(self, q):
        """Nodes whose upstream node x - c_q lies outside a non-periodic lattice."""
        torch = self.torch
        y = torch.arange(self.ny)[:, None].expand(self.ny, self.nx)
        x = torch.arange(self.nx)[None, :].expand(self.ny, self.nx)
        sx, sy = x - CX[q], y - CY[q]
        out = torch.zeros(self.ny, self.nx, dtype=torch.bool)
        if not self.periodic[0]:
            out |= (sx < 0) | (sx >= self.nx)
        if not self.periodic[1]:
            out |= (sy < 0) | (sy >= self.ny)
        return out

    def _stream(self, f):
        """Post-stream populations (the oracle's push, written as a pull):
        from the upstream node, or, where that lies outside, the node's own
        reflected population minus the moving-wall term."""
        torch = self.torch
        out = []
        for q in range(9):
            v = torch.roll(f[q], shifts=(CY[q], CX[q]), dims=(0, 1))
            o = self._outside(q)
            if q and bool(o.any()):
                p = OPP[q]
                cu = CX[p] * self.wall_u[0] + CY[p] * self.wall_u[1]
                term = torch.where(self.moving, torch.full_like(v, 6.0 * W[p] * cu), torch.zeros_like(v))
                v = torch.where(o, f[p] - term, v)
            out.append(v)
        return torch.stack(out)

    def objective(self, gamma, omega, fx, fy):
        torch = self.torch
        S = [omega if t else torch.tensor(s, dtype=torch.float64) for s, t in zip(self.S0, self.tied)]
        f = _feq(torch, self.rho0, self.u0[0], self.u0[1])
        n = self.nx * self.ny
        J = torch.zeros((), dtype=torch.float64)
        cx = torch.tensor(CX, dtype=torch.float64)[:, None, None]
        cy = torch.tensor(CY, dtype=torch.float64)[:, None, None]
        for t in range(1, self.steps + 1):
            f = self._stream(f)
            r = f.sum(dim=0)
            jx = (f * cx).sum(dim=0)
            jy = (f * cy).sum(dim=0)
            inv = 1.0 / r
            ux = jx * inv + 0.5 * fx / r
            uy = jy * inv + 0.5 * fy / r
            Fx = fx * torch.ones_like(r)
            Fy = fy * torch.ones_like(r)
            if gamma is not None:
                sc = 1.0 / (0.5 * gamma + 1.0)
                ux = ux * sc
                uy = uy * sc
                Fx = Fx - gamma * r * ux
                Fy = Fy - gamma * r * uy
            if t >= self.first:
                term = self.w[0] * r + self.w[1] * r * ux + self.w[2] * r * uy
                J = J + ((gamma * term) if self.drag else term).sum()
            if self.op == BGK:
                f = self._bgk(f, r, ux, uy, Fx, Fy, omega)
            elif self.op == MRT:
                f = self._mrt(f, r, ux, uy, Fx, Fy, S)
            else:
                avg = None
                if self.op == CM_OPT:
                    pxx = f[1] + f[3] + f[5] + f[6] + f[7] + f[8]
                    pyy = f[2] + f[4] + f[5] + f[6] + f[7] + f[8]
                    pxy = f[5] - f[6] + f[7] - f[8]
                    pim = torch.sqrt(pxx * pxx + 2.0 * pxy * pxy + pyy * pyy)
                    avg = (r.sum() / n, (r * torch.sqrt(ux * ux + uy * uy)).sum() / n, pim.sum() / n)
                f = self._cm(f, r, ux, uy, Fx, Fy, S, avg)
        return J

    def _bgk(self, f, r, ux, uy, Fx, Fy, om):
        torch = self.torch
        feq = _feq(torch, r, ux, uy)
        cs2 = 1.0 / 3.0
        out = []
        for q in range(9):
            c1, c2 = float(CX[q]), float(CY[q])
            cu = c1 * ux + c2 * uy
            ft = W[q] * ((1.0 - 0.5 * om) * ((c1 - ux) / cs2 + cu * c1 / (cs2 * cs2)) * Fx
                         + (1.0 - 0.5 * om) * ((c2 - uy) / cs2 + cu * c2 / (cs2 * cs2)) * Fy)
            out.append(f[q] - om * (f[q] - feq[q]) + ft)
        return torch.stack(out)

    def _mrt(self, f, r, ux, uy, Fx, Fy, S):
        torch = self.torch
        feq = _feq(torch, r, ux, uy)
        fu = Fx * ux + Fy * uy
        F = [torch.zeros_like(r), 6.0 * fu, -6.0 * fu, Fx, -Fx, Fy, -Fy, 2.0 * (Fx * ux - Fy * uy), Fx * uy + Fy * ux]
        m = torch.einsum("ki,iyx->kyx", self.M, f)
        me = torch.einsum("ki,iyx->kyx", self.M, feq)
        mp = torch.stack([m[k] - S[k] * (m[k] - me[k]) + (1.0 - S[k] / 2.0) * F[k] for k in range(9)])
        return torch.einsum("ki,iyx->kyx", self.Minv, mp)

    def _cm(self, f, r, ux, uy, Fx, Fy, S, avg):
        torch = self.torch
        ks = [torch.zeros_like(r) for _ in range(8)]
        pi = [torch.zeros_like(r) for _ in range(3)]
        for i in range(9):
            ccx, ccy = CX[i] - ux, CY[i] - uy
            ccx2, ccy2 = ccx * ccx, ccy * ccy
            fi = f[i]
            ks[0] = ks[0] + fi * ccx
            ks[1] = ks[1] + fi * ccy
            ks[2] = ks[2] + fi * (ccx2 + ccy2)
            ks[3] = ks[3] + fi * (ccx2 - ccy2)
            ks[4] = ks[4] + fi * ccx * ccy
            ks[5] = ks[5] + fi * ccx2 * ccy
            ks[6] = ks[6] + fi * ccx * ccy2
            ks[7] = ks[7] + fi * ccx2 * ccy2
            pi[0] = pi[0] + fi * float(CX[i] * CX[i])
            pi[1] = pi[1] + fi * float(CX[i] * CY[i])
            pi[2] = pi[2] + fi * float(CY[i] * CY[i])
        k = [r] + ks
        cs2 = 1.0 / 3.0
        zero = torch.zeros_like(r)
        keq = [r, zero, zero, 2.0 * r * cs2, zero, zero, zero, zero, r * cs2 * cs2]
        F = [zero, Fx, Fy, zero, zero, zero, Fy * cs2, Fx * cs2, zero]
        hor = None
        if avg is not None:
            pimag = torch.sqrt(pi[0] * pi[0] + 2.0 * pi[1] * pi[1] + pi[2] * pi[2])
            jmag = torch.sqrt(ux * ux + uy * uy) * r
            # the oracle's constants are the float32 literals of adapters.cuh:77
            ts = (np.float64(np.float32(0.0003)) * (r / avg[0]) + np.float64(np.float32(-0.00775)) * (jmag / avg[1])
                  + np.float64(np.float32(0.00016)) * (pimag / avg[2]) + np.float64(np.float32(0.0087)))
            ts = torch.where(ts > 0.0, ts, torch.full_like(ts, float(np.float32(0.005))))
            ts = torch.where(ts < float(np.float32(1.5)), ts, torch.full_like(ts, float(np.float32(1.5))))
            hor = 1.0 / (3.0 * ts + 0.5)
        kp = []
        for i in range(9):
            s = hor if (hor is not None and i > 5) else S[i]
            kp.append(k[i] - s * (k[i] - keq[i]) + (1.0 - 0.5 * s) * F[i])
        c00, c10, c01 = kp[0], kp[1], kp[2]
        c20, c02 = (kp[3] + kp[4]) * 0.5, (kp[3] - kp[4]) * 0.5
        c11, c21, c12, c22 = kp[5], kp[6], kp[7], kp[8]
        m00 = c00
        m10 = c10 + ux * c00
        m01 = c01 + uy * c00
        m20 = c20 + 2.0 * ux * c10 + ux * ux * c00
        m02 = c02 + 2.0 * uy * c01 + uy * uy * c00
        m11 = c11 + ux * c01 + uy * c10 + ux * uy * c00
        m21 = c21 + 2.0 * ux * c11 + uy * c20 + ux * ux * c01 + 2.0 * ux * uy * c10 + ux * ux * uy * c00
        m12 = c12 + 2.0 * uy * c11 + ux * c02 + uy * uy * c10 + 2.0 * ux * uy * c01 + ux * uy * uy * c00
        m22 = (c22 + 2.0 * ux * c12 + 2.0 * uy * c21 + ux * ux * c02 + uy * uy * c20 + 4.0 * ux * uy * c11
               + 2.0 * ux * uy * uy * c10 + 2.0 * ux * ux * uy * c01 + ux * ux * uy * uy * c00)
        out = [None] * 9
        out[0] = m00 - m20 - m02 + m22
        out[1] = 0.5 * (m10 + m20 - m12 - m22)
        out[3] = 0.5 * (-m10 + m20 + m12 - m22)
        out[2] = 0.5 * (m01 + m02 - m21 - m22)
        out[4] = 0.5 * (-m01 + m02 + m21 - m22)
        out[5] = 0.25 * (m11 + m21 + m12 + m22)
        out[6] = 0.25 * (-m11 + m21 - m12 + m22)
        out[7] = 0.25 * (m11 - m21 - m12 + m22)
        out[8] = 0.25 * (-m11 - m21 + m12 + m22)
        return torch.stack(out)

    def gradient(self, gamma, omega, fx, fy):
        """(J, dJ/dgamma [ny, nx], dJ/domega, dJ/dFx, dJ/dFy) in FP64."""
        torch = self.torch
        g = torch.tensor(np.asarray(gamma, np.float64), requires_grad=True)
        om = torch.tensor(float(omega), dtype=torch.float64, requires_grad=True)
        Fx = torch.tensor(float(fx), dtype=torch.float64, requires_grad=True)
        Fy = torch.tensor(float(fy), dtype=torch.float64, requires_grad=True)
        J = self.objective(g, om, Fx, Fy)
        J.backward()
        return float(J.detach()), g.grad.numpy().copy(), float(om.grad), float(Fx.grad), float(Fy.grad)
