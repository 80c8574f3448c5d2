"""Generate tests/golden/steady_cavity256_mrt.npz: the FP64 oracle's
lid-driven cavity (256 x 256, MRT, half-way walls, moving lid 0.1, Re 1000 on
the side, rho = 1 and u = 0 at the start) run to its steady state, as the
reference field for the storage forms' steady-state error.

Steady means: the relative L2 change of the velocity field over the last
1000 steps is at most 1e-6 (RESIDUAL).  The run advances 1000 steps at a
time until then (at most MAX_STEPS).

  u        velocity [2][64][64]: every 4th node in x and y (node 4j, 4i)
  u_prev   the same 1000 steps earlier (how far from steady the flow is)
  meta     JSON: the case's parameters, the steps run and the residual

Takes tens of minutes of host CPU (OpenMP):
  python tests/golden/make_steady_cavity.py [out.npz]
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "tests"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

N, SUB = 256, 4
RESIDUAL, MAX_STEPS = 1e-6, 2000000


def main(out):
    import cases as C
    c = C.cavity_moving_wall(N, N, op=C.MRT, nu=0.1 * N / 1000.0, u_lid=0.1)
    o = C.make_oracle(c, precision="f64")
    o.step(1000)
    _, u, _ = o.moments()
    steps, res = 1000, 1.0
    while steps < MAX_STEPS:
        u_prev = u
        o.step(1000)
        steps += 1000
        _, u, _ = o.moments()
        res = float(np.linalg.norm(u - u_prev) / np.linalg.norm(u))
        if steps % 50000 == 0:
            print(steps, res, flush=True)
        if res <= RESIDUAL:
            break
    meta = {"n": N, "steps": steps, "op": "MRT", "nu": 0.1 * N / 1000.0, "u_lid": 0.1, "subsample": SUB,
            "residual_last_1000_steps": res, "steady_criterion": RESIDUAL,
            "flags": "half-way bounce-back walls, moving-wall lid (cases.cavity_moving_wall)"}
    np.savez_compressed(out, u=u[:, ::SUB, ::SUB], u_prev=u_prev[:, ::SUB, ::SUB], meta=json.dumps(meta))
    print(out, "steps", steps, "residual over the last 1000 steps", res)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "steady_cavity256_mrt.npz"))
