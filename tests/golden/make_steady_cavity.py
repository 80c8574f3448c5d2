"""Generate tests/golden/steady_cavity256_mrt.npz: the FP64 oracle's
lid-driven cavity (256 x 256, MRT, half-way walls, moving lid 0.1, Re 1000 on
the side, rho = 1 and u = 0 at the start) after 100,000 steps -- close to
its steady state -- as the reference field for the 16-bit storage forms'
steady-state error.

  u        velocity [2][64][64]: every 4th node in x and y (node 4j, 4i)
  u_prev   the same 1000 steps earlier (how far from steady the flow is)
  meta     JSON: the case's parameters

Takes a few minutes of host CPU (OpenMP):
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

N, STEPS, SUB = 256, 100000, 4


def main(out):
    import cases as C
    c = C.cavity_moving_wall(N, N, op=C.MRT, nu=0.1 * N / 1000.0, u_lid=0.1)
    o = C.make_oracle(c, precision="f64")
    o.step(STEPS - 1000)
    _, u_prev, _ = o.moments()
    o.step(1000)
    _, u, _ = o.moments()
    meta = {"n": N, "steps": STEPS, "op": "MRT", "nu": 0.1 * N / 1000.0, "u_lid": 0.1, "subsample": SUB,
            "flags": "half-way bounce-back walls, moving-wall lid (cases.cavity_moving_wall)"}
    np.savez_compressed(out, u=u[:, ::SUB, ::SUB], u_prev=u_prev[:, ::SUB, ::SUB], meta=json.dumps(meta))
    print(out, "residual over the last 1000 steps",
          float(np.linalg.norm(u - u_prev) / np.linalg.norm(u)))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "steady_cavity256_mrt.npz"))
