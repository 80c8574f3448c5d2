"""Golden vectors from the reference's own build pin the oracle (CPU) and
the engine (GPU).

tests/golden/*.npz were written by tests/golden/make_golden.py from the
reference's LBM<2> compiled by oracle/ref_build.sh and run on a GB300: the
populations, density, velocity and force after steps 1, 2, 17 and 40 (20 for
CM<OptimalAdapter>) of ten small cases covering every operator, the shipped
2-D boundary functors, body force and the IBM cylinder.  Both the oracle and
the engine run with every reference quirk switched on and start from the
dumped step-0 fields.

Tolerance: the reference computes in FP32, so |diff| <= 5e-6 on every field
(the observed maximum is about 1.3e-6).
"""
import glob
import json
import os

import numpy as np
import pytest

import oracle as O

# the reference build's dumps (the steady-state field of make_steady_cavity.py
# is the FP64 oracle's and has its own test)
GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "*.npz"))
                if not os.path.basename(p).startswith(("steady_", "ref_validation")))
TOL = 5e-6


def load(path):
    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    nu = np.float32(meta["LBX_NU"])
    # the reference rounds tau and omega to float (scenario.cuh:36-38)
    om = float(np.float32(1) / (np.float32(3) * nu + np.float32(0.5)))
    op = meta["LBX_OPID"]
    S = [0, 1.0, 1.4, 0, 1.2, 0, 1.9, om, om] if op == 1 else [0, 0, 0, 1, om, om, 1, 1, 1]
    S = [float(np.float32(s)) for s in S]
    u_bc = float(np.float32({1: 0.04, 2: 0.1}.get(meta["LBX_CASE"], 0.05)))
    case = dict(nx=meta["NX"], ny=meta["NY"], op=op, omega=om, S=S,
                periodic=(meta["periodic_x"], meta["periodic_y"]), u_bc=u_bc)
    return z, meta, case


def test_golden_files_present():
    assert len(GOLDEN) == 10


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_reference_build(path):
    z, meta, c = load(path)
    o = O.Oracle(c["nx"], c["ny"], op=c["op"], omega=c["omega"], S=c["S"], periodic=c["periodic"],
                 quirks=O.QUIRKS_REFERENCE, u_bc=c["u_bc"])
    o.set_flags(z["flags"])
    o.init(z["rho_0"], z["u_0"], z["F_0"])
    if z["markers"].size:
        o.set_markers(z["markers"])
    done = 0
    for t in meta["steps"][1:]:
        o.step(t - done)
        done = t
        rho, u, F = o.moments()
        assert np.abs(o.populations() - z["f_%d" % t]).max() <= TOL
        assert np.abs(rho - z["rho_%d" % t]).max() <= TOL
        assert np.abs(u - z["u_%d" % t]).max() <= TOL
        assert np.abs(F - z["F_%d" % t]).max() <= TOL


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_engine_matches_reference_build(path):
    import lbmx

    z, meta, c = load(path)
    L = lbmx.Lattice(c["nx"], c["ny"], op=c["op"], omega=c["omega"], S=c["S"], periodic=c["periodic"],
                     quirks=lbmx.QUIRKS_REFERENCE, u_bc=c["u_bc"])
    L.set_flags(z["flags"])
    L.init(z["rho_0"], z["u_0"], z["F_0"])
    if z["markers"].size:
        L.set_markers(z["markers"])
    done = 0
    for t in meta["steps"][1:]:
        L.step(t - done)
        done = t
        rho, u, _ = L.moments()
        f = L.populations()
        m = np.isfinite(f)  # slots that streamed out of the domain are not kept
        assert np.abs(f[m] - z["f_%d" % t][m]).max() <= TOL
        assert np.abs(rho - z["rho_%d" % t]).max() <= TOL
        assert np.abs(u - z["u_%d" % t]).max() <= TOL
