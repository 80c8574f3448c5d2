"""Generate the golden vectors of tests/golden/ from the reference's own build.

Runs every harness binary built by oracle/ref_build.sh (the reference's
LBM<2> through its main-loop call sequence, src/main.cu:96-114) on a GPU and
packs its dumps into one compressed .npz per case:

  f_<t>     post-collision populations, planes [9][ny][nx] (reference order)
  rho_<t>   density, u_<t> force-corrected velocity [2][ny][nx],
  F_<t>     force [2][ny][nx] -- the reference's d_rho / d_u / d_force
  flags     boundary flags [ny][nx];  markers  IBM points [n][2]
  meta      JSON: the case's compile-time parameters

Usage (on a machine with a GPU and the built binaries):
  python tests/golden/make_golden.py [out_dir]
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
BIN = os.path.join(REPO, "oracle", "_ref", "bin")
RECIPE = os.path.join(REPO, "oracle", "ref_build.sh")

STEPS = {"tg_cmopt": (20, [0, 1, 2, 9, 20])}
DEFAULT_STEPS = (40, [0, 1, 2, 17, 40])


def parse_defs(defs):
    meta = {"periodic_x": "-DPERIODIC_X" in defs, "periodic_y": "-DPERIODIC_Y" in defs,
            "markers": "-DLBX_NO_MARKERS" not in defs}
    for tok in defs.split():
        if tok.startswith("-D") and "=" in tok:
            k, v = tok[2:].split("=", 1)
            meta[k] = float(v.rstrip("f")) if k == "LBX_NU" else int(v)
    return meta


def read_dump(path):
    with open(path, "rb") as fh:
        hdr = np.frombuffer(fh.read(20), np.int32)
        assert hdr[0] == 0x4658424C, "bad dump " + path
        nx, ny, t, nm = (int(v) for v in hdr[1:])
        n = nx * ny
        f = np.frombuffer(fh.read(36 * n), np.float32).reshape(ny, nx, 9).transpose(2, 0, 1)
        rho = np.frombuffer(fh.read(4 * n), np.float32).reshape(ny, nx)
        u = np.frombuffer(fh.read(8 * n), np.float32).reshape(ny, nx, 2).transpose(2, 0, 1)
        F = np.frombuffer(fh.read(8 * n), np.float32).reshape(ny, nx, 2).transpose(2, 0, 1)
        xy = np.frombuffer(fh.read(8 * nm), np.float32).reshape(nm, 2)
        flags = np.frombuffer(fh.read(4 * n), np.int32).reshape(ny, nx)
    return t, f, rho, u, F, xy, flags


def main(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    cases = subprocess.check_output(["bash", RECIPE, "list"], text=True).split("\n")
    for line in filter(None, cases):
        name, defs = line.split("|", 1)
        nsteps, at = STEPS.get(name, DEFAULT_STEPS)
        with tempfile.TemporaryDirectory() as tmp:
            subprocess.run([os.path.join(BIN, name), tmp, str(nsteps)] + [str(a) for a in at], check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            arrays = {}
            for t_req in at:
                t, f, rho, u, F, xy, flags = read_dump(os.path.join(tmp, "t%06d.bin" % t_req))
                arrays["f_%d" % t] = f
                arrays["rho_%d" % t] = rho
                arrays["u_%d" % t] = u
                arrays["F_%d" % t] = F
                arrays["markers"] = xy
                arrays["flags"] = flags.astype(np.uint8)
        meta = parse_defs(defs)
        meta.update(name=name, steps=at)
        arrays["meta"] = np.array(json.dumps(meta))
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), **arrays)
        print("wrote", name)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
