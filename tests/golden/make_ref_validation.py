"""Writes tests/golden/ref_validation.npz: what the reference's own build
reports for its unchanged 2-D scenario headers (Taylor-Green, lid-driven
cavity, Poiseuille, flow past a cylinder) when its main loop runs them.

Needs a CUDA GPU and the patched reference sources under oracle/_ref/src
(`oracle/ref_build.sh sources`, run where the reference checkout is
mounted).  It builds oracle/ref_validate.cu once per scenario
(`ref_build.sh validators`), runs each binary to the dump steps and stores,
per step, the scenario's compute_error and a strided probe of the velocity
field its validator read (every PROBE-th node in x and y, both components).

    python tests/golden/make_ref_validation.py
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
RECIPE = os.path.join(REPO, "oracle", "ref_build.sh")
BIN = os.path.join(REPO, "oracle", "_ref", "bin")
OUT = os.path.join(HERE, "ref_validation.npz")

# the reference's main loop runs 20000 steps and validates every 100
STEPS = [100, 1000, 5000, 20000]
PROBE = 8


def validators():
    out = subprocess.check_output(["bash", RECIPE, "validators-list"], text=True)
    rows = []
    for line in out.splitlines():
        name, header, struct, defs = line.split("|")
        d = dict(tok[2:].split("=", 1) if "=" in tok else (tok[2:], "1") for tok in defs.split())
        rows.append(dict(name=name, header=header, struct=struct, defs=defs, nx=int(d["NX"]), ny=int(d["NY"])))
    return rows


def probe(u_aos, nx, ny):
    return u_aos.reshape(ny, nx, 2)[::PROBE, ::PROBE, :]


def main():
    subprocess.check_call(["bash", RECIPE, "validators"])
    meta = {"steps": STEPS, "probe_stride": PROBE, "scenarios": {}}
    arrays = {}
    for v in validators():
        with tempfile.TemporaryDirectory() as d:
            out = subprocess.check_output([os.path.join(BIN, v["name"]), d] + [str(s) for s in STEPS], text=True)
            errs = {}
            for line in out.split("\n"):
                parts = line.split()
                if len(parts) == 2 and parts[0].isdigit():
                    errs[int(parts[0])] = float(parts[1])
            probes = [probe(np.fromfile(os.path.join(d, "u%d.bin" % t), dtype=np.float32), v["nx"], v["ny"])
                      for t in STEPS]
        arrays[v["name"] + "_err"] = np.array([errs[t] for t in STEPS], np.float32)
        arrays[v["name"] + "_u"] = np.stack(probes).astype(np.float32)
        meta["scenarios"][v["name"]] = dict(header=v["header"], struct=v["struct"], defs=v["defs"])
        print(v["name"], {t: errs[t] for t in STEPS}, flush=True)
    np.savez_compressed(OUT, meta=json.dumps(meta), **arrays)
    print("wrote", OUT)


if __name__ == "__main__":
    sys.exit(main())
