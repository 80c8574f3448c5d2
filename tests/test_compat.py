"""Source compatibility with cuda-lbm scenarios (the ScenarioTrait contract).

* CPU: the reference's own unchanged 2-D scenario headers (Taylor-Green,
  lid-driven cavity, Poiseuille) compile against cuda-lbm_gb300/compat,
  including their compute_error validators.  The flow-past-cylinder header
  does not compile as shipped, against the reference's own headers either
  (its ScenarioTrait names the template BGK without <2>,
  flowPastCylinderScenario.cuh:12); with that one token fixed, in a
  temporary copy, it compiles too.
* GPU: the golden scenarios (oracle/ref_scenarios.cuh) -- the very source the
  reference's build ran to write tests/golden/ -- run on lbmx through
  lbmx_compat::create and reproduce the reference's dumps.
"""
import ctypes
import glob
import json
import os
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
COMPAT = os.path.join(REPO, "cuda-lbm_gb300", "compat")
INCLUDE = os.path.join(REPO, "include")
REF_SCEN = "/root/reference/src/scenarios"
BUILD = os.path.join(REPO, "tests", "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

UNCHANGED = [
    ("taylorGreen/taylorGreenScenario.cuh", "TaylorGreenScenario", "-DNX=256 -DNY=256 -DSCALE=2 -DPERIODIC_X -DPERIODIC_Y"),
    ("lidDrivenCavity/lidDrivenCavityScenario.cuh", "LidDrivenScenario", "-DNX=129 -DNY=129"),
    ("poiseuille/poiseuilleScenario.cuh", "PoiseuilleScenario", "-DNX=150 -DNY=100 -DPERIODIC_X"),
]


@pytest.mark.skipif(not os.path.isdir(REF_SCEN), reason="reference checkout not mounted")
@pytest.mark.parametrize("header,name,defs", UNCHANGED, ids=[u[1] for u in UNCHANGED])
def test_reference_scenario_headers_compile_unchanged(header, name, defs, tmp_path):
    _compile_scenario(os.path.join(REF_SCEN, header), name, defs, tmp_path)


def _compile_scenario(header_path, name, defs, tmp_path, extra_includes=()):
    src = tmp_path / "use_scenario.cu"
    src.write_text(
        '#include "lbmx_scenario.cuh"\n'
        '#include "%s"\n'
        "int build(lbmx_handle** h) { return lbmx_compat::create<%s>(h); }\n"
        "float validate() { lbmx_compat::Solver<%s> s; s.step(1); return %s::compute_error(s); }\n"
        % (header_path, name, name, name))
    cmd = ["nvcc"] + ARCH + ["-std=c++17", "-c", "-w", "-I" + COMPAT, "-I" + INCLUDE] + \
        ["-I" + d for d in extra_includes] + defs.split() + [str(src), "-o", str(tmp_path / "use_scenario.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


@pytest.mark.skipif(not os.path.isdir(REF_SCEN), reason="reference checkout not mounted")
def test_reference_cylinder_scenario_compiles_with_its_template_argument_fixed(tmp_path):
    # the one change the reference's own build needs too: `BGK` -> `BGK<2>`
    # in the ScenarioTrait argument list; the functors header is used as is
    d = os.path.join(REF_SCEN, "flowPastCylinder")
    text = open(os.path.join(d, "flowPastCylinderScenario.cuh"), newline="").read().replace("\r\n", "\n")
    lines = text.split("\n")
    fixed = [i for i, ln in enumerate(lines) if ln.strip() == "BGK"]
    assert len(fixed) == 1
    lines[fixed[0]] = lines[fixed[0]].replace("BGK", "BGK<2>")
    copy = tmp_path / "flowPastCylinderScenario.cuh"
    copy.write_text("\n".join(lines))
    _compile_scenario(str(copy), "FlowPastCylinderScenario", "-DNX=400 -DNY=100", tmp_path, extra_includes=(d,))


def _case_flags(name):
    out = subprocess.check_output(["bash", os.path.join(REPO, "oracle", "ref_build.sh"), "list"], text=True)
    for line in out.splitlines():
        case, defs = line.split("|", 1)
        if case == name:
            return defs.split()
    raise KeyError(name)


def _build_runner(name):
    import build as B
    lib = B.build()
    os.makedirs(BUILD, exist_ok=True)
    so = os.path.join(BUILD, "compat_%s.so" % name)
    cmd = ["nvcc"] + ARCH + ["-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-w", "-I" + COMPAT, "-I" + INCLUDE,
                             "-I" + os.path.join(REPO, "oracle")] + _case_flags(name) + \
        [os.path.join(REPO, "tests", "compat", "compat_runner.cu"), "-L" + os.path.dirname(lib), "-llbmx",
         "-Xlinker", "-rpath," + os.path.dirname(lib), "-o", so]
    subprocess.run(cmd, check=True, capture_output=True)
    return so


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tg_mrt", "cavity_bgk", "poiseuille_ibm_bgk", "channel_zg_bgk"])
def test_golden_scenario_runs_unchanged_on_lbmx(name):
    z = np.load(os.path.join(REPO, "tests", "golden", name + ".npz"))
    meta = json.loads(str(z["meta"]))
    steps = meta["steps"][1:]
    lib = ctypes.CDLL(_build_runner(name))
    nx, ny = ctypes.c_int(), ctypes.c_int()
    lib.scenario_lattice(ctypes.byref(nx), ctypes.byref(ny))
    n = nx.value * ny.value
    f = np.zeros((len(steps), 9, ny.value, nx.value), np.float32)
    rho = np.zeros((len(steps), ny.value, nx.value), np.float32)
    u = np.zeros((len(steps), 2, ny.value, nx.value), np.float32)
    arr = (ctypes.c_int * len(steps))(*steps)
    P = ctypes.c_void_p
    rc = lib.run_scenario(arr, len(steps), P(f.ctypes.data), P(rho.ctypes.data), P(u.ctypes.data))
    assert rc == 0
    # the compat run starts from its own evaluation of the Init functor and
    # its own create_cylinder, so it differs from the dumps by float rounding
    for k, t in enumerate(steps):
        m = np.isfinite(f[k])
        assert np.abs(f[k][m] - z["f_%d" % t][m]).max() <= 2e-5
        assert np.abs(rho[k] - z["rho_%d" % t]).max() <= 2e-5
        assert np.abs(u[k] - z["u_%d" % t]).max() <= 2e-5
