"""CPU checks of the C-ABI library: it builds, loads and exports every
entry point declared in include/lbmx.h (no compute calls: no GPU here)."""
import ctypes
import os
import re

import build as B

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(REPO, "include", "lbmx.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(lbmx_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    path = B.build()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 17
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    import lbmx
    assert set(declared_symbols()) <= set(lbmx.EXPORTED)


def test_version_and_defaults_without_gpu():
    import lbmx
    lib = lbmx.load_library(B.build())
    assert lib.lbmx_version() == 1
    p = lbmx.Params()
    lib.lbmx_params_default(ctypes.byref(p))
    assert p.op == 0 and p.storage == 0 and p.ibm_iters == 3 and abs(p.rho_out - 1) < 1e-7
    assert ctypes.sizeof(lbmx.Params) == 4 * 10 + 4 * 17 + 4 + 8  # matches the C struct


def test_create_rejects_lattices_whose_padded_plane_overflows():
    # rows are padded to whole 128-node tiles and node offsets are 32-bit:
    # 129 x 16,646,000 nodes fit in 2^31 but their padded plane (256 per row)
    # does not.  The size checks come before any device call.
    import lbmx
    lib = lbmx.load_library(B.build())
    for nx, ny in ((129, 16646000), (1 << 16, 1 << 16)):
        p = lbmx.Params()
        lib.lbmx_params_default(ctypes.byref(p))
        p.nx, p.ny = nx, ny
        h = ctypes.c_void_p()
        assert lib.lbmx_create(ctypes.byref(p), ctypes.byref(h)) == 8  # LBMX_ERR_TOO_LARGE
        assert not h.value

