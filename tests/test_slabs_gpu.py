"""y-slabs of the engine on one GPU: a lattice split into two or three
slab handles (lbmx_set_slab, halo rows copied by lbmx_halo_get/put into
device buffers, CM_OPT averages folded from lbmx_opt_partials) steps bit
for bit as the whole lattice -- populations, density and velocity of every
owned row -- for BGK, MRT, CM and CM_OPT, FP32 and FP16-offset storage,
walled and periodic lattices, odd and even step counts."""
import numpy as np
import pytest

import cases as C
import lbmx
import lbmx_slabs as S

pytestmark = pytest.mark.gpu


def _run_slabs(c, nslabs, steps, storage):
    import torch
    stream = torch.cuda.Stream()
    slabs = []
    for k in range(nslabs):
        g = S.SlabGeometry(c["ny"], nslabs, k, c["periodic"][1])
        slabs.append((S.make_slab_lattice(lbmx, c, g, storage=storage, stream=stream.cuda_stream), g))
    comm = S.LocalComm(slabs, lambda nbytes: torch.empty(nbytes, dtype=torch.uint8, device="cuda"))
    # the same step variants as the whole lattice's lbmx_step: moments stored
    # on the last step only
    S.step_slabs(comm, steps - 1, c["nx"] * c["ny"], flags=0)
    S.step_slabs(comm, 1, c["nx"] * c["ny"])
    return slabs


def _compare(c, slabs, whole):
    rw, uw, sw = whole.moments()
    pw = np.nan_to_num(whole.populations(), nan=-7.0)
    mass = 0.0
    for L, g in slabs:
        r, u, s = L.moments()
        p = np.nan_to_num(L.populations(), nan=-7.0)
        assert np.array_equal(g.owned(r), rw[g.y0:g.y1])
        assert np.array_equal(g.owned(u), uw[:, g.y0:g.y1])
        assert np.array_equal(g.owned(p), pw[:, g.y0:g.y1])
        mass += s[0]
    # the slabs' sums cover their owned rows only
    assert abs(mass - sw[0]) <= 1e-9 * abs(sw[0])


CASES = {
    "cavity": lambda op: C.random_state(C.cavity_moving_wall(70, 44, op=op, nu=0.05), seed=2),
    "taylor_green": lambda op: C.random_state(C.taylor_green(48, 40, op=op), seed=3),
    "channel": lambda op: C.random_state(C.channel(64, 36, op=op, nu=0.04, u_in=0.04, inlet="zouhe",
                                                   outlet="pressure"), seed=4),
}


@pytest.mark.parametrize("op", [C.BGK, C.MRT, C.CM, C.CM_OPT])
@pytest.mark.parametrize("case", sorted(CASES))
def test_two_slabs_match_the_whole_lattice(op, case):
    c = CASES[case](op)
    steps = 21 if op == C.CM_OPT else 40
    whole = C.make_lattice(c)
    whole.step(steps)
    _compare(c, _run_slabs(c, 2, steps, 0), whole)


@pytest.mark.parametrize("storage", [0, 1])
@pytest.mark.parametrize("steps", [1, 2, 33])
def test_three_slabs_match_the_whole_lattice(storage, steps):
    c = C.random_state(C.cavity_moving_wall(96, 60, op=C.MRT, nu=0.03), seed=9)
    whole = C.make_lattice(c, storage=storage)
    whole.step(steps)
    _compare(c, _run_slabs(c, 3, steps, storage), whole)


def test_slab_rejects_markers_and_periodic_y():
    c = C.taylor_green(32, 24)
    L = lbmx.Lattice(32, 24, periodic=(True, True))
    with pytest.raises(lbmx.LbmxError):
        L.set_slab(1, 0)
    L2 = lbmx.Lattice(32, 24)
    L2.set_slab(3, 5)
    with pytest.raises(lbmx.LbmxError):
        L2.set_markers(C.cylinder_markers(16, 12, 4, 8))
