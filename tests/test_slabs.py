"""The y-slab exchange protocol (cuda-lbm_gb300/lbmx_slabs.py) on the CPU.

A lattice split into slabs must step bit for bit as the whole lattice.  The
lattice here is the numpy restatement of the engine's in-place slot layout
(tests/aa_numpy.py), so the planes and rows the protocol exchanges are
exactly the engine's.  The same protocol runs the engine's slabs on one GPU
in tests/test_slabs_gpu.py.
  * the row split and ghost rows of SlabGeometry;
  * three slabs in one process (LocalComm), with and without a grid-average
    term folded from the slabs' integer partial sums;
  * two slabs on two gloo CPU ranks (DistComm): halo rows travel as host
    buffers by point-to-point messages, the partial sums by an int64
    all-reduce.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

import aa_numpy as A
import lbmx_slabs as S


def _state(nx, ny, seed):
    rng = np.random.default_rng(seed)
    rho = 1.0 + 0.02 * rng.standard_normal((ny, nx))
    u = 0.03 * rng.standard_normal((2, ny, nx))
    return rho, u


def _whole(rho, u, steps, averaged):
    L = A.AALattice(rho, u, omega=1.3, averaged=averaged)
    L.step(steps)
    return L


def _slab(rho, u, g, averaged):
    return A.AALattice(g.take(rho), g.take(u), omega=1.3, ghost_mask=g.ghost_mask, averaged=averaged,
                       whole_nodes=rho.size)


def test_geometry_covers_every_row_once():
    for ny, n in ((64, 2), (65, 3), (10, 5)):
        for periodic in (False, True):
            gs = [S.SlabGeometry(ny, n, k, periodic) for k in range(n)]
            owned = np.concatenate([np.arange(g.y0, g.y1) for g in gs])
            assert np.array_equal(owned, np.arange(ny))
            for g in gs:
                rows = g.rows()
                assert len(rows) == g.ny_handle
                assert np.array_equal(rows[g.first_owned:g.last_owned + 1], np.arange(g.y0, g.y1))
                if g.has_lower:
                    assert rows[0] == (g.y0 - 1) % ny and g.ghost_mask & 1
                if g.has_upper:
                    assert rows[-1] == g.y1 % ny and g.ghost_mask & 2
            assert gs[0].has_lower == periodic and gs[-1].has_upper == periodic
    with pytest.raises(ValueError):
        S.SlabGeometry(3, 2, 0, False)


def test_averages_match_the_engines_formula():
    sums = np.array([1073741824 * 1000 + 12345, 7, -3], np.int64)
    a = S.averages_from_sums(sums, 1000)
    assert a.dtype == np.float32
    assert a[0] == np.float32((float(sums[0]) * 2.0 ** -30) / 1000.0)


@pytest.mark.parametrize("averaged", [False, True])
@pytest.mark.parametrize("steps", [1, 2, 13])
def test_local_slabs_match_the_whole_lattice(averaged, steps):
    nx, ny, n = 24, 30, 3
    rho, u = _state(nx, ny, 3)
    whole = _whole(rho, u, steps, averaged)
    slabs = []
    for k in range(n):
        g = S.SlabGeometry(ny, n, k, True)
        slabs.append((_slab(rho, u, g, averaged), g))
    comm = S.LocalComm(slabs, lambda nbytes: np.empty(nbytes, np.uint8))
    S.step_slabs(comm, steps, rho.size)
    for L, g in slabs:
        assert np.array_equal(g.owned(L.F), whole.F[:, g.y0:g.y1])


def test_exchange_is_needed():
    """Without the exchange the slabs drift from the whole lattice (the test
    above is not trivially satisfied)."""
    nx, ny = 24, 30
    rho, u = _state(nx, ny, 4)
    whole = _whole(rho, u, 3, False)
    g = S.SlabGeometry(ny, 2, 0, True)
    L = _slab(rho, u, g, False)
    L.step(3)
    assert not np.array_equal(g.owned(L.F), whole.F[:, g.y0:g.y1])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, steps, averaged, q):
    import sys
    import torch.distributed as dist
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path[:0] = [here, os.path.join(os.path.dirname(here), "cuda-lbm_gb300")]
    import aa_numpy as A2
    import lbmx_slabs as S2
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    nx, ny = 20, 26
    rho, u = _state(nx, ny, 11)
    g = S2.SlabGeometry(ny, world, rank, True)
    L = A2.AALattice(g.take(rho), g.take(u), omega=1.3, ghost_mask=g.ghost_mask, averaged=averaged,
                     whole_nodes=rho.size)
    S2.step_slabs(S2.DistComm(L, g, dist), steps, rho.size)
    whole = A2.AALattice(rho, u, omega=1.3, averaged=averaged)
    whole.step(steps)
    q.put((rank, bool(np.array_equal(g.owned(L.F), whole.F[:, g.y0:g.y1]))))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("averaged", [False, True])
def test_two_gloo_ranks_match_the_whole_lattice(averaged):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, 9, averaged, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, True), (1, True)]
