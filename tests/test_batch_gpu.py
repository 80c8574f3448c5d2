"""Batched stepping (lbmx_batch_*): many lattices, one persistent launch per step.

Each lattice of a batch must come out bit for bit as when stepped alone --
the batched kernel runs the same per-node arithmetic, only the work split
differs -- for every tile shape, with and without CUDA-graph replay, with
edge pre-passes (ZG, pressure outlet, regularized corners), per-node force
fields and odd lattice sizes.  The autotuner must leave the lattices as it
found them.
"""
import numpy as np
import pytest

import cases as C
import lbmx

pytestmark = pytest.mark.gpu


def mixed_cases(op, quirks=0):
    rng = np.random.default_rng(11)
    F = 1e-5 * rng.standard_normal((2, 40, 80))
    return [
        C.random_state(C.cavity_moving_wall(150, 70, op=op, quirks=quirks), seed=1),
        C.random_state(C.taylor_green(64, 48, op=op, quirks=quirks), seed=2),
        C.random_state(C.channel(200, 40, op=op, outlet="zg", quirks=quirks), seed=3),
        C.random_state(C.poiseuille(96, 33, op=op, quirks=quirks), seed=4),
        C.random_state(C.cavity_regularized(37, 29, op=op, quirks=quirks), seed=5),
        C.random_state(C.channel(130, 66, op=op, outlet="pressure", quirks=quirks), seed=6),
        C.random_state(C.taylor_green(80, 40, op=op, quirks=quirks, force=F), seed=7),
        C.random_state(C.cavity_moving_wall(300, 12, op=op, quirks=quirks), seed=8),
    ]


def assert_same(alone, batched):
    for a, b in zip(alone, batched):
        assert a.t == b.t
        ra, ua, _ = a.moments()
        rb, ub, _ = b.moments()
        np.testing.assert_array_equal(ra, rb)
        np.testing.assert_array_equal(ua, ub)
        np.testing.assert_array_equal(np.nan_to_num(a.populations(), nan=7.0),
                                      np.nan_to_num(b.populations(), nan=7.0))


@pytest.mark.parametrize("storage", [0, 1, 2])
@pytest.mark.parametrize("op", [C.BGK, C.MRT, C.CM])
@pytest.mark.parametrize("tile_w,tile_h,ctas,chunk,graph", [(64, 8, 2, 1, 0), (128, 4, 1, 3, 4), (128, 8, 2, 2, 16)])
def test_batch_matches_lattices_stepped_alone(op, storage, tile_w, tile_h, ctas, chunk, graph):
    cs = mixed_cases(op)
    alone = [C.make_lattice(c, storage=storage) for c in cs]
    batched = [C.make_lattice(c, storage=storage) for c in cs]
    for L in alone:
        L.step(41)
    B = lbmx.Batch(batched)
    B.set_config(tile_w=tile_w, tile_h=tile_h, ctas_per_sm=ctas, chunk=chunk, graph_steps=graph)
    B.step(38, flags=0)
    B.step(3)
    assert_same(alone, batched)
    B.close()


def test_batch_reference_quirks_on_a_shared_stream():
    # every lattice on one stream: the batch runs on it directly
    torch = pytest.importorskip("torch")
    s = torch.cuda.Stream()
    cs = mixed_cases(C.MRT, quirks=C.QUIRKS_REFERENCE)
    alone = [C.make_lattice(c) for c in cs]
    batched = [C.make_lattice(c, stream=s.cuda_stream) for c in cs]
    for L in alone:
        L.step(17)
    B = lbmx.Batch(batched)
    B.step(9)
    B.step(8)
    assert_same(alone, batched)


def test_batch_matches_oracle():
    c = C.random_state(C.cavity_moving_wall(70, 50, op=C.MRT), seed=9)
    o = C.make_oracle(c, precision="f32")
    L = C.make_lattice(c)
    other = C.make_lattice(C.taylor_green(64, 64, op=C.MRT))
    B = lbmx.Batch([other, L])
    B.step(25)
    o.step(25)
    rho, u, _ = L.moments()
    ro, uo, _ = o.moments()
    np.testing.assert_allclose(rho, ro, rtol=0, atol=2e-6)
    np.testing.assert_allclose(u, uo, rtol=0, atol=2e-6)


def test_autotune_leaves_the_lattices_unchanged():
    cs = mixed_cases(C.MRT)
    Ls = [C.make_lattice(c, storage=1) for c in cs]
    ref = [C.make_lattice(c, storage=1) for c in cs]
    for L in Ls + ref:
        L.step(3)
    before = [np.nan_to_num(L.populations(), nan=7.0) for L in Ls]
    B = lbmx.Batch(Ls)
    cfg = B.autotune(trial_steps=3)
    assert (cfg["tile_w"], cfg["tile_h"]) in ((64, 8), (128, 4), (128, 8))
    assert cfg["ctas_per_sm"] in (1, 2, 3) and cfg["chunk"] >= 1
    assert B.config == cfg
    for L, p in zip(Ls, before):
        assert L.t == 3
        np.testing.assert_array_equal(np.nan_to_num(L.populations(), nan=7.0), p)
    B.step(26)
    for L in ref:
        L.step(26)
    assert_same(ref, Ls)


def test_lattices_restepped_alone_after_a_batch():
    cs = mixed_cases(C.BGK)[:3]
    alone = [C.make_lattice(c) for c in cs]
    mixed = [C.make_lattice(c) for c in cs]
    B = lbmx.Batch(mixed)
    B.step(5)
    for L in mixed:
        L.step(4)
    for L in alone:
        L.step(9)
    assert_same(alone, mixed)
    with pytest.raises(lbmx.LbmxError):
        mixed[0].step(1)
        B.step(1)  # lattice 0 is now one step ahead of the others


def test_batch_finite_check():
    c = C.taylor_green(64, 48, op=C.BGK)
    rho = np.array(c["rho"], np.float32)
    rho[10, 10] = np.nan
    bad = dict(c, rho=rho)
    B = lbmx.Batch([C.make_lattice(c), C.make_lattice(bad)])
    with pytest.raises(lbmx.LbmxError) as e:
        B.step(2, flags=lbmx.STEP_STORE_MOMENTS | lbmx.STEP_CHECK_FINITE)
    assert e.value.code == 7


def test_batch_rejects_what_it_cannot_run():
    tg = C.taylor_green(64, 48, op=C.BGK)
    a, b = C.make_lattice(tg), C.make_lattice(tg)
    with pytest.raises(lbmx.LbmxError):
        lbmx.Batch([a, C.make_lattice(C.taylor_green(64, 48, op=C.MRT))])
    with pytest.raises(lbmx.LbmxError):
        lbmx.Batch([a, C.make_lattice(tg, storage=1)])
    with pytest.raises(lbmx.LbmxError) as e:
        lbmx.Batch([C.make_lattice(C.taylor_green(64, 48, op=C.CM_OPT))])
    assert e.value.code == 6
    with pytest.raises(lbmx.LbmxError) as e:
        lbmx.Batch([C.make_lattice(C.channel(96, 48, markers=C.cylinder_markers(30, 24, 6, 24)))])
    assert e.value.code == 6
    with pytest.raises(lbmx.LbmxError):
        lbmx.Batch([a, a])
    b.step(1)
    with pytest.raises(lbmx.LbmxError):
        lbmx.Batch([a, b])
    B = lbmx.Batch([a])
    for bad in (dict(tile_w=96), dict(tile_w=64, tile_h=4), dict(ctas_per_sm=4), dict(chunk=0), dict(graph_steps=3)):
        with pytest.raises(lbmx.LbmxError):
            B.set_config(**bad)
