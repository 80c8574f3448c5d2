"""Checkpoint / restart and .vti output through the C-ABI.

A checkpoint holds the dynamic state only (populations in storage form, the
edge store, the step count, the CM_OPT averages) plus a CRC-32; a handle
built with the same params, flags, force and markers continues bit for bit.
"""
import os

import numpy as np
import pytest

import cases as C
import lbmx

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage", [0, 1])
@pytest.mark.parametrize("k", [3, 4])
def test_restart_is_bit_exact(tmp_path, storage, k):
    c = C.random_state(C.cavity_regularized(96, 64, op=C.MRT, quirks=C.QUIRKS_REFERENCE), seed=5)
    a = C.make_lattice(c, storage=storage)
    a.step(k)
    a.save(str(tmp_path / "s.ckpt"))
    a.step(11)
    ra, ua, _ = a.moments()
    b = C.make_lattice(c, storage=storage)
    b.load(str(tmp_path / "s.ckpt"))
    assert b.t == k
    b.step(11)
    rb, ub, _ = b.moments()
    assert np.array_equal(ra, rb) and np.array_equal(ua, ub)
    assert np.array_equal(np.nan_to_num(a.populations()), np.nan_to_num(b.populations()))


@pytest.mark.parametrize("storage", [0, 1])
def test_restart_with_markers_is_bit_exact(tmp_path, storage):
    """An IBM cylinder resumes bit for bit: the marker rounds are recomputed
    from the stored populations each step, and their spread is ordered."""
    mk = C.cylinder_markers(40.3, 30.7, 8.0, 48)
    c = C.channel(128, 64, op=C.BGK, nu=0.03, u_in=0.05, inlet="parabolic", outlet="zouhe_p", markers=mk)
    a = C.make_lattice(c, storage=storage)
    a.step(37)
    a.save(str(tmp_path / "s.ckpt"))
    a.step(50)
    ra, ua, _ = a.moments()
    Fa, da = a.marker_forces()
    b = C.make_lattice(c, storage=storage)
    b.load(str(tmp_path / "s.ckpt"))
    b.step(50)
    rb, ub, _ = b.moments()
    Fb, db = b.marker_forces()
    assert np.array_equal(ra, rb) and np.array_equal(ua, ub)
    assert np.array_equal(Fa, Fb) and np.array_equal(np.asarray(da), np.asarray(db))


def test_restart_rejects_corrupt_or_foreign_files(tmp_path):
    c = C.taylor_green(64, 48, op=C.BGK)
    a = C.make_lattice(c)
    a.step(2)
    path = str(tmp_path / "s.ckpt")
    a.save(path)
    raw = bytearray(open(path, "rb").read())
    raw[200] ^= 0x40
    bad = str(tmp_path / "bad.ckpt")
    open(bad, "wb").write(raw)
    with pytest.raises(lbmx.LbmxError) as e:
        C.make_lattice(c).load(bad)
    assert "CRC" in str(e.value)
    other = C.make_lattice(C.taylor_green(64, 32, op=C.BGK))
    with pytest.raises(lbmx.LbmxError):
        other.load(path)
    with pytest.raises(lbmx.LbmxError):
        C.make_lattice(c, storage=1).load(path)


def test_vti_holds_the_stored_moments(tmp_path):
    c = C.random_state(C.taylor_green(40, 24, op=C.MRT), seed=2)
    L = C.make_lattice(c)
    L.step(5)
    rho, u, _ = L.moments()
    path = str(tmp_path / "out.vti")
    L.write_vti(path)
    data = open(path, "rb").read()
    head, _, rest = data.partition(b"<AppendedData encoding=\"raw\">\n   _")
    assert b'WholeExtent="0 39 0 23 0 0"' in head
    n = 40 * 24
    nb = int(np.frombuffer(rest[:8], np.uint64)[0])
    assert nb == 4 * n
    r = np.frombuffer(rest[8:8 + nb], np.float32).reshape(24, 40)
    nv = int(np.frombuffer(rest[8 + nb:16 + nb], np.uint64)[0])
    v = np.frombuffer(rest[16 + nb:16 + nb + nv], np.float32).reshape(24, 40, 3)
    assert np.array_equal(r, rho)
    assert np.array_equal(v[..., 0], u[0]) and np.array_equal(v[..., 1], u[1]) and not v[..., 2].any()


def test_per_step_sums_read_without_waiting():
    # LBMX_STEP_SUMS reduces the FP64 sums in every step's kernel; the async
    # readback delivers each step's sums once the stream has reached it
    import ctypes
    c = C.random_state(C.cavity_moving_wall(80, 60, op=C.MRT), seed=3)
    a = C.make_lattice(c)
    b = C.make_lattice(c)
    ring = (ctypes.c_double * (3 * 6))()
    for k in range(6):
        a.step(1, flags=lbmx.STEP_SUMS)
        a._check(a.lib.lbmx_moment_sums_async(a.h, ctypes.addressof(ring) + 24 * k))
    a.synchronize()
    for k in range(6):
        b.step(1)
        _, _, s = b.moments()
        # fixed-point sums: the same bits from the sums-only variant (published
        # one launch late) and from the full variant, in any tile order
        assert list(ring[3 * k: 3 * k + 3]) == list(s)


def test_step_sums_series():
    import ctypes
    c = C.random_state(C.taylor_green(64, 48, op=C.BGK), seed=4)
    a = C.make_lattice(c)
    b = C.make_lattice(c)
    series = (ctypes.c_double * (3 * 5))()
    a._check(a.lib.lbmx_step_sums(a.h, 5, lbmx.STEP_STORE_MOMENTS, ctypes.addressof(series)))
    a.synchronize()
    for k in range(5):
        b.step(1)
        _, _, s = b.moments()
        assert list(series[3 * k: 3 * k + 3]) == list(s)
    np.testing.assert_array_equal(a.moments()[1], b.moments()[1])


def test_sums_across_mixed_step_kinds():
    # sums-only steps publish their sums one launch late: through the next
    # step of any kind, or at the end of the call; a plain step leaves the
    # last published sums alone
    import ctypes
    c = C.random_state(C.cavity_moving_wall(96, 72, op=C.MRT), seed=8)
    a = C.make_lattice(c)
    b = C.make_lattice(c)
    got = (ctypes.c_double * 3)()
    a.step(3, flags=lbmx.STEP_SUMS)
    a.step(2, flags=lbmx.STEP_SUMS | lbmx.STEP_STORE_MOMENTS)
    _, _, s5 = a.moments()
    a.step(1, flags=0)
    a._check(a.lib.lbmx_moment_sums_async(a.h, ctypes.addressof(got)))
    a.synchronize()
    b.step(5)
    _, _, r5 = b.moments()
    assert list(s5) == list(r5) and list(got) == list(r5)


@pytest.mark.parametrize("storage", [0, 1])
def test_single_steps_around_batched_steps(storage):
    # the step kernel alternates two work counters by step parity; batched
    # steps in between use the batch's own, so the lattice re-arms both
    c = C.random_state(C.cavity_moving_wall(120, 88, op=C.MRT), seed=9)
    a = C.make_lattice(c, storage=storage)
    b = C.make_lattice(c, storage=storage)
    a.step(3)
    B = lbmx.Batch([a])
    B.step(3)
    B.close()
    a.step(2)
    a.step(1, flags=lbmx.STEP_SUMS)
    b.step(9)
    assert np.array_equal(np.nan_to_num(a.populations()), np.nan_to_num(b.populations()))


@pytest.mark.parametrize("storage", [0, 1, 2])
@pytest.mark.parametrize("nx", [96, 99])
def test_sums_match_the_stored_moments(storage, nx):
    # widths short of a whole tile: the sums must cover exactly the lattice's
    # nodes (tile lanes past the edge hold no nodes), in both step parities
    c = C.random_state(C.cavity_moving_wall(nx, 70, op=C.MRT), seed=10)
    L = C.make_lattice(c, storage=storage)
    for k in (3, 4):
        L.step(1 if k == 4 else 3)
        rho, u, s = L.moments()
        r64 = rho.astype(np.float64)
        # fixed-point terms of 2^-30; interior units add their two nodes in
        # FP32 first (one rounding of about 1e-7 per pair)
        assert abs(s[0] - r64.sum()) <= 2e-7 * r64.sum()
        assert abs(s[1] - (r64 * u[0]).sum()) <= 1e-6 * np.abs(r64 * u[0]).sum()
        assert abs(s[2] - (r64 * u[1]).sum()) <= 1e-6 * np.abs(r64 * u[1]).sum()


def kinetic_energy_of(rho, u):
    r64, u64 = rho.astype(np.float64), u.astype(np.float64)
    return 0.5 * (r64 * (u64[0] ** 2 + u64[1] ** 2)).sum()


@pytest.mark.parametrize("storage", [0, 1])
@pytest.mark.parametrize("nx", [96, 99])
def test_kinetic_energy_matches_the_stored_moments(storage, nx):
    # LBMX_STEP_KINETIC_ENERGY: 1/2 sum rho |u|^2 reduced inside the step, in
    # both step parities, on widths short of a whole tile
    c = C.random_state(C.cavity_moving_wall(nx, 70, op=C.MRT), seed=11)
    L = C.make_lattice(c, storage=storage)
    for n in (3, 1):
        L.step(n, flags=lbmx.STEP_STORE_MOMENTS | lbmx.STEP_KINETIC_ENERGY)
        rho, u, _ = L.moments()
        ref = kinetic_energy_of(rho, u)
        ke = L.kinetic_energy()
        # fixed-point terms of 2^-30; interior units add their two nodes' terms
        # in FP32 first
        assert abs(ke - ref) <= 1e-6 * ref + rho.size * 1e-9, (ke, ref)
    # a step that reduces the sums without the flag reports no kinetic energy
    L.step(1)
    assert L.kinetic_energy() == 0.0


def test_kinetic_energy_series():
    # the four-wide series: mass and momentum bit for bit as without the
    # flag, the kinetic energy bit for bit as single steps that store it;
    # into pageable host memory (a copy per step) and device memory (written
    # by the step kernel itself)
    import torch
    c = C.random_state(C.cavity_moving_wall(96, 72, op=C.MRT), seed=12)
    n = 6
    plain = C.make_lattice(c).step_sums(n)
    host = C.make_lattice(c).step_sums(n, lbmx.STEP_KINETIC_ENERGY)
    d = C.make_lattice(c)
    dev = torch.zeros(4 * n, dtype=torch.float64, device="cuda")
    d._check(d.lib.lbmx_step_sums(d.h, n, lbmx.STEP_KINETIC_ENERGY, dev.data_ptr()))
    d.synchronize()
    dev = dev.cpu().numpy().reshape(n, 4)
    r = C.make_lattice(c)
    single = []
    for _ in range(n):
        r.step(1, flags=lbmx.STEP_STORE_MOMENTS | lbmx.STEP_KINETIC_ENERGY)
        single.append(r.kinetic_energy())
    assert host.shape == (n, 4) and plain.shape == (n, 3)
    np.testing.assert_array_equal(host[:, :3], plain)
    np.testing.assert_array_equal(dev, host)
    np.testing.assert_array_equal(host[:, 3], np.array(single))
    assert np.all(host[:, 3] > 0)


def test_kinetic_energy_decays_at_the_taylor_green_rate():
    # u ~ exp(-nu (kx^2 + ky^2) t), so the kinetic energy decays at twice that
    # rate; BGK on 64 x 64 nodes (k dx = 0.098) is within a fraction of a percent
    c = C.taylor_green(64, 64, op=C.BGK, nu=0.01, u0=0.04)
    L = C.make_lattice(c)
    s = L.step_sums(600, lbmx.STEP_KINETIC_ENERGY)
    ke = s[:, 3]
    k2 = 2 * (2 * np.pi / 64) ** 2
    rate = -np.log(ke[599] / ke[99]) / 500.0
    assert abs(rate / (2 * 0.01 * k2) - 1.0) < 2e-2, rate / (2 * 0.01 * k2)
    # the mass moves only by the FP32 rounding of the populations: about
    # 1.4e-8 per node per step, 8e-6 of the mass in 600 steps, as much as a
    # plain float32 numpy BGK step drifts on this case (float64: 1e-16)
    assert np.all(np.abs(s[:, 0] - 64 * 64) <= 5e-5 * 64 * 64)
