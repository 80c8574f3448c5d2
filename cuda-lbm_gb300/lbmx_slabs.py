"""y-slab decomposition of one D2Q9 lattice over several engine handles.

The reference runs one lattice on one device (src/main.cu:39-41).  Here a
lattice of ny rows is split into slabs of whole rows; each slab is an
ordinary handle whose lattice adds a ghost row on every side that has a
neighbouring slab (lbmx_set_slab).  Ghost rows are never stepped: they hold
copies of the neighbours' boundary rows.

The exchange follows from the in-place (AA) streaming of the engine.  In an
own-node step (even step index) every node reads and writes only its own
slots: nothing crosses a slab edge.  In a neighbour-access step (odd index)
a boundary row reads the populations that stream in from the neighbour's row
and writes those that stream out into it -- in both cases planes 4, 7, 8
(LOWER) of the row below and planes 2, 5, 6 (UPPER) of the row above.  So
around an odd step each slab
  before: fills its lower ghost row's LOWER planes from the lower
          neighbour's top row, its upper ghost row's UPPER planes from the
          upper neighbour's bottom row;
  after:  returns its lower ghost row's LOWER planes into the lower
          neighbour's top row, its upper ghost row's UPPER planes into the
          upper neighbour's bottom row.
That is three populations per edge, each way, twice per pair of steps.  With
CM<OptimalAdapter> the slabs' integer fixed-point average sums
(lbmx_opt_partials) are added over all slabs before every step -- integer
addition, so exactly the whole lattice's sums -- and the averages set on
each slab (lbmx_set_averages).  A split lattice therefore steps bit for bit
as the whole one.

`LocalComm` runs all slabs in this process (on one GPU, device buffers);
`DistComm` runs one slab per torch.distributed rank (gloo with host buffers,
or NCCL with device buffers).  The lattice objects only need halo_get,
halo_put, step, opt_partials, set_averages, synchronize and a step count t.
"""
import numpy as np

LOWER = (1 << 4) | (1 << 7) | (1 << 8)  # south-moving populations: planes 4, 7, 8
UPPER = (1 << 2) | (1 << 5) | (1 << 6)  # north-moving populations: planes 2, 5, 6
CM_OPT = 3
FIX_SCALE = 2.0 ** -30  # units of the fixed-point sums


class SlabGeometry:
    """Rows of slab k of `nslabs` over a lattice of ny rows (whole rows,
    the remainder spread over the first slabs).  Owned rows are
    [y0, y1); the handle's rows are [lo, hi) of the whole lattice (with
    wrap-around when it is periodic in y), ghost rows included."""

    def __init__(self, ny, nslabs, k, periodic_y):
        if nslabs < 1 or not 0 <= k < nslabs or ny < 2 * nslabs:
            raise ValueError("cannot split %d rows into %d slabs" % (ny, nslabs))
        base, extra = divmod(ny, nslabs)
        self.y0 = k * base + min(k, extra)
        self.y1 = self.y0 + base + (1 if k < extra else 0)
        self.k, self.nslabs, self.ny, self.periodic_y = k, nslabs, ny, bool(periodic_y)
        split = nslabs > 1
        self.has_lower = split and (periodic_y or k > 0)
        self.has_upper = split and (periodic_y or k < nslabs - 1)
        self.lower = (k - 1) % nslabs if self.has_lower else None
        self.upper = (k + 1) % nslabs if self.has_upper else None
        self.lo = self.y0 - (1 if self.has_lower else 0)
        self.hi = self.y1 + (1 if self.has_upper else 0)
        self.ny_handle = self.hi - self.lo
        self.ghost_mask = (1 if self.has_lower else 0) | (2 if self.has_upper else 0)
        self.first_owned = 1 if self.has_lower else 0
        self.last_owned = self.first_owned + (self.y1 - self.y0) - 1
        # a single slab keeps the lattice's own periodicity
        self.handle_periodic_y = self.periodic_y and not split

    def rows(self):
        """Whole-lattice row index of every handle row."""
        return np.arange(self.lo, self.hi) % self.ny

    def take(self, a):
        """The handle's rows of an array whose last two axes are (ny, nx)."""
        return np.ascontiguousarray(np.asarray(a)[..., self.rows(), :])

    def owned(self, a):
        """The owned rows of an array over the handle's rows."""
        return np.asarray(a)[..., self.first_owned:self.last_owned + 1, :]

    def flags(self, flags):
        """The handle's flags: the lattice's, with ghost rows plain fluid
        (they are never stepped)."""
        f = self.take(flags).astype(np.uint8)
        if self.has_lower:
            f[0] = 0
        if self.has_upper:
            f[-1] = 0
        return f


def averages_from_sums(sums3, nodes):
    """CM_OPT averages from whole-lattice fixed-point sums, as the engine's
    last CTA forms them: float32(double(sum) * 2^-30 / double(nodes))."""
    s = np.asarray(sums3, np.int64).astype(np.float64) * FIX_SCALE
    return (s / np.float64(nodes)).astype(np.float32)


class LocalComm:
    """All slabs in this process.  `slabs` is a list of (lattice, geometry)
    in slab order; buffers are made by `make_buf(nbytes)` (e.g. CUDA byte
    tensors for engine lattices on one GPU)."""

    def __init__(self, slabs, make_buf):
        self.slabs = slabs
        self.make_buf = make_buf

    def local(self):
        return self.slabs

    def swap(self, sends):
        """sends[i] = (to_lower, to_upper) of local slab i; returns
        (from_lower, from_upper) per slab."""
        out = []
        for L, g in self.slabs:
            fl = sends[g.lower][1] if g.has_lower else None
            fu = sends[g.upper][0] if g.has_upper else None
            out.append((fl, fu))
        return out

    def allreduce(self, vecs):
        tot = np.zeros(3, np.int64)
        for v in vecs:
            tot += np.asarray(v, np.int64)
        return [tot] * len(vecs)


class DistComm:
    """One slab per torch.distributed rank (rank k holds slab k).  Buffers
    are CPU byte tensors for gloo or CUDA byte tensors for NCCL; sends and
    receives are paired non-blocking point-to-point operations."""

    def __init__(self, lattice, geometry, dist, device="cpu"):
        import torch
        self.torch, self.dist, self.device = torch, dist, device
        self.slabs = [(lattice, geometry)]

    def local(self):
        return self.slabs

    def make_buf(self, nbytes):
        return self.torch.empty(nbytes, dtype=self.torch.uint8, device=self.device)

    def swap(self, sends):
        # Messages going up carry tag 1, going down tag 2.  The order is the
        # same on every rank (sends up then down, receives from below then
        # from above), so they also pair where one rank is both neighbours
        # (two slabs of a periodic lattice) and tags are not matched.
        (to_lower, to_upper), = sends
        L, g = self.slabs[0]
        ops, fl, fu = [], None, None
        if g.has_upper:
            ops.append(self.dist.P2POp(self.dist.isend, to_upper, g.upper, tag=1))
        if g.has_lower:
            ops.append(self.dist.P2POp(self.dist.isend, to_lower, g.lower, tag=2))
        if g.has_lower:
            fl = self.make_buf(to_lower.numel())
            ops.append(self.dist.P2POp(self.dist.irecv, fl, g.lower, tag=1))
        if g.has_upper:
            fu = self.make_buf(to_upper.numel())
            ops.append(self.dist.P2POp(self.dist.irecv, fu, g.upper, tag=2))
        if ops:
            for r in self.dist.batch_isend_irecv(ops):
                r.wait()
        return [(fl, fu)]

    def allreduce(self, vecs):
        t = self.torch.tensor(np.asarray(vecs[0], np.int64), dtype=self.torch.int64, device=self.device)
        self.dist.all_reduce(t)
        return [t.cpu().numpy()]


def _bytes(L, mask):
    return bin(mask).count("1") * L.nx * L.elem_size


def step_slabs(comm, nsteps, whole_nodes, flags=None):
    """Advance every slab of `comm` by nsteps steps in lockstep.  `flags`
    are lbmx_step_ex flags for each single step (default: store moments)."""
    slabs = comm.local()
    op = slabs[0][0].op
    for _ in range(int(nsteps)):
        odd = (slabs[0][0].t + 1) & 1
        if odd:
            _exchange(comm, before=True)
        if op == CM_OPT:
            tot = comm.allreduce([L.opt_partials() for L, _ in slabs])
            for (L, _), t in zip(slabs, tot):
                L.set_averages(averages_from_sums(t, whole_nodes))
        for L, _ in slabs:
            if flags is None:
                L.step(1)
            else:
                L.step(1, flags)
        if odd:
            _exchange(comm, before=False)


def _exchange(comm, before):
    slabs = comm.local()
    sends = []
    for L, g in slabs:
        to_lower = to_upper = None
        if g.has_lower:
            # before: my bottom row's UPPER planes feed the lower neighbour's
            # upper ghost; after: my lower ghost's LOWER planes go back
            row, mask = (g.first_owned, UPPER) if before else (0, LOWER)
            to_lower = L.halo_get(row, mask, comm.make_buf(_bytes(L, mask)))
        if g.has_upper:
            row, mask = (g.last_owned, LOWER) if before else (g.ny_handle - 1, UPPER)
            to_upper = L.halo_get(row, mask, comm.make_buf(_bytes(L, mask)))
        sends.append((to_lower, to_upper))
    for L, _ in slabs:
        L.synchronize()
    recv = comm.swap(sends)
    for (L, g), (fl, fu) in zip(slabs, recv):
        if fl is not None:
            # before: the lower neighbour's top row (LOWER) into my lower
            # ghost; after: its upper ghost (UPPER) into my bottom row
            L.halo_put(0 if before else g.first_owned, LOWER if before else UPPER, fl)
        if fu is not None:
            L.halo_put(g.ny_handle - 1 if before else g.last_owned, UPPER if before else LOWER, fu)
    for L, _ in slabs:
        L.synchronize()


def make_slab_lattice(lbmx, case, geometry, storage=0, options=0, stream=None, device=0):
    """An engine handle for slab `geometry` of a lattice described by a case
    dict (nx, ny, op, omega, S, periodic, quirks, u_bc, wall_u, rho_out,
    flags, rho, u, force, optional gamma): the slab's rows of every field,
    ghost rows included, plain fluid flags on the ghost rows."""
    g = geometry
    px, _ = case["periodic"]
    L = lbmx.Lattice(case["nx"], g.ny_handle, op=case["op"], omega=case["omega"], S=case["S"],
                     periodic=(px, g.handle_periodic_y), storage=storage, quirks=case["quirks"], options=options,
                     u_bc=case["u_bc"], wall_u=case["wall_u"], rho_out=case["rho_out"], device=device, stream=stream)
    L.set_slab(g.ghost_mask, g.lo, g.ny if g.periodic_y and g.nslabs > 1 else 0)
    L.set_flags(g.flags(case["flags"]))
    force = None if case["force"] is None else g.take(np.asarray(case["force"], np.float32))
    L.init(g.take(np.asarray(case["rho"], np.float32)), g.take(np.asarray(case["u"], np.float32)), force)
    if case.get("gamma") is not None:
        L.set_brinkman(g.take(np.asarray(case["gamma"], np.float32)))
    return L
