"""A channel lattice split into y-slabs across ranks (one GPU each), with
host-staged halo exchange.

The reference runs one lattice on one adapter; this is the decomposition of
a single large grid for several GPUs.  Rank r of W owns global rows
[r h, (r + 1) h) (h = ny / W) in a local lattice of h + 2 rows: local row 0
and row h + 1 are ghost rows that stand for the neighbouring slabs' edge
rows, so the local lattice's periodic wrap in y never reaches across the
slab.  After every step the populations that cross a cut are exchanged:
the last real row's south-moving slots (5 sw, 6 s, 7 se) go to the next
rank's top ghost row, the first real row's north-moving slots (0 nw, 1 n,
2 ne) to the previous rank's bottom ghost row (rank W - 1 and rank 0 are
neighbours: the channel is periodic in y).  Ghost rows also carry the
neighbours' solid bits.  That is 3 planes x nx words per cut face and
direction per step; the ghost rows' own (wrong) step results are always
overwritten before anything reads them, so the slabs together advance
exactly as one lattice would.

`Exchanger` moves the rows: `DistExchanger` over torch.distributed (gloo on
host buffers; every wait bounded by a timeout, after which the step raises),
`LocalExchanger` between slabs held by one process.
"""
import datetime

import numpy as np

from . import EDGE_CHANNEL, F32

SOUTH = (5, 6, 7)  # slots moving to larger row index
NORTH = (0, 1, 2)


class LocalExchanger:
    """Slabs of one process (in rank order): exchange by copying."""

    def __init__(self, slabs):
        self.slabs = slabs

    def exchange(self):
        outs = [(s.lat.read_rows(s.h, 1, SOUTH), s.lat.read_rows(1, 1, NORTH)) for s in self.slabs]
        W = len(self.slabs)
        for r, s in enumerate(self.slabs):
            s.lat.write_rows(0, SOUTH, outs[(r - 1) % W][0])
            s.lat.write_rows(s.h + 1, NORTH, outs[(r + 1) % W][1])


class DistExchanger:
    """One slab per rank over torch.distributed point-to-point messages."""

    def __init__(self, slab, timeout_s=30.0):
        import torch
        import torch.distributed as dist
        self.torch, self.dist = torch, dist
        self.slab = slab
        self.timeout = datetime.timedelta(seconds=timeout_s)

    def exchange(self):
        torch, dist, s = self.torch, self.dist, self.slab
        r, W = s.rank, s.world
        up, down = (r - 1) % W, (r + 1) % W
        send_s = torch.from_numpy(s.lat.read_rows(s.h, 1, SOUTH).view(np.uint8).copy())
        send_n = torch.from_numpy(s.lat.read_rows(1, 1, NORTH).view(np.uint8).copy())
        recv_s = torch.empty_like(send_s)
        recv_n = torch.empty_like(send_n)
        if W == 1:
            recv_s.copy_(send_s)
            recv_n.copy_(send_n)
        else:
            ops = [dist.P2POp(dist.isend, send_s, down), dist.P2POp(dist.irecv, recv_s, up),
                   dist.P2POp(dist.isend, send_n, up), dist.P2POp(dist.irecv, recv_n, down)]
            for w in dist.batch_isend_irecv(ops):
                if not w.wait(self.timeout):
                    raise TimeoutError("halo exchange with ranks %d / %d timed out" % (up, down))
        dt = s.lat.storage_dtype
        s.lat.write_rows(0, SOUTH, recv_s.numpy().view(dt).reshape(3, 1, s.nx))
        s.lat.write_rows(s.h + 1, NORTH, recv_n.numpy().view(dt).reshape(3, 1, s.nx))


class SlabLattice:
    """Rank `rank`'s slab of an nx x ny channel lattice.  `make_lattice(nx,
    rows)` builds the local lattice (default: lbm_gb300.Lattice in channel
    mode with the given omega and storage); the exchanger is attached with
    `attach`."""

    def __init__(self, nx, ny, omega, rank, world, storage=F32, u_in=0.1, make_lattice=None):
        if ny % world or ny // world < 2:
            raise ValueError("ny = %d does not split into %d slabs of >= 2 rows" % (ny, world))
        self.nx, self.ny, self.rank, self.world = nx, ny, rank, world
        self.h = ny // world
        self.y0 = rank * self.h
        if make_lattice is None:
            from . import Lattice

            def make_lattice(x, y):
                lat = Lattice(x, y, omega, EDGE_CHANNEL, storage)
                lat.set_inlet_velocity(u_in)
                return lat
        self.lat = make_lattice(nx, self.h + 2)
        self.exchanger = None

    def attach(self, exchanger):
        self.exchanger = exchanger

    def local_rows(self):
        """Global row of each local row (ghosts included)."""
        return (self.y0 - 1 + np.arange(self.h + 2)) % self.ny

    def set_mask(self, global_mask):
        self.lat.draw_mask(np.asarray(global_mask)[self.local_rows()])

    def write_populations(self, global_pops):
        """Start from a global state [9, ny, nx] (the slab's rows and the ghost rows)."""
        self.lat.write_populations(np.asarray(global_pops)[:, self.local_rows()])

    def populations(self, f64=False):
        return self.lat.populations(f64=f64)[:, 1:self.h + 1] if f64 else self.lat.populations()[:, 1:self.h + 1]

    def field(self, name):
        return self.lat.field(name)[1:self.h + 1]

    def step(self, n=1):
        for _ in range(n):
            self.lat.iterate(1)
            self.exchanger.exchange()


def run_local(slabs, n):
    """Advance slabs held by one process together (LocalExchanger)."""
    ex = slabs[0].exchanger
    for _ in range(n):
        for s in slabs:
            s.lat.iterate(1)
        ex.exchange()
