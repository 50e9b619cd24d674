"""A channel lattice split into y-slabs across ranks (one GPU each), with the
halo exchange overlapped with the interior rows.

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
direction per step.

Overlapped step (`SlabLattice.step` with an exchanger that has `overlap`):
  1. the edge rows 1 and h of the next step (lbm_step_rows), then their
     crossing populations into the send buffers;
  2. the exchange starts (on its own CUDA stream for device buffers);
  3. the interior rows 2 .. h-1 complete the step, while the rows travel;
  4. the received rows go into the ghost rows of the new state.
The ghost rows are never computed; real rows read only their crossing
populations and solid bits, so the slabs together advance exactly as one
lattice would.  Without `overlap` (host exchangers over plain lattices) the
whole local lattice steps, then the exchange overwrites the ghost rows.

Exchangers:
  * `LocalExchanger`: slabs held by one process; host copies, or, with
    device=True, the overlapped schedule with device buffers (every slab's
    lattice on one CUDA stream, so the copies need no other ordering);
  * `DistExchanger`: one slab per rank over torch.distributed.  With the
    NCCL backend the halo rows stay on the device and move on a side stream
    while the interior rows run; with gloo they are staged through host
    memory.  Every wait is bounded (a timeout for host waits, the process
    group's timeout for NCCL).
"""
import datetime

import numpy as np

from . import EDGE_CHANNEL, F32

SOUTH = (5, 6, 7)  # slots moving to larger row index
NORTH = (0, 1, 2)


def _is_device(buf):
    return hasattr(buf, "data_ptr")


class SlabLattice:
    """Rank `rank`'s slab of an nx x ny channel lattice.  `make_lattice(nx,
    rows)` builds the local lattice (default: lbm_gb300.Lattice in channel
    mode with the given omega and storage); the exchanger is attached with
    `attach`.  `rounding` = (mode, seed) sets the local lattice's rounding
    (Lattice.set_rounding); its row origin is the slab's first row less one
    (the ghost row), so stochastic rounding matches the undivided lattice."""

    def __init__(self, nx, ny, omega, rank, world, storage=F32, u_in=0.1, make_lattice=None, rounding=None):
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
        if hasattr(self.lat, "set_row_origin"):
            self.lat.set_row_origin(self.y0 - 1)
        if rounding is not None:
            self.lat.set_rounding(*rounding)
        self.exchanger = None
        self.bufs = None

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

    # -- halo buffers: 3 planes x nx storage words each ------------------------
    def make_buffers(self, device):
        """send_s / send_n (this slab's crossing rows) and recv_s / recv_n (the
        neighbours'), as device tensors or host arrays."""
        dt = np.dtype(self.lat.storage_dtype)
        if device:
            import torch
            n = 3 * self.nx * dt.itemsize
            self.bufs = {k: torch.empty(n, dtype=torch.uint8, device="cuda")
                         for k in ("send_s", "send_n", "recv_s", "recv_n")}
        else:
            self.bufs = {k: np.zeros((3, 1, self.nx), dt) for k in ("send_s", "send_n", "recv_s", "recv_n")}
        return self.bufs

    def _read(self, y, slots, buf):
        if _is_device(buf):
            self.lat.read_rows_device(y, 1, slots, buf.data_ptr())
        else:
            buf[...] = self.lat.read_rows(y, 1, slots)

    def _write(self, y, slots, buf):
        if _is_device(buf):
            self.lat.write_rows_device(y, 1, slots, buf.data_ptr())
        else:
            self.lat.write_rows(y, slots, buf)

    # -- the overlapped step, in its three parts ---------------------------------
    def begin_step(self, moments=False):
        """Edge rows of the next step, then their crossing rows into the send buffers."""
        h = self.h
        self.lat.step_rows(1, 2, moments=moments)
        self.lat.step_rows(h, h + 1, complete=h == 2, moments=moments)
        self._read(h, SOUTH, self.bufs["send_s"])
        self._read(1, NORTH, self.bufs["send_n"])

    def interior(self, moments=False):
        """The interior rows; the step is complete afterwards."""
        if self.h > 2:
            self.lat.step_rows(2, self.h, complete=True, moments=moments)

    def end_step(self, recv_s, recv_n):
        """The neighbours' crossing rows into the ghost rows of the new state."""
        self._write(0, SOUTH, recv_s)
        self._write(self.h + 1, NORTH, recv_n)

    def step(self, n=1, moments_last=True):
        ex = self.exchanger
        for i in range(n):
            if getattr(ex, "overlap", False):
                m = moments_last and i == n - 1
                self.begin_step(m)
                handle = ex.start(self)
                self.interior(m)
                ex.finish(self, handle)
            else:
                self.lat.iterate(1)
                ex.exchange()


class LocalExchanger:
    """Slabs of one process (in rank order), advanced by run_local.
    Default: whole-lattice steps and host copies.  overlap=True: the
    overlapped schedule with halo buffers in host memory, or with device=True
    in device memory (every slab's lattice then queues on one CUDA stream)."""

    def __init__(self, slabs, device=False, overlap=None):
        self.slabs = slabs
        self.device = device
        self.overlap = device if overlap is None else overlap
        if self.overlap:
            for s in slabs:
                s.make_buffers(device)

    def exchange(self):
        outs = [(s.lat.read_rows(s.h, 1, SOUTH), s.lat.read_rows(1, 1, NORTH)) for s in self.slabs]
        W = len(self.slabs)
        for r, s in enumerate(self.slabs):
            s.lat.write_rows(0, SOUTH, outs[(r - 1) % W][0])
            s.lat.write_rows(s.h + 1, NORTH, outs[(r + 1) % W][1])


class DistExchanger:
    """One slab per rank over torch.distributed point-to-point messages.

    With the NCCL backend (device=None picks it from the process group) the
    halo rows stay in device buffers and move on a side stream that waits for
    the edge rows and is waited for before the ghost rows are written, so the
    interior rows of the step run while they travel.  Otherwise the rows are
    staged through host memory and each wait is bounded by `timeout_s`.
    overlap=None takes the overlapped schedule whenever the lattice can step
    row ranges; overlap=False keeps whole-lattice steps."""

    def __init__(self, slab, timeout_s=30.0, device=None, overlap=None):
        import torch
        import torch.distributed as dist
        self.torch, self.dist = torch, dist
        self.slab = slab
        self.timeout = datetime.timedelta(seconds=timeout_s)
        if device is None:
            device = dist.is_initialized() and dist.get_backend() == "nccl"
        self.device = device
        self.overlap = device or (hasattr(slab.lat, "step_rows") if overlap is None else overlap)
        if self.overlap:
            slab.make_buffers(device)
            if device:
                self.side = torch.cuda.Stream()

    # whole-lattice steps with host-staged rows (plain lattices)
    def exchange(self):
        s = self.slab
        if s.bufs is None:
            s.make_buffers(False)
        s.bufs["send_s"][...] = s.lat.read_rows(s.h, 1, SOUTH)
        s.bufs["send_n"][...] = s.lat.read_rows(1, 1, NORTH)
        self._host_p2p(s.bufs)
        s.end_step(s.bufs["recv_s"], s.bufs["recv_n"])

    def _host_p2p(self, b):
        torch, dist, s = self.torch, self.dist, self.slab
        r, W = s.rank, s.world
        up, down = (r - 1) % W, (r + 1) % W
        t = {k: torch.from_numpy(v.reshape(-1).view(np.uint8)) for k, v in b.items()}
        if W == 1:
            t["recv_s"].copy_(t["send_s"])
            t["recv_n"].copy_(t["send_n"])
            return
        ops = [dist.P2POp(dist.isend, t["send_s"], down), dist.P2POp(dist.irecv, t["recv_s"], up),
               dist.P2POp(dist.isend, t["send_n"], up), dist.P2POp(dist.irecv, t["recv_n"], down)]
        for w in dist.batch_isend_irecv(ops):
            if not w.wait(self.timeout):
                raise TimeoutError("halo exchange with ranks %d / %d timed out" % (up, down))

    # the overlapped step
    def start(self, s):
        if not self.device:
            self._host_p2p(s.bufs)  # the edge rows were read synchronously
            return None
        torch, dist = self.torch, self.dist
        main = _stream_of(s.lat)
        self.side.wait_stream(main)  # the send buffers hold the edge rows
        b = s.bufs
        r, W = s.rank, s.world
        up, down = (r - 1) % W, (r + 1) % W
        with torch.cuda.stream(self.side):
            if W == 1:
                b["recv_s"].copy_(b["send_s"])
                b["recv_n"].copy_(b["send_n"])
                return None
            ops = [dist.P2POp(dist.isend, b["send_s"], down), dist.P2POp(dist.irecv, b["recv_s"], up),
                   dist.P2POp(dist.isend, b["send_n"], up), dist.P2POp(dist.irecv, b["recv_n"], down)]
            return dist.batch_isend_irecv(ops)

    def finish(self, s, handle):
        if self.device:
            torch = self.torch
            with torch.cuda.stream(self.side):
                for w in handle or ():
                    w.wait()  # orders the side stream after the transfers
            _stream_of(s.lat).wait_stream(self.side)
        s.end_step(s.bufs["recv_s"], s.bufs["recv_n"])


def _stream_of(lat):
    """The lattice's CUDA stream as a torch stream (0: the legacy default stream)."""
    import torch
    p = lat.get_stream()
    return torch.cuda.ExternalStream(p) if p else torch.cuda.default_stream()


def run_local(slabs, n):
    """Advance slabs held by one process together: whole-lattice steps and
    host copies, or (LocalExchanger with overlap) the overlapped schedule,
    each slab's ghost rows taken from its neighbours' send buffers."""
    ex = slabs[0].exchanger
    if getattr(ex, "overlap", False):
        W = len(slabs)
        for i in range(n):
            m = i == n - 1
            for s in slabs:
                s.begin_step(m)
            for s in slabs:
                s.interior(m)
            for r, s in enumerate(slabs):
                s.end_step(slabs[(r - 1) % W].bufs["send_s"], slabs[(r + 1) % W].bufs["send_n"])
        return
    for _ in range(n):
        for s in slabs:
            s.lat.iterate(1)
        ex.exchange()
