"""Batched lattices: many independent channel domains advanced by one
persistent launch per step (include/lbm_batch.h).

The reference has no batched form; each domain here behaves exactly like a
`Lattice(nx, ny, omega, EDGE_CHANNEL, storage)` with `set_inlet_velocity(u)`,
`init_equilibrium(1, u, 0, noise, seed + d)` and `draw_mask(mask)`.

Across several GPUs the domains are dealt out whole (`partition`: longest
processing time first, by cell count), each rank running a Batch of its
share; nothing crosses between ranks but the FP64 conservation sums
(`sharded_totals`).
"""
import ctypes
import json

import numpy as np

from . import FIELD, F32, _check, _ptr, load_library
from .geometry import SplitMix64, random_layout


class Batch:
    def __init__(self, nx, ny, omega, u_in, storage=F32):
        L = load_library()
        self.nx = np.ascontiguousarray(nx, dtype=np.uint32)
        self.ny = np.ascontiguousarray(ny, dtype=np.uint32)
        self.omega = np.ascontiguousarray(omega, dtype=np.float32)
        self.u_in = np.ascontiguousarray(u_in, dtype=np.float32)
        n = self.nx.size
        if not (self.ny.size == self.omega.size == self.u_in.size == n):
            raise ValueError("nx, ny, omega and u_in need one entry per domain")
        self.count, self.storage = n, int(storage)
        h = ctypes.c_void_p()
        _check(L.lbm_batch_create(n, _ptr(self.nx), _ptr(self.ny), _ptr(self.omega), _ptr(self.u_in),
                                  self.storage, ctypes.byref(h)))
        self._h = h
        self._lib = L

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lbm_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self):
        c, cells, steps = ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_uint64()
        _check(self._lib.lbm_batch_info(self._h, ctypes.byref(c), ctypes.byref(cells), ctypes.byref(steps)))
        return c.value, cells.value, steps.value

    def stream(self):
        v = ctypes.c_void_p()
        _check(self._lib.lbm_batch_get_stream(self._h, ctypes.byref(v)))
        return v.value or 0

    def set_mask(self, d, mask):
        m = np.ascontiguousarray(mask, dtype=np.uint8).reshape(-1)
        if m.size != int(self.nx[d]) * int(self.ny[d]):
            raise ValueError("mask of domain %d has %d cells" % (d, m.size))
        _check(self._lib.lbm_batch_set_mask(self._h, int(d), _ptr(m)))

    def init_equilibrium(self, noise=0.0, seed=0):
        _check(self._lib.lbm_batch_init_equilibrium(self._h, float(noise), int(seed)))

    def step(self, n):
        _check(self._lib.lbm_batch_step(self._h, int(n)))

    def synchronize(self):
        _check(self._lib.lbm_batch_synchronize(self._h))

    def field(self, d, name):
        code = FIELD[name] if isinstance(name, str) else int(name)
        out = np.zeros(int(self.nx[d]) * int(self.ny[d]), np.float32)
        _check(self._lib.lbm_batch_read_field(self._h, int(d), code, _ptr(out)))
        return out.reshape(int(self.ny[d]), int(self.nx[d]))

    def populations(self, d):
        out = np.zeros(9 * int(self.nx[d]) * int(self.ny[d]), np.float32)
        _check(self._lib.lbm_batch_read_populations(self._h, int(d), _ptr(out)))
        return out.reshape(9, int(self.ny[d]), int(self.nx[d]))

    def conservation(self):
        """FP64 (mass, x momentum, y momentum) over each domain's fluid cells,
        shape (count, 3) (lbm_batch_conservation)."""
        out = np.zeros(3 * len(self.nx), np.float64)
        _check(self._lib.lbm_batch_conservation(self._h, _ptr(out)))
        return out.reshape(-1, 3)

    def set_rounding(self, mode, seed=0):
        """Rounding of the stored words (Lattice.set_rounding): domain d rounds
        as a single lattice with seed `seed + d`; stochastic rounding needs
        f16 / bf16 storage."""
        _check(self._lib.lbm_batch_set_rounding(self._h, int(mode), int(seed) & 0xFFFFFFFF))

    @property
    def rounding(self):
        """(mode, seed)."""
        m, sd = ctypes.c_int(), ctypes.c_uint32()
        _check(self._lib.lbm_batch_get_rounding(self._h, ctypes.byref(m), ctypes.byref(sd)))
        return m.value, sd.value

    def set_schedule(self, variant=0, dynamic=0, rows=None):
        r = None if rows is None else np.ascontiguousarray(rows, dtype=np.int32)
        _check(self._lib.lbm_batch_set_schedule(self._h, int(variant), int(dynamic), None if r is None else _ptr(r)))

    def autotune(self, steps_per_trial=40):
        buf = ctypes.create_string_buffer(16384)
        _check(self._lib.lbm_batch_autotune(self._h, int(steps_per_trial), buf, len(buf)))
        return json.loads(buf.value.decode())


def partition(nx, ny, world):
    """Deal whole domains out to `world` ranks, longest processing time first:
    domains in decreasing cell count (ties by index), each to the rank with
    the fewest cells so far (ties to the lowest rank).  Returns one ascending
    index array per rank.  No rank ends more than one domain's cells above
    the mean."""
    cells = np.asarray(nx, np.int64) * np.asarray(ny, np.int64)
    order = sorted(range(len(cells)), key=lambda d: (-int(cells[d]), d))
    load = [0] * world
    parts = [[] for _ in range(world)]
    for d in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(d)
        load[r] += int(cells[d])
    return [np.array(sorted(p), np.int64) for p in parts]


def sharded_totals(local, dist=None):
    """Whole-batch FP64 totals from one rank's per-domain conservation sums
    (Batch.conservation of its share): the ranks' column sums are gathered
    and added in rank order, so every rank gets the same bits whatever the
    transport.  Without a process group, the local column sums."""
    mine = np.asarray(local, np.float64).reshape(-1, 3).sum(axis=0)
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return mine
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.from_numpy(mine).to(dev)
    parts = [torch.empty_like(t) for _ in range(dist.get_world_size())]
    dist.all_gather(parts, t)
    total = np.zeros(3, np.float64)
    for p in parts:
        total = total + p.cpu().numpy()
    return total


def batched_workload(count, seed, wmin=128, wmax=1024, hmin=64, hmax=512, fmin=0.05, fmax=0.15, tau=(0.51, 0.8),
                     u=(0.02, 0.1)):
    """Seeded domain list: width uniform in [wmin, wmax] and height uniform in
    [hmin, hmax], both multiples of 32; circle / rectangle barriers up to a
    solid fraction uniform in [fmin, fmax] (the last shape may overshoot),
    none in the first tenth or the last fifth of the columns (a wake region
    before the zero-gradient outflow); tau and inlet velocity uniform in the
    given ranges.  Returns (nx, ny, omega, u_in, masks)."""
    rng = SplitMix64(seed)
    nx, ny, om, uu, masks = [], [], [], [], []
    for d in range(count):
        w = 32 * rng.randint(wmin // 32, wmax // 32)
        h = 32 * rng.randint(hmin // 32, hmax // 32)
        t = rng.uniform(*tau)
        nx.append(w)
        ny.append(h)
        om.append(np.float32(1.0 / t))
        uu.append(np.float32(rng.uniform(*u)))
        frac = rng.uniform(fmin, fmax)
        masks.append(random_layout(w, h, frac, rng.next_u64(), rmin=3.0, rmax=max(4.0, min(w, h) / 10.0),
                                   inlet_clearance=max(8, w // 10), outlet_clearance=max(16, w // 5)))
    return (np.array(nx, np.uint32), np.array(ny, np.uint32), np.array(om, np.float32), np.array(uu, np.float32),
            masks)
