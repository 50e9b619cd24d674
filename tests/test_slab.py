"""y-slab decomposition: two gloo ranks on CPU (numpy stand-in lattice per
slab, host-staged halo exchange over torch.distributed) reproduce the
undivided lattice exactly; a rank that stops exchanging makes the other's
step fail within its timeout instead of hanging."""
import os
import socket

import numpy as np
import pytest

from slab_cpu_lattice import NumpyLattice, W9


def state(nx, ny, seed):
    rng = np.random.default_rng(seed)
    pops = W9[:, None, None] * (1 + 0.02 * rng.standard_normal((9, ny, nx)))
    pops[5] += 0.01
    mask = (rng.random((ny, nx)) < 0.06).astype(np.uint8)
    mask[:, :3] = 0
    return pops, mask


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, nx, ny, steps, out_dir, mode):
    import torch.distributed as dist
    from lbm_gb300.slab import DistExchanger, SlabLattice
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pops, mask = state(nx, ny, 3)
    slab = SlabLattice(nx, ny, 1.0 / 0.6, rank, world, make_lattice=lambda x, y: NumpyLattice(x, y, 1.0 / 0.6))
    slab.set_mask(mask)
    slab.write_populations(pops)
    slab.attach(DistExchanger(slab, timeout_s=2.0, overlap=mode == "overlap"))
    if mode == "silent" and rank == 1:
        import time
        time.sleep(6.0)  # never exchanges
        return
    try:
        slab.step(steps)
        np.save(os.path.join(out_dir, "slab%d.npy" % rank), slab.populations())
    except Exception as e:  # the timeout path
        with open(os.path.join(out_dir, "err%d.txt" % rank), "w") as f:
            f.write(type(e).__name__ + ": " + str(e))
    finally:
        if mode != "silent":
            dist.destroy_process_group()


def _spawn(world, nx, ny, steps, out_dir, mode="run"):
    import torch.multiprocessing as mp
    mp.start_processes(_worker, args=(world, _free_port(), nx, ny, steps, str(out_dir), mode), nprocs=world,
                       join=True, start_method="spawn")


@pytest.mark.parametrize("world,mode", [(2, "run"), (2, "overlap"), (3, "overlap")])
def test_gloo_ranks_match_the_undivided_lattice(tmp_path, world, mode):
    """Whole-lattice steps then the exchange ("run"), and the overlapped
    schedule: edge rows, exchange, interior rows, ghost rows ("overlap")."""
    nx, ny, steps = 24, 18, 9
    _spawn(world, nx, ny, steps, tmp_path, mode)
    pops, mask = state(nx, ny, 3)
    ref = NumpyLattice(nx, ny, 1.0 / 0.6)
    ref.draw_mask(mask)
    ref.write_populations(pops)
    ref.iterate(steps)
    got = np.concatenate([np.load(tmp_path / ("slab%d.npy" % r)) for r in range(world)], axis=1)
    np.testing.assert_array_equal(got, ref.populations())


def test_a_silent_rank_times_out_the_exchange(tmp_path):
    _spawn(2, 16, 8, 3, tmp_path, mode="silent")
    err = (tmp_path / "err0.txt").read_text()
    assert err, "rank 0 should report the failed exchange"


@pytest.mark.parametrize("overlap", [False, True])
def test_local_exchanger_three_slabs_match(overlap):
    from lbm_gb300.slab import LocalExchanger, SlabLattice, run_local
    nx, ny = 20, 12
    pops, mask = state(nx, ny, 5)
    slabs = [SlabLattice(nx, ny, 1.0 / 0.7, r, 3, make_lattice=lambda x, y: NumpyLattice(x, y, 1.0 / 0.7))
             for r in range(3)]
    ex = LocalExchanger(slabs, overlap=overlap)
    for s in slabs:
        s.set_mask(mask)
        s.write_populations(pops)
        s.attach(ex)
    run_local(slabs, 7)
    ref = NumpyLattice(nx, ny, 1.0 / 0.7)
    ref.draw_mask(mask)
    ref.write_populations(pops)
    ref.iterate(7)
    np.testing.assert_array_equal(np.concatenate([s.populations() for s in slabs], axis=1), ref.populations())
    with pytest.raises(ValueError):
        SlabLattice(nx, 13, 1.0, 0, 3, make_lattice=lambda x, y: None)
