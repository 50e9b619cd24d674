"""The seeded synthetic workloads against the configurations they stand for
(CPU only): the bench grid, the batched domain list, the closure layouts and
the large grid.  Sizes, ranges and clearances are checked on the generated
inputs themselves."""
import numpy as np
import pytest


def test_bench_workload_grid():
    """4096 x 2048, 200 seeded circles with radii in [4, 32], none within 64
    cells of the inlet (the explicit count and radii are kept; the solid
    fraction they give is reported, not forced)."""
    import bench
    m = bench.workload_mask()
    assert m.shape == (bench.NY, bench.NX) == (2048, 4096)
    assert m.dtype == np.uint8 and set(np.unique(m)) <= {0, 1}
    assert not m[:, :64].any()  # centres at x >= 64 + r: nothing left of column 64
    frac = m.mean()
    assert 0.015 < frac < 0.05
    assert m is not bench.workload_mask() and np.array_equal(m, bench.workload_mask())  # seeded


def test_batched_workload_ranges():
    from lbm_gb300 import batch
    nx, ny, om, u, masks = batch.batched_workload(512, 1)
    assert len(masks) == nx.size == ny.size == om.size == u.size == 512
    assert (nx % 32 == 0).all() and nx.min() >= 128 and nx.max() <= 1024
    assert (ny % 32 == 0).all() and ny.min() >= 64 and ny.max() <= 512
    tau = 1.0 / om.astype(np.float64)
    assert tau.min() >= 0.51 - 1e-6 and tau.max() <= 0.8 + 1e-6
    assert u.min() >= 0.02 - 1e-7 and u.max() <= 0.1 + 1e-7
    fr = np.array([m.mean() for m in masks])
    assert np.median(fr) > 0.05 and fr.max() < 0.25
    for w, h, m in zip(nx, ny, masks):
        assert m.shape == (h, w)
        assert not m[:, :max(8, int(w) // 10)].any()  # inlet clearance
        assert not m[:, int(w) - max(16, int(w) // 5):].any()  # wake before the outflow
    # widths and heights cover their ranges
    assert nx.min() <= 192 and nx.max() >= 960 and ny.min() <= 96 and ny.max() >= 480


@pytest.mark.parametrize("index", [0, 65])
def test_closure_layouts(index):
    """Fine 2048 x 1024 layouts of circles with radii in [6, 20] up to 8 %
    solid, none within 64 cells of the inlet; the coarse mask is the 4 x 4
    block majority."""
    from lbm_gb300 import closure as cl
    from lbm_gb300.geometry import random_circles
    m = random_circles(2048, 1024, 10 ** 6, 6.0, 20.0, 1000 + index, inlet_clearance=64, target_fraction=0.08)
    assert m.shape == (1024, 2048)
    assert 0.08 <= m.mean() < 0.09
    assert not m[:, :64].any()
    c = cl.coarse_solid(m, 4)
    assert c.shape == (256, 512)
    blocks = m.reshape(256, 4, 512, 4).sum(axis=(1, 3))
    np.testing.assert_array_equal(c, (blocks > 8).astype(np.uint8))
    assert cl.coarse_tau(0.52, 4) == pytest.approx(0.505)


def test_large_grid_layout():
    """16384 x 8192 with circles of radius 8-64 at about 8 % solid."""
    from lbm_gb300.geometry import random_circles
    m = random_circles(16384, 8192, 10 ** 7, 8, 64, 1, inlet_clearance=64, target_fraction=0.08)
    assert m.shape == (8192, 16384)
    assert 0.08 <= m.mean() < 0.082
    assert not m[:, :64].any()
