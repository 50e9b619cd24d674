"""Host-side pieces of the learned closure (CPU only): the block average of
the fine velocity, the error measure, the coarse solid mask, the smoothing
window and the per-cell rollout-label fit, the last with the coarse runs
replaced by synthetic fields whose error is a known parabola in delta_tau."""
import numpy as np
import pytest


def test_block_average_over_fluid_cells():
    from lbm_gb300 import closure as cl
    rng = np.random.default_rng(0)
    u = rng.standard_normal((2, 8, 12))
    mask = np.zeros((8, 12), np.uint8)
    mask[0:2, 0:2] = 1  # a partly solid block
    mask[4:8, 8:12] = 1  # and a fully solid one (its average is 0)
    got = cl.block_average(u, mask, 4)
    assert got.shape == (2, 2, 3)
    fl = mask == 0
    for by in range(2):
        for bx in range(3):
            sel = fl[4 * by:4 * by + 4, 4 * bx:4 * bx + 4]
            blk = u[:, 4 * by:4 * by + 4, 4 * bx:4 * bx + 4]
            want = blk[:, sel].mean(axis=1) if sel.any() else np.zeros(2)
            np.testing.assert_allclose(got[:, by, bx], want, rtol=1e-12)


def test_rel_error_skips_solids_and_inlet_and_flags_divergence():
    from lbm_gb300 import closure as cl
    uf = np.ones((2, 4, 5))
    uc = uf.copy()
    uc[:, :, 0] = 100.0  # inlet column: ignored
    solid = np.zeros((4, 5), np.uint8)
    solid[1, 2] = 1
    uc[:, 1, 2] = -7.0  # solid: ignored
    assert cl.rel_error(uc, uf, solid) == 0.0
    uc[0, 2, 3] = 1.5
    n_fluid = 4 * 4 - 1
    assert cl.rel_error(uc, uf, solid) == pytest.approx(0.5 / np.sqrt(2 * n_fluid))
    uc[1, 3, 4] = np.nan
    assert cl.rel_error(uc, uf, solid) == float("inf")


def test_box_window_mean_with_replicated_edges():
    from lbm_gb300 import closure as cl
    rng = np.random.default_rng(1)
    a = rng.standard_normal((7, 9))
    got = cl._box(a, 2)
    p = np.pad(a, 2, mode="edge")
    want = np.array([[p[y:y + 5, x:x + 5].mean() for x in range(9)] for y in range(7)])
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12)


def test_coarse_solid_is_the_block_majority():
    from lbm_gb300 import closure as cl
    m = np.zeros((8, 8), np.uint8)
    m[0:4, 0:4].flat[:9] = 1  # 9 of 16: solid
    m[0:4, 4:8].flat[:8] = 1  # 8 of 16: fluid (a tie stays fluid)
    np.testing.assert_array_equal(cl.coarse_solid(m, 4), np.array([[1, 0], [0, 0]], np.uint8))


def test_rollout_labels_find_each_cells_parabola_minimum(monkeypatch):
    """Synthetic rollouts: the coarse velocity at delta_tau = d differs from
    the fine one by (d - d*(x, y)) in one component, so each cell's squared
    error is a parabola with its minimum at d*.  d* is constant over bands of
    5 columns, so the cells whose 5 x 5 smoothing window stays inside one band
    (edges are replicated) must get d* back where it lies inside the
    candidate range, and the range's end outside it; a diverged candidate is
    dropped from the fit and from the range."""
    from lbm_gb300 import closure as cl
    H, W = 10, 15
    dstar = np.zeros((H, W))
    dstar[:, 0:5], dstar[:, 5:10], dstar[:, 10:15] = 0.013, 0.031, 0.5
    uf = np.zeros((2, H, W))
    uf[1] = 1.0  # a nonzero reference for the relative errors
    diverge = {}

    def fake_run_average(nx, ny, tau, u, mask, steps, every, avg_from, seed, **kw):
        d = tau - 0.505
        uc = np.zeros((2, ny, nx))
        uc[0] = d - dstar
        uc[1] = 1.0
        if diverge.get("at") is not None and abs(d - diverge["at"]) < 1e-9:
            uc[:] = np.nan
        return uc, 0.0, 0

    monkeypatch.setattr(cl, "run_average", fake_run_average)
    mask = np.zeros((H, W), np.uint8)
    label, weight, rels = cl.rollout_labels(mask, 0.505, 0.06, 100, 10, uf, 0)
    assert len(rels) == len(cl.CANDIDATES)
    np.testing.assert_allclose(label[:, 0:3], 0.013, atol=1e-9)
    np.testing.assert_allclose(label[:, 7], 0.031, atol=1e-9)
    np.testing.assert_allclose(label[:, 12:15], max(cl.CANDIDATES), atol=1e-12)  # clipped to the range
    assert ((label[:, 3:7] > 0.013) & (label[:, 3:7] < 0.031)).all()  # windows across two bands: in between
    assert (weight[:, 1:] > 0).all() and (weight[:, 0] == 0).all()  # inlet column carries no weight
    assert weight[:, 1:].mean() == pytest.approx(1.0)
    # the smallest candidate diverges: it leaves the fit and the lower end of the range
    diverge["at"] = 0.0
    label, weight, rels = cl.rollout_labels(mask, 0.505, 0.06, 100, 10, uf, 0)
    assert rels[0] == float("inf")
    assert label.min() >= sorted(cl.CANDIDATES)[1] - 1e-12
    np.testing.assert_allclose(label[:, 7], 0.031, atol=1e-9)
