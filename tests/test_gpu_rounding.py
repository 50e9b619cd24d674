"""Stochastic rounding of the 16-bit storage words (lbm_set_rounding): every
kernel variant, edge mode, storage reference and launch path matches the
oracle bit for bit, and the rounding is a function of (seed, step, cell,
direction) only: graph replays, call lengths, row-range steps, slabs and
checkpoint resumes give the same state."""
import numpy as np
import pytest

from test_gpu_parity import assert_same_state, run_pair

pytestmark = pytest.mark.gpu


def sr_pair(lbm, P, nx, ny, storage, edge, store_inlet, kernel, rows, seed, steps, mask_frac=0.1, rng_seed=0):
    rng = np.random.default_rng(rng_seed)
    omega = float(np.float32(rng.uniform(0.7, 1.9)))
    mask = (rng.random((ny, nx)) < mask_frac).astype(np.uint8)
    lat, o = run_pair(lbm, P, nx, ny, omega, edge, storage, storage, 0, mask, ux=0.08, noise=1e-2,
                      seed=int(rng.integers(1 << 30)), rows=rows, kernel=kernel, store_inlet=store_inlet)
    lat.set_rounding(lbm.ROUND_STOCHASTIC, seed)
    o.set_rounding(1, seed)
    lat.iterate(steps)
    o.step(steps)
    return lat, o


@pytest.mark.parametrize("storage", [1, 2])
@pytest.mark.parametrize("edge", [0, 1])
@pytest.mark.parametrize("store_inlet", [False, True])
@pytest.mark.parametrize("nx,ny,rows", [(70, 41, 8), (1100, 700, 9)])
@pytest.mark.parametrize("kernel", [0, 1, 3, 6, 9, 11, 12])
def test_gpu_stochastic_rounding_matches_oracle(lbm, cuda_ok, oracle_mod, storage, edge, store_inlet, nx, ny, rows,
                                                kernel):
    lat, o = sr_pair(lbm, oracle_mod, nx, ny, storage, edge, store_inlet, kernel, rows, seed=0xC0FFEE + kernel,
                     steps=45, rng_seed=nx + 7 * kernel + 3 * storage + edge)
    assert lat.rounding == (lbm.ROUND_STOCHASTIC, 0xC0FFEE + kernel)
    assert_same_state(lat, o)
    lat.close()


@pytest.mark.parametrize("storage,kernel", [(1, 11), (2, 3), (1, 0)])
def test_gpu_stochastic_rounding_call_lengths_and_graphs(lbm, cuda_ok, oracle_mod, storage, kernel):
    """Captured graphs read their step index from a device word set before
    each replay: runs of any call lengths, with and without graphs, equal
    the oracle and one another."""
    P = oracle_mod
    L = lbm.load_library()
    plan = [1, 7, 7, 7, 2, 64, 65, 33, 7, 100]
    states = []
    for graphs in (1, 0):
        lat, o = sr_pair(lbm, P, 300, 70, storage, 1, False, kernel, 8, seed=17, steps=0, rng_seed=3)
        lbm._check(L.lbm_set_graphs(lat.handle, graphs))
        for n in plan:
            lat.iterate(n)
            o.step(n)
        assert lat.get_compute_num() == sum(plan)
        assert_same_state(lat, o)
        states.append(lat.populations())
        lat.close()
    np.testing.assert_array_equal(states[0], states[1])


def test_gpu_stochastic_rounding_seed_mode_and_storage(lbm, cuda_ok, oracle_mod):
    P = oracle_mod
    runs = {}
    for seed in (5, 5, 6):
        lat, o = sr_pair(lbm, P, 130, 60, 1, 1, False, 11, 8, seed=seed, steps=40, rng_seed=9)
        assert_same_state(lat, o)
        runs.setdefault(seed, []).append(lat.populations())
        lat.close()
    np.testing.assert_array_equal(runs[5][0], runs[5][1])
    assert not np.array_equal(runs[5][0], runs[6][0])
    # back to nearest: the round-to-nearest oracle again
    lat, o = sr_pair(lbm, P, 130, 60, 1, 1, False, 11, 8, seed=5, steps=10, rng_seed=9)
    lat.set_rounding(lbm.ROUND_NEAREST)
    o.set_rounding(0)
    assert lat.rounding == (lbm.ROUND_NEAREST, 0)
    lat.iterate(20)
    o.step(20)
    assert_same_state(lat, o)
    lat.close()
    # f32 / f64 storage refuse it; an unknown mode is refused
    with lbm.Lattice(64, 32, 1.2, lbm.EDGE_CHANNEL, lbm.F32) as lat:
        with pytest.raises(lbm.LBMError):
            lat.set_rounding(lbm.ROUND_STOCHASTIC, 1)
        assert lat.rounding == (lbm.ROUND_NEAREST, 0)
    with lbm.Lattice(64, 32, 1.2, lbm.EDGE_CHANNEL, lbm.F16) as lat:
        with pytest.raises(lbm.LBMError):
            lat.set_rounding(2, 1)


def test_gpu_stochastic_rounding_row_ranges(lbm, cuda_ok, oracle_mod):
    """A step taken as row ranges (lbm_step_rows) hashes every row with the
    step's index: the same state as whole steps."""
    P = oracle_mod
    lat, o = sr_pair(lbm, P, 200, 64, 1, 1, True, 11, 8, seed=99, steps=0, rng_seed=4)
    for k in range(12):
        last = k == 11  # every range of the last step writes its moments
        lat.step_rows(0, 5, moments=last)
        lat.step_rows(40, 64, moments=last)
        lat.step_rows(5, 40, complete=True, moments=last)
        o.step(1)
    assert_same_state(lat, o)
    lat.close()


@pytest.mark.parametrize("storage,kernel,slabs,overlap", [(1, 11, 2, False), (2, 3, 3, True), (1, 13, 4, True)])
def test_gpu_stochastic_rounding_slabs_match_one_lattice(lbm, cuda_ok, storage, kernel, slabs, overlap):
    """Slabs set their row origin, so their rounding hashes global rows and the
    decomposition reproduces the undivided lattice bit for bit."""
    from lbm_gb300 import geometry
    from lbm_gb300.slab import LocalExchanger, SlabLattice, run_local
    nx, ny, steps = 300, 96, 31
    mask = geometry.random_layout(nx, ny, 0.1, 7, rmin=3.0, inlet_clearance=10)
    ref = lbm.Lattice(nx, ny, 1.0 / 0.56, lbm.EDGE_CHANNEL, storage)
    ref.set_tuning(8, kernel)
    ref.set_inlet_velocity(0.07)
    ref.init_equilibrium(1.0, 0.07, 0.0, 1e-2, 4)
    ref.draw_mask(mask)
    start = ref.populations(f64=True)
    ss = [SlabLattice(nx, ny, 1.0 / 0.56, r, slabs, storage=storage, u_in=0.07, rounding=(1, 1234))
          for r in range(slabs)]
    ex = LocalExchanger(ss, device=overlap, overlap=overlap)
    for s in ss:
        s.lat.set_tuning(8, kernel)
        s.set_mask(mask)
        s.write_populations(start)
        s.attach(ex)
        assert s.lat.row_origin == s.y0 - 1
    ref.set_rounding(lbm.ROUND_STOCHASTIC, 1234)
    ref.write_populations(start)
    ref.iterate(steps)
    run_local(ss, steps)
    got = np.concatenate([s.populations() for s in ss], axis=1)
    np.testing.assert_array_equal(got, ref.populations())
    for s in ss:
        s.lat.close()
    ref.close()


@pytest.mark.parametrize("storage", [1, 2])
def test_gpu_stochastic_rounding_checkpoint_resume(lbm, cuda_ok, oracle_mod, storage):
    """The rounding mode, seed and row origin travel with a checkpoint: a
    resumed run continues the uninterrupted one bit for bit."""
    P = oracle_mod
    lat, o = sr_pair(lbm, P, 160, 50, storage, 1, True, 11, 8, seed=4242, steps=23, rng_seed=8)
    lat.set_row_origin(-7)
    o.set_row_origin(-7)
    buf = lat.checkpoint()
    info = lbm.checkpoint_info(buf)
    assert (info["rounding"], info["rounding_seed"], info["row_origin"]) == (1, 4242, -7)
    lat.iterate(30)
    o.step(30)
    assert_same_state(lat, o)
    want = lat.populations()
    lat.close()
    with lbm.Lattice(160, 50, 1.3, lbm.EDGE_CHANNEL, storage) as again:
        assert again.rounding == (lbm.ROUND_NEAREST, 0)
        again.restore(buf)
        assert again.rounding == (lbm.ROUND_STOCHASTIC, 4242) and again.row_origin == -7
        again.iterate(30)
        np.testing.assert_array_equal(again.populations(), want)


def test_gpu_stochastic_rounding_full_size(lbm, cuda_ok, oracle_mod):
    """The 4096 x 2048 workload (200 circles, tau 0.55, ux 0.08) in f16 with
    f - w words, default kernel, 200 steps with stochastic rounding: the
    populations equal the oracle's bit for bit on the full grid (graph
    replays with the step index read from the clock word, programmatic
    launches between steps)."""
    from lbm_gb300 import geometry
    P = oracle_mod
    nx, ny = 4096, 2048
    mask = geometry.random_circles(nx, ny, 200, 4, 32, seed=1, inlet_clearance=64)
    lat, o = run_pair(lbm, P, nx, ny, 1.0 / 0.55, 1, lbm.F16, P.P_F16, 0, mask, ux=0.08, noise=1e-4, seed=1,
                      rows=2, kernel=11, sr_seed=0x5EED)
    lat.iterate(200)
    o.step(200)
    np.testing.assert_array_equal(lat.populations(), o.state()[0].astype(np.float32))
    lat.close()
