"""Batched lattices on the GPU: every domain of a batch bit-exact against the
CPU oracle run of that domain alone, under every schedule the autotuner can
pick, across CUDA-graph replays, mask edits and re-initialisation."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (nx, ny): strips narrower than, equal to and wider than 256 columns, ragged
# heights, one domain shorter than a band
SIZES = [(100, 40), (256, 64), (300, 70), (520, 33), (37, 130), (700, 257), (64, 3), (1030, 96), (129, 200)]


def make_batch(lbm, storage, seed=11):
    from lbm_gb300 import batch, geometry
    rng = np.random.default_rng(seed)
    nx = np.array([s[0] for s in SIZES], np.uint32)
    ny = np.array([s[1] for s in SIZES], np.uint32)
    omega = np.array([1.0 / rng.uniform(0.51, 0.8) for _ in SIZES], np.float32)
    u_in = np.array([rng.uniform(0.02, 0.1) for _ in SIZES], np.float32)
    masks = [geometry.random_layout(int(x), int(y), rng.uniform(0.05, 0.15), 100 + d, rmin=2.0,
                                    inlet_clearance=4) for d, (x, y) in enumerate(SIZES)]
    b = batch.Batch(nx, ny, omega, u_in, storage)
    return b, masks


def oracle_for(P, b, d, prec, mask, noise, seed):
    o = P.Oracle(int(b.nx[d]), int(b.ny[d]), float(b.omega[d]), P.EDGE_CHANNEL, prec)
    o.set_inlet(float(b.u_in[d]), apply=False)
    o.init_equilibrium(1.0, float(b.u_in[d]), 0.0, float(np.float32(noise)), seed + d)
    o.set_mask(mask)
    return o


def assert_domain(b, d, o):
    pops, rho, jx, jy = o.state()
    np.testing.assert_array_equal(b.populations(d), pops.astype(np.float32), err_msg="domain %d" % d)
    np.testing.assert_array_equal(b.field(d, "rho"), rho.astype(np.float32), err_msg="domain %d" % d)
    np.testing.assert_array_equal(b.field(d, "jx"), jx.astype(np.float32), err_msg="domain %d" % d)
    np.testing.assert_array_equal(b.field(d, "jy"), jy.astype(np.float32), err_msg="domain %d" % d)


@pytest.mark.parametrize("storage,prec", [(0, 0), (1, 1), (2, 2)])
def test_gpu_batch_matches_oracle_per_domain(lbm, cuda_ok, oracle_mod, storage, prec):
    """47 steps (one plain launch, two graph replays of 20, then plain
    launches), a mask edit on two domains, 3 more steps: every domain equals
    its oracle run bit for bit."""
    P = oracle_mod
    b, masks = make_batch(lbm, storage)
    with b:
        b.init_equilibrium(1e-2, 5)
        orc = []
        for d, m in enumerate(masks):
            b.set_mask(d, m)
            orc.append(oracle_for(P, b, d, prec, m, 1e-2, 5))
        b.step(47)
        for o in orc:
            o.step(47)
        for d in range(b.count):
            assert_domain(b, d, orc[d])
        for d in (1, 5):
            m = masks[d].copy()
            m[:, int(b.nx[d]) // 2] = 1
            m[::3, int(b.nx[d]) // 2] = 0
            b.set_mask(d, m)
            orc[d].set_mask(m)
        b.step(3)
        for o in orc:
            o.step(3)
        for d in range(b.count):
            assert_domain(b, d, orc[d])
        b.synchronize()
        assert b.info()[2] == 50


@pytest.mark.parametrize("storage,prec", [(1, 1), (2, 2)])
@pytest.mark.parametrize("variant,dynamic", [(2, 0), (3, 1), (4, 2), (0, 1)])
def test_gpu_batch_stochastic_rounding_matches_oracle_per_domain(lbm, cuda_ok, oracle_mod, storage, prec, variant,
                                                                 dynamic):
    """Stochastic rounding in the batch: domain d rounds as a single lattice
    with seed + d, through plain launches and graph replays (47 steps), every
    schedule form, bit for bit against its oracle run."""
    P = oracle_mod
    b, masks = make_batch(lbm, storage)
    with b:
        b.set_schedule(variant, dynamic, [32, 64, 32])
        b.set_rounding(lbm.ROUND_STOCHASTIC, 900)
        assert b.rounding == (lbm.ROUND_STOCHASTIC, 900)
        b.init_equilibrium(1e-2, 5)
        orc = []
        for d, m in enumerate(masks):
            b.set_mask(d, m)
            o = oracle_for(P, b, d, prec, m, 1e-2, 5)
            o.set_rounding(1, 900 + d)
            orc.append(o)
        b.step(47)
        for o in orc:
            o.step(47)
        for d in range(b.count):
            assert_domain(b, d, orc[d])
    f32, _ = make_batch(lbm, 0)
    with f32:
        with pytest.raises(lbm.LBMError):
            f32.set_rounding(lbm.ROUND_STOCHASTIC, 1)


# (variant, schedule: 0 static, 1 tickets, 2 static through one ring, band rows); [5, 64, 7] gives
# tiles shorter than the deepest ring, so one ring carries several of a CTA's tiles at once
SCHEDULES = [(v, dyn, rows) for v in range(6) for dyn in (0, 1, 2) for rows in ([32, 32, 32], [5, 64, 7], [3, 2, 3])]


@pytest.mark.parametrize("storage", [0, 1])
def test_gpu_batch_every_schedule_gives_the_same_state(lbm, cuda_ok, storage):
    b, masks = make_batch(lbm, storage, seed=3)
    ref = None
    with b:
        for d, m in enumerate(masks):
            b.set_mask(d, m)
        for v, dyn, rows in SCHEDULES:
            b.set_schedule(v, dyn, rows)
            b.init_equilibrium(1e-2, 9)
            b.step(45)
            got = [b.populations(d) for d in range(b.count)]
            if ref is None:
                ref = got
            else:
                for d in range(b.count):
                    np.testing.assert_array_equal(got[d], ref[d], err_msg="schedule %s domain %d" %
                                                  ((v, dyn, rows), d))


@pytest.mark.parametrize("storage,prec", [(0, 0), (1, 1)])
def test_gpu_batch_one_ring_matches_oracle(lbm, cuda_ok, oracle_mod, storage, prec):
    """The static schedule through one ring (2), with short bands so that a
    CTA's tiles follow each other within a single ring depth: every domain
    bit-exact against its oracle run over graph replays and plain steps."""
    P = oracle_mod
    b, masks = make_batch(lbm, storage, seed=6)
    with b:
        b.set_schedule(3 if storage else 0, 2, [4, 3, 5])
        b.init_equilibrium(1e-2, 5)
        orc = []
        for d, m in enumerate(masks):
            b.set_mask(d, m)
            orc.append(oracle_for(P, b, d, prec, m, 1e-2, 5))
        b.step(23)
        b.step(1)
        for d, o in enumerate(orc):
            o.step(24)
            assert_domain(b, d, o)


def test_gpu_batch_two_cells_per_thread_in_f32(lbm, cuda_ok, oracle_mod):
    P = oracle_mod
    b, masks = make_batch(lbm, 0, seed=4)
    with b:
        b.set_schedule(3, 1, [16, 16, 16])
        b.init_equilibrium(1e-2, 2)
        orc = []
        for d, m in enumerate(masks):
            b.set_mask(d, m)
            orc.append(oracle_for(P, b, d, P.P_F32, m, 1e-2, 2))
        b.step(25)
        for d, o in enumerate(orc):
            o.step(25)
            assert_domain(b, d, o)


def test_gpu_batch_autotune_then_parity(lbm, cuda_ok, oracle_mod):
    P = oracle_mod
    b, masks = make_batch(lbm, 1, seed=8)
    with b:
        for d, m in enumerate(masks):
            b.set_mask(d, m)
        rep = b.autotune(24)
        ch = rep["chosen"]
        assert ch["ring_stages"] in (4, 6, 8) and ch["cells_per_thread"] in (1, 2)
        assert ch["strip_columns"] in (256, 512)
        assert ch["schedule"] in ("dynamic", "static_longest_first", "static_one_ring")
        assert len(rep["trials"]) >= 8 and ch["ms_per_step"] > 0
        b.init_equilibrium(1e-3, 1)
        b.step(41)
        for d in (0, 3, 5, 8):
            o = oracle_for(P, b, d, P.P_F16, masks[d], 1e-3, 1)
            o.step(41)
            assert_domain(b, d, o)


def test_gpu_batch_fields_before_first_step(lbm, cuda_ok, oracle_mod):
    P = oracle_mod
    b, masks = make_batch(lbm, 0)
    with b:
        b.init_equilibrium(1e-2, 3)
        o = oracle_for(P, b, 2, P.P_F32, np.zeros_like(masks[2]), 1e-2, 3)
        pops = o.state()[0]  # the oracle has no moments before its first step: sum its populations
        np.testing.assert_array_equal(b.populations(2), pops.astype(np.float32))
        cx = np.array([-1, 0, 1, -1, 0, 1, -1, 0, 1], np.float64)
        np.testing.assert_allclose(b.field(2, "rho"), pops.sum(0), rtol=1e-6)
        np.testing.assert_allclose(b.field(2, "jx"), np.tensordot(cx, pops, 1), rtol=1e-5, atol=1e-7)


def test_gpu_batch_argument_errors(lbm, cuda_ok):
    from lbm_gb300 import batch
    one = np.ones(1, np.float32)
    with pytest.raises(lbm.LBMError):
        batch.Batch([64], [32], one, one * 0.05, lbm.F64)
    with pytest.raises(lbm.LBMError):
        batch.Batch([2], [32], one, one * 0.05)
    with pytest.raises(lbm.LBMError):
        batch.Batch([64], [32], one * 2.5, one * 0.05)
    with batch.Batch([64, 80], [32, 40], [1.0, 1.2], [0.05, 0.06]) as b:
        out = np.zeros(80 * 40, np.float32)
        assert b._lib.lbm_batch_read_field(b._h, 2, 0, out.ctypes.data) == 1  # LBM_ERR_ARG: no domain 2
        assert b._lib.lbm_batch_set_mask(b._h, 0, None) == 1
        with pytest.raises(lbm.LBMError):
            b.set_schedule(7, 0)
        assert b.info()[:2] == (2, 64 * 32 + 80 * 40)


def test_gpu_sharded_batch_matches_the_whole(lbm, cuda_ok):
    """The domains dealt to two ranks (batch.partition), run as two batches one
    after the other on this GPU: every domain's state and conservation sums
    are those of the undivided batch bit for bit, the gathered totals agree
    with its sums, and each domain's sums agree with a single lattice's
    lbm_conservation of the same run."""
    from lbm_gb300 import batch
    whole, masks = make_batch(lbm, lbm.F32)
    for d, m in enumerate(masks):
        whole.set_mask(d, m)
    whole.init_equilibrium(0.0, 0)
    whole.step(33)
    want = whole.conservation()
    assert want.shape == (len(SIZES), 3) and np.isfinite(want).all()
    parts = batch.partition(whole.nx, whole.ny, 2)
    shards = []
    for p in parts:
        with batch.Batch(whole.nx[p], whole.ny[p], whole.omega[p], whole.u_in[p], lbm.F32) as b:
            for i, d in enumerate(p):
                b.set_mask(i, masks[d])
            b.init_equilibrium(0.0, 0)
            b.step(33)
            got = b.conservation()
            np.testing.assert_array_equal(got, want[p])
            for i, d in enumerate(p):
                np.testing.assert_array_equal(b.populations(i), whole.populations(d))
            shards.append(got)
    total = batch.sharded_totals(shards[0]) + batch.sharded_totals(shards[1])
    np.testing.assert_allclose(total, want.sum(axis=0), rtol=1e-13)
    d = 5
    with lbm.Lattice(int(whole.nx[d]), int(whole.ny[d]), float(whole.omega[d]), lbm.EDGE_CHANNEL, lbm.F32) as lat:
        lat.set_inlet_velocity(float(whole.u_in[d]))
        lat.init_equilibrium(1.0, float(whole.u_in[d]), 0.0, 0.0, 0)
        lat.draw_mask(masks[d])
        lat.iterate(33)
        np.testing.assert_allclose(lat.conservation(), want[d], rtol=1e-12)
    whole.close()
