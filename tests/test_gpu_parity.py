"""GPU parity: the fused sm_103a step through the C ABI against the CPU oracle
and the reference-shader fixtures.

Bar: bit-exact for f32, f64, f16 and bf16 storage (the kernel evaluates the
reference's expressions in source order with no FMA contraction, like the
oracle).  Derived fields (velocity, speed, vorticity) are compared with a
relative tolerance of 1e-6, written per test.
"""
import hashlib

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

CASES = ["cfg0_256x128_1000", "small_64x32_300", "odd_33x17_200", "tiny_8x6_50"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("rows,kernel", [(8, 0), (3, 0), (8, 1), (3, 1), (1, 1), (8, 2), (1, 2), (13, 3), (3, 4),
                                         (40, 5), (8, 6), (3, 7), (5, 8)])
def test_gpu_matches_reference_fixture(lbm, cuda_ok, name, rows, kernel):
    g = golden(name)
    nx, ny, steps = int(g["nx"]), int(g["ny"]), int(g["steps"])
    with lbm.Lattice(nx, ny, float(g["omega"]), lbm.EDGE_REF, lbm.F32) as lat:
        lat.set_tuning(rows, kernel)
        lat.init_equilibrium(1.0, float(g["ux"]), 0.0, float(g["noise"]), int(g["seed"]))
        assert sha(lat.populations()) == str(g["init_sha"])
        lat.draw_mask(g["mask"])
        lat.iterate(steps)
        lat.synchronize()
        assert lat.get_compute_num() == steps
        np.testing.assert_array_equal(lat.field("rho"), g["rho"])
        np.testing.assert_array_equal(lat.field("jx"), g["jx"])
        np.testing.assert_array_equal(lat.field("jy"), g["jy"])
        curl = lat.field("curl")
        inner = np.zeros((ny, nx), bool)
        inner[: ny - 1, 1:] = True
        np.testing.assert_array_equal(curl[inner], g["curl"][inner])
        assert sha(lat.populations()) == str(g["pops_sha"])


def test_gpu_matches_reference_edits_fixture(lbm, cuda_ok):
    g = golden("edits_48x24")
    nx, ny = int(g["nx"]), int(g["ny"])
    with lbm.Lattice(nx, ny, float(g["omega"]), lbm.EDGE_REF, lbm.F32) as lat:
        lat.init_equilibrium(1.0, 0.1, 0.0, 1e-3, 21)
        lat.draw_mask(g["mask"])
        lat.iterate(40)
        lat.draw_points(g["draw"])
        lat.iterate(25)
        lat.update_omega_buffer(float(g["omega2"]))
        lat.iterate(35)
        np.testing.assert_array_equal(lat.mask(), g["barrier_after"].astype(np.uint8))
        np.testing.assert_array_equal(lat.populations(), g["pops"])
        np.testing.assert_array_equal(lat.field("rho"), g["rho"])


def test_gpu_matches_reference_single_cell_fixture(lbm, cuda_ok):
    g = golden("single_cell_40x20")
    nx, ny = int(g["nx"]), int(g["ny"])
    for d in range(9):
        with lbm.Lattice(nx, ny, float(g["omega"]), lbm.EDGE_REF, lbm.F32) as lat:
            lat.single_cell(d)
            lat.iterate(int(g["steps"]))
            np.testing.assert_array_equal(lat.populations(), g["pops_%d" % d])


def run_pair(lbm, P, nx, ny, omega, edge, storage, prec, steps, mask, ux=0.1, noise=1e-3, seed=0, rows=8,
             chunks=None, edits=None, kernel=1, store_inlet=None, sr_seed=None):
    lat = lbm.Lattice(nx, ny, omega, edge, storage)
    lat.set_tuning(rows, kernel)
    o = P.Oracle(nx, ny, float(np.float32(omega)), edge, prec)
    if store_inlet is not None:  # else both keep their default (16-bit words relative to the rest weights)
        lat.set_storage_reference(store_inlet)
        o.set_storage_reference(store_inlet)
    lat.set_inlet_velocity(ux)  # channel inlet speed (no field reset)
    o.set_inlet(float(np.float32(ux)), apply=False)
    lat.init_equilibrium(1.0, ux, 0.0, noise, seed)
    o.init_equilibrium(1.0, float(np.float32(ux)), 0.0, float(np.float32(noise)), seed)
    if mask is not None:
        lat.draw_mask(mask)
        o.set_mask(mask)
    if sr_seed is not None:  # stochastic rounding of the stored 16-bit words
        lat.set_rounding(lbm.ROUND_STOCHASTIC, sr_seed)
        o.set_rounding(1, sr_seed)
    for k, c in enumerate(chunks or [steps]):
        lat.iterate(c)
        o.step(c)
        if edits and k < len(edits):
            edits[k](lat, o)
    return lat, o


def assert_same_state(lat, o, f64=False):
    pops, rho, jx, jy = o.state()
    t = np.float64 if f64 else np.float32
    np.testing.assert_array_equal(lat.populations(f64=f64), pops.astype(t))
    np.testing.assert_array_equal(lat.field("rho"), rho.astype(np.float32))
    np.testing.assert_array_equal(lat.field("jx"), jx.astype(np.float32))
    np.testing.assert_array_equal(lat.field("jy"), jy.astype(np.float32))


@pytest.mark.parametrize("storage,prec,f64", [(0, 0, False), (1, 1, False), (3, 3, True)])
@pytest.mark.parametrize("pinned", [False, True])
def test_gpu_caller_noise_initialisation(lbm, cuda_ok, oracle_mod, storage, prec, f64, pinned):
    """lbm_init_equilibrium_noise (set_equil with a caller noise
    array) from pageable and from page-locked host memory: the same state as
    the oracle's, and the same 30 steps after it."""
    import torch
    P = oracle_mod
    nx, ny = 150, 70
    rng = np.random.default_rng(11 + storage)
    noise = (rng.uniform(-1e-2, 1e-2, (2, ny, nx))).astype(np.float32)
    if pinned:
        buf = torch.from_numpy(noise).pin_memory()
        noise_in = buf.numpy()
    else:
        noise_in = noise
    mask = (rng.random((ny, nx)) < 0.08).astype(np.uint8)
    lat = lbm.Lattice(nx, ny, float(np.float32(1 / 0.6)), 1, storage)
    o = P.Oracle(nx, ny, float(np.float32(1 / 0.6)), 1, prec)
    lat.set_inlet_velocity(0.06)
    o.set_inlet(float(np.float32(0.06)), apply=False)
    lat.init_equilibrium_noise(1.0, 0.06, 0.0, noise_in)
    o.init_equilibrium_noise(1.0, float(np.float32(0.06)), 0.0, noise)
    t = np.float64 if f64 else np.float32
    np.testing.assert_array_equal(lat.populations(f64=f64), o.state()[0].astype(t))
    lat.draw_mask(mask)
    o.set_mask(mask)
    lat.iterate(30)
    o.step(30)
    assert_same_state(lat, o, f64=f64)
    lat.init_equilibrium_noise(1.0, 0.06, 0.0, None)
    o.init_equilibrium(1.0, float(np.float32(0.06)), 0.0, 0.0, 0)
    np.testing.assert_array_equal(lat.populations(f64=f64), o.state()[0].astype(t))
    lat.close()


@pytest.mark.parametrize("edge", [0, 1])
@pytest.mark.parametrize("kernel", [0, 1, 3, 6])
def test_gpu_config0_both_edge_modes(lbm, cuda_ok, oracle_mod, edge, kernel):
    """256 x 128, tau 0.6, ux 0.1 +- 1e-4 noise, r=12 circle at (64,64), 1000 steps."""
    from lbm_gb300 import geometry
    P = oracle_mod
    mask = geometry.single_circle(256, 128, 64, 64, 12)
    if edge == 0:
        mask[0] = 1
        mask[-1] = 1
    lat, o = run_pair(lbm, P, 256, 128, 1.0 / 0.6, edge, lbm.F32, P.P_F32, 1000, mask, ux=0.1, noise=1e-4, seed=0,
                      kernel=kernel)
    assert_same_state(lat, o)
    lat.close()


STORAGES = [(0, 0, False), (3, 3, True), (1, 1, False), (2, 2, False)]  # (lbm storage, oracle prec, f64 read)


@pytest.mark.parametrize("storage,prec,f64", STORAGES)
@pytest.mark.parametrize("edge", [0, 1])
@pytest.mark.parametrize("nx,ny,rows", [(8, 6, 1), (33, 17, 4), (70, 41, 8), (129, 64, 5), (131, 20, 3),
                                        (600, 37, 7), (1100, 700, 9)])
@pytest.mark.parametrize("kernel", [0, 1, 2, 3, 5, 6, 8, 9, 10, 11, 12])
def test_gpu_random_small_grids(lbm, cuda_ok, oracle_mod, storage, prec, f64, edge, nx, ny, rows, kernel):
    P = oracle_mod
    rng = np.random.default_rng(nx * 1000 + ny + 7 * storage + edge)
    omega = float(np.float32(rng.uniform(0.7, 1.9)))
    mask = (rng.random((ny, nx)) < 0.15).astype(np.uint8)
    lat, o = run_pair(lbm, P, nx, ny, omega, edge, storage, prec, 60, mask, ux=0.07, noise=1e-2,
                      seed=int(rng.integers(1 << 30)), rows=rows, kernel=kernel)
    assert_same_state(lat, o, f64=f64)
    lat.close()


@pytest.mark.parametrize("edge", [0, 1])
@pytest.mark.parametrize("storage,store_inlet,sr", [(0, True, False), (1, True, False), (2, True, False),
                                                    (1, False, False), (2, False, False), (1, True, True),
                                                    (2, False, True)])
def test_gpu_state_edits_between_steps(lbm, cuda_ok, oracle_mod, edge, storage, store_inlet, sr):
    """Barrier edits, omega and inlet changes between iterate calls keep the
    reference's step semantics (the fused state is materialised first).  In
    16-bit storage the inlet change re-expresses the stored words against the
    new inlet equilibrium (or, with the rest-weight reference, leaves them),
    and the last edit switches the storage reference; every step of it
    matches the oracle bit for bit, with stochastic rounding too (the edits
    and re-expressions round to nearest, the steps stochastically)."""
    P = oracle_mod
    nx, ny = 64, 40
    rng = np.random.default_rng(5 + edge)
    mask = (rng.random((ny, nx)) < 0.08).astype(np.uint8)

    def draw(lat, o):
        pairs = np.stack([rng.integers(0, nx * ny + 10, 40), rng.integers(0, 2, 40)], 1).astype(np.uint32)
        lat.draw_points(pairs)
        o.barrier_pairs(pairs)

    def omega(lat, o):
        w = float(np.float32(1.0 / (3.0 * 0.03 + 0.5)))
        lat.update_omega_buffer(w)
        o.set_omega(w)

    def inlet(lat, o):
        lat.set_inlet_velocity(0.05)
        o.set_inlet(float(np.float32(0.05)))

    def reset_barrier(lat, o):
        lat.reset_barrier()
        o.reset_barrier()

    def switch_reference(lat, o):
        lat.set_storage_reference(not store_inlet)
        o.set_storage_reference(not store_inlet)
        assert lat.storage_reference == (not store_inlet)

    lat, o = run_pair(lbm, P, nx, ny, 1.0 / 0.7, edge, storage, storage, 0, mask, chunks=[7, 5, 1, 9, 4, 6, 5],
                      edits=[draw, omega, inlet, draw, reset_barrier, switch_reference], store_inlet=store_inlet,
                      sr_seed=77 if sr else None)
    assert_same_state(lat, o)
    assert lat.get_compute_num() == o.step_count
    lat.close()


@pytest.mark.parametrize("storage", [1, 2])
@pytest.mark.parametrize("edge", [0, 1])
@pytest.mark.parametrize("nx,ny,rows", [(33, 17, 4), (129, 64, 5), (1100, 700, 9), (2048, 96, 2)])
@pytest.mark.parametrize("kernel", [1, 3, 7, 9, 11, 12, 13])
def test_gpu_inlet_reference_16bit(lbm, cuda_ok, oracle_mod, storage, edge, nx, ny, rows, kernel):
    """16-bit words relative to the inlet equilibrium (lbm_set_storage_reference
    1): the shifted form of the collision, with bounced words re-expressed,
    matches the oracle bit for bit in every kernel variant, f16 and bf16."""
    P = oracle_mod
    rng = np.random.default_rng(nx * 31 + ny + 5 * storage + edge)
    omega = float(np.float32(rng.uniform(0.7, 1.9)))
    mask = (rng.random((ny, nx)) < 0.1).astype(np.uint8)
    lat, o = run_pair(lbm, P, nx, ny, omega, edge, storage, storage, 50, mask, ux=0.08, noise=1e-2,
                      seed=int(rng.integers(1 << 30)), rows=rows, kernel=kernel, store_inlet=True)
    assert lat.storage_reference
    assert_same_state(lat, o)
    lat.close()


def test_gpu_read_between_steps_does_not_perturb(lbm, cuda_ok, oracle_mod):
    P = oracle_mod
    nx, ny = 50, 30
    lat, o = run_pair(lbm, P, nx, ny, 1.0 / 0.55, 1, lbm.F32, P.P_F32, 0, None, chunks=[3])
    for _ in range(4):
        lat.populations()
        lat.field("curl")
        lat.iterate(5)
        o.step(5)
    assert_same_state(lat, o)
    lat.close()


def test_gpu_derived_fields(lbm, cuda_ok, oracle_mod):
    """ux = jx/rho, uy, speed and vorticity from the moments (rel tol 1e-6)."""
    from lbm_gb300 import geometry
    P = oracle_mod
    nx, ny = 96, 48
    mask = geometry.single_circle(nx, ny, 30, 24, 6)
    lat, o = run_pair(lbm, P, nx, ny, 1.0 / 0.6, 1, lbm.F32, P.P_F32, 200, mask)
    _, rho, jx, jy = o.state()
    ux, uy = jx / rho, jy / rho
    np.testing.assert_allclose(lat.field("ux"), ux, rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(lat.field("uy"), uy, rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(lat.field("speed"), np.hypot(ux, uy), rtol=1e-6, atol=1e-9)
    yu = np.roll(np.arange(ny), 1)
    yd = np.roll(np.arange(ny), -1)
    xl = np.clip(np.arange(nx) - 1, 0, nx - 1)
    xr = np.clip(np.arange(nx) + 1, 0, nx - 1)
    dx = (uy[:, xr] - uy[:, xl]) / np.maximum(xr - xl, 1)[None, :]
    dy = (ux[yd, :] - ux[yu, :]) / 2.0
    np.testing.assert_allclose(lat.field("vorticity"), dx + dy, rtol=1e-5, atol=1e-7)
    lat.close()


def test_gpu_conservation_sums(lbm, cuda_ok, oracle_mod):
    P = oracle_mod
    nx, ny = 200, 100
    rng = np.random.default_rng(3)
    mask = (rng.random((ny, nx)) < 0.1).astype(np.uint8)
    for storage, prec in ((lbm.F32, P.P_F32), (lbm.F64, P.P_F64)):
        lat, o = run_pair(lbm, P, nx, ny, 1.0 / 0.6, 1, storage, prec, 30, mask)
        _, rho, jx, jy = o.state()
        fluid = mask == 0
        got = lat.conservation()
        want = np.array([rho[fluid].sum(), jx[fluid].sum(), jy[fluid].sum()])
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-9)
        lat.close()


def test_gpu_nonfinite_upload_is_reported(lbm, cuda_ok):
    """A NaN injected into an upload surfaces as LBM_ERR_STATE at synchronize."""
    with lbm.Lattice(40, 20, 1.0, lbm.EDGE_CHANNEL, lbm.F32) as lat:
        pops = lat.populations()
        pops[4, 10, 20] = np.nan
        lat.write_populations(pops)
        lat.iterate(2)
        with pytest.raises(lbm.LBMError) as e:
            lat.synchronize()
        assert e.value.code == 4


def test_gpu_full_size_channel_matches_oracle(lbm, cuda_ok, oracle_mod):
    """4096 x 2048 with 200 seeded circles (the large single-grid workload),
    f32, 12 steps: bit-exact against the oracle on the full grid."""
    from lbm_gb300 import geometry
    P = oracle_mod
    nx, ny = 4096, 2048
    mask = geometry.random_circles(nx, ny, 200, 4, 32, seed=1)
    lat, o = run_pair(lbm, P, nx, ny, 1.0 / 0.55, 1, lbm.F32, P.P_F32, 12, mask, ux=0.08, noise=0.0)
    _, rho, jx, jy = o.state()
    np.testing.assert_array_equal(lat.field("rho"), rho.astype(np.float32))
    np.testing.assert_array_equal(lat.field("jx"), jx.astype(np.float32))
    lat.close()


@pytest.mark.parametrize("kernel", [0, 1, 3, 8, 9])
def test_gpu_graph_replay_is_transparent(lbm, cuda_ok, oracle_mod, kernel):
    """Runs of steps replayed from captured graphs (the default) give the same
    state as plain launches, across an omega change between calls (which must
    recapture) and against the oracle."""
    P = oracle_mod
    nx, ny = 130, 70
    rng = np.random.default_rng(11)
    mask = (rng.random((ny, nx)) < 0.06).astype(np.uint8)
    L = lbm.load_library()
    states = []
    for graphs in (1, 0):
        lat, o = run_pair(lbm, P, nx, ny, 1.0 / 0.6, 1, lbm.F32 if kernel < 8 else lbm.F16,
                          P.P_F32 if kernel < 8 else P.P_F16, 0, mask, kernel=kernel)
        lbm._check(L.lbm_set_graphs(lat.handle, graphs))
        lat.iterate(53)
        o.step(53)
        w = float(np.float32(1.0 / 0.7))
        lat.update_omega_buffer(w)
        o.set_omega(w)
        lat.iterate(41)
        o.step(41)
        assert_same_state(lat, o)
        states.append(lat.populations())
        lat.close()
    np.testing.assert_array_equal(states[0], states[1])


@pytest.mark.parametrize("storage,prec,kernel", [(0, 0, 3), (1, 1, 11), (0, 0, 0)])
def test_gpu_repeated_short_calls_replay_whole_call_graphs(lbm, cuda_ok, oracle_mod, storage, prec, kernel):
    """Short lbm_step calls repeated with the same length replay one captured
    graph per starting buffer parity (odd lengths alternate the two); a new
    length, an omega change and a state edit recapture or fall back to plain
    launches.  The state must match the oracle and a run without graphs."""
    P = oracle_mod
    nx, ny = 300, 70
    rng = np.random.default_rng(5)
    mask = (rng.random((ny, nx)) < 0.05).astype(np.uint8)
    L = lbm.load_library()
    plan = [7, 7, 7, 7, 2, 2, 64, 65, 7, 7]
    states = []
    for graphs in (1, 0):
        lat, o = run_pair(lbm, P, nx, ny, 1.0 / 0.6, 1, storage, prec, 0, mask, kernel=kernel)
        lbm._check(L.lbm_set_graphs(lat.handle, graphs))
        for i, n in enumerate(plan):
            if i == 8:
                w = float(np.float32(1.0 / 0.7))
                lat.update_omega_buffer(w)
                o.set_omega(w)
            lat.iterate(n)
            o.step(n)
        assert_same_state(lat, o)
        assert lat.get_compute_num() == sum(plan)
        states.append(lat.populations())
        lat.close()
    np.testing.assert_array_equal(states[0], states[1])
