"""y-slab decomposition on one GPU: slabs stepped one after another in one
process (no kernel waits on another) with host-staged halo rows reproduce the
undivided lattice bit for bit, in f32 and 16-bit storage, through every step
kernel."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage,kernel,slabs", [(0, 3, 2), (0, 0, 3), (1, 8, 2), (2, 1, 4), (1, 11, 2), (2, 9, 3)])
def test_gpu_slabs_match_one_lattice(lbm, cuda_ok, storage, kernel, slabs):
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
    ss = [SlabLattice(nx, ny, 1.0 / 0.56, r, slabs, storage=storage, u_in=0.07) for r in range(slabs)]
    ex = LocalExchanger(ss)
    for s in ss:
        s.lat.set_tuning(8, kernel)
        s.set_mask(mask)
        s.write_populations(start)
        s.attach(ex)
    # the same start: the undivided lattice from the uploaded state too
    ref.write_populations(start)
    ref.iterate(steps)
    run_local(ss, steps)
    got = np.concatenate([s.populations() for s in ss], axis=1)
    np.testing.assert_array_equal(got, ref.populations())
    np.testing.assert_array_equal(np.concatenate([s.field("rho") for s in ss]), ref.field("rho"))
    for s in ss:
        s.lat.close()
    ref.close()


@pytest.mark.parametrize("storage,kernel,slabs", [(0, 3, 2), (0, 0, 3), (1, 11, 2), (1, 13, 4), (2, 7, 3),
                                                  (0, 3, 48), (3, 0, 2)])
def test_gpu_overlapped_slabs_match_one_lattice(lbm, cuda_ok, storage, kernel, slabs):
    """The overlapped schedule: each slab steps its edge rows (lbm_step_rows),
    copies their crossing populations to device buffers, steps its interior
    rows, then takes its ghost rows from the neighbours' buffers.  Bit-exact
    against the undivided lattice, populations and the last step's moments,
    down to slabs of two rows (no interior) and with f64 storage."""
    import torch
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
    stream = torch.cuda.Stream()
    ss = [SlabLattice(nx, ny, 1.0 / 0.56, r, slabs, storage=storage, u_in=0.07) for r in range(slabs)]
    for s in ss:
        s.lat.set_stream(stream.cuda_stream)
        s.lat.set_tuning(8, kernel)
        s.set_mask(mask)
        s.write_populations(start)
    ex = LocalExchanger(ss, device=True)
    for s in ss:
        s.attach(ex)
    ref.write_populations(start)
    ref.iterate(steps)
    run_local(ss, steps)
    f64 = storage == 3
    got = np.concatenate([s.populations(f64=f64) for s in ss], axis=1)
    np.testing.assert_array_equal(got, ref.populations(f64=f64))
    for name in ("rho", "jx", "jy"):
        np.testing.assert_array_equal(np.concatenate([s.field(name) for s in ss]), ref.field(name))
    assert all(s.lat.get_compute_num() == steps for s in ss)
    for s in ss:
        s.lat.close()
    ref.close()


def test_gpu_step_rows_matches_lbm_step_and_guards_the_state(lbm, cuda_ok, oracle_mod):
    """lbm_step_rows in any split of the rows gives lbm_step's result; while a
    step is incomplete, state-changing calls are refused with LBM_ERR_STATE
    and row-range arguments are checked."""
    from lbm_gb300 import geometry
    nx, ny = 130, 41
    mask = geometry.random_layout(nx, ny, 0.08, 2, rmin=2.0, inlet_clearance=6)
    a = lbm.Lattice(nx, ny, 1.0 / 0.6, lbm.EDGE_CHANNEL, lbm.F32)
    b = lbm.Lattice(nx, ny, 1.0 / 0.6, lbm.EDGE_CHANNEL, lbm.F32)
    for lat in (a, b):
        lat.set_inlet_velocity(0.06)
        lat.init_equilibrium(1.0, 0.06, 0.0, 1e-3, 8)
        lat.draw_mask(mask)
    a.iterate(9)
    splits = [[(0, ny)], [(20, 41), (0, 20)], [(0, 1), (1, 2), (2, 40), (40, 41)], [(5, 30), (0, 5), (30, 41)]]
    for k in range(9):
        sp = splits[k % len(splits)]
        for i, (y0, y1) in enumerate(sp):
            b.step_rows(y0, y1, complete=i == len(sp) - 1, moments=k == 8)
    np.testing.assert_array_equal(b.populations(), a.populations())
    np.testing.assert_array_equal(b.field("rho"), a.field("rho"))
    assert b.get_compute_num() == 9
    b.step_rows(0, 10)
    for call in (lambda: b.iterate(1), lambda: b.populations(), lambda: b.draw_mask(mask),
                 lambda: b.field("rho")):
        with pytest.raises(lbm.LBMError) as e:
            call()
        assert e.value.code == 4
    for y0, y1 in ((10, 10), (5, 42), (30, 20)):
        with pytest.raises(lbm.LBMError):
            b.step_rows(y0, y1)
    b.step_rows(10, ny, complete=True)
    a.iterate(1)
    np.testing.assert_array_equal(b.populations(), a.populations())
    a.close()
    b.close()


@pytest.mark.parametrize("storage,kernel,slabs", [(0, 3, 2), (1, 11, 3), (2, 7, 2)])
def test_gpu_overlapped_slabs_follow_inlet_changes(lbm, cuda_ok, storage, kernel, slabs):
    """An inlet ramp between steps (lbm_set_inlet_velocity on every slab,
    which materialises the state and, in 16-bit storage, re-expresses the
    words against the new inlet equilibrium, ghost rows included): the slabs
    still match the undivided lattice bit for bit."""
    import torch
    from lbm_gb300 import geometry
    from lbm_gb300.slab import LocalExchanger, SlabLattice, run_local
    nx, ny = 300, 96
    mask = geometry.random_layout(nx, ny, 0.1, 5, rmin=3.0, inlet_clearance=10)
    ref = lbm.Lattice(nx, ny, 1.0 / 0.56, lbm.EDGE_CHANNEL, storage)
    ref.set_tuning(8, kernel)
    ref.set_inlet_velocity(0.0)
    ref.init_equilibrium(1.0, 0.0, 0.0, 1e-3, 9)
    ref.draw_mask(mask)
    start = ref.populations(f64=True)
    stream = torch.cuda.Stream()
    ss = [SlabLattice(nx, ny, 1.0 / 0.56, r, slabs, storage=storage, u_in=0.0) for r in range(slabs)]
    for s in ss:
        s.lat.set_stream(stream.cuda_stream)
        s.lat.set_tuning(8, kernel)
        s.set_mask(mask)
        s.write_populations(start)
    ex = LocalExchanger(ss, device=True)
    for s in ss:
        s.attach(ex)
    ref.write_populations(start)
    for i in range(1, 5):
        ref.iterate(7)
        run_local(ss, 7)
        u = 0.02 * i
        ref.set_inlet_velocity(u)
        for s in ss:
            s.lat.set_inlet_velocity(u)
    ref.iterate(5)
    run_local(ss, 5)
    got = np.concatenate([s.populations() for s in ss], axis=1)
    np.testing.assert_array_equal(got, ref.populations())
    for name in ("rho", "jx", "jy"):
        np.testing.assert_array_equal(np.concatenate([s.field(name) for s in ss]), ref.field(name))
    for s in ss:
        s.lat.close()
    ref.close()
