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
