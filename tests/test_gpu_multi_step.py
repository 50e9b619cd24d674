"""GPU: small lattices take a whole lbm_step call in one cooperative launch
(k_step_ws_multi: the staged step's grid, steps separated by a grid-wide
barrier, each CTA's bulk-copy ring running through all steps).  The state
after it is the oracle's bit for bit, in both edge modes and every storage
the path serves, and equals the state that one launch per step gives (graphs
and launch fusion off), with the learned closure on as well."""
import numpy as np
import pytest

from test_gpu_parity import assert_same_state, run_pair

pytestmark = pytest.mark.gpu

CASES = [(0, 0, 1, 3), (0, 0, 0, 3), (1, 1, 1, 7), (2, 2, 1, 7), (1, 1, 0, 7), (1, 1, 1, 7, True)]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("nx,ny,rows", [(33, 17, 2), (130, 70, 3), (513, 200, 8), (1000, 300, 2)])
def test_gpu_multi_step_matches_oracle(lbm, cuda_ok, oracle_mod, case, nx, ny, rows):
    storage, prec, edge, kernel = case[:4]
    store_inlet = case[4] if len(case) > 4 else None
    P = oracle_mod
    rng = np.random.default_rng(nx + 3 * ny + storage)
    mask = (rng.random((ny, nx)) < 0.1).astype(np.uint8)
    # the first call steps the materialised state (one launch); the calls after it are fused
    lat, o = run_pair(lbm, P, nx, ny, float(np.float32(rng.uniform(0.8, 1.9))), edge, storage, prec, 0, mask,
                      ux=0.07, noise=1e-2, seed=5, rows=rows, chunks=[1, 37, 2, 3, 20], kernel=kernel,
                      store_inlet=store_inlet)
    assert lat.get_compute_num() == 63
    assert_same_state(lat, o)
    lat.synchronize()
    lat.close()


@pytest.mark.parametrize("storage,kernel", [(0, 3), (1, 7)])
def test_gpu_multi_step_equals_one_launch_per_step_with_the_closure(lbm, cuda_ok, storage, kernel):
    import ctypes
    from lbm_gb300 import closure, geometry
    L = lbm.load_library()
    w = closure.init_params(5)
    nx, ny = 256, 128
    mask = geometry.random_circles(nx, ny, 40, 3, 8, seed=2, inlet_clearance=8)
    out = []
    for fused in (True, False):
        with lbm.Lattice(nx, ny, 1 / 0.53, lbm.EDGE_CHANNEL, storage) as lat:
            lat.set_tuning(2, kernel)
            lat.set_graphs(fused)
            lat.set_inlet_velocity(0.05)
            lat.init_equilibrium(1.0, 0.05, 0.0, 1e-3, 3)
            lat.draw_mask(mask)
            lat.iterate(3)
            lbm._check(L.lbm_closure_set_weights(lat.handle, w.ctypes.data_as(ctypes.c_void_p), w.size))
            lbm._check(L.lbm_closure_enable(lat.handle, 1.0))
            for _ in range(3):
                lbm._check(L.lbm_closure_infer(lat.handle))
                lat.iterate(20)
            lat.synchronize()
            out.append((lat.populations(), lat.field("rho"), lat.field("jx")))
    for a, b in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, b)
