"""GPU: work queued on a lattice's stream before lbm_set_stream comes first.

A handle starts on its own non-blocking stream; a caller that moves it to
another stream (a torch stream, the legacy default stream) expects the steps,
re-bases and initialisations already queued to finish before the new
stream's work touches the same buffers.  lbm_set_stream makes the new stream
wait for the old one on the device.  Each case queues milliseconds of work,
switches at once, and compares with the same calls on one stream: bit for
bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NX, NY = 2048, 1024


def _layout():
    from lbm_gb300 import geometry
    return geometry.random_circles(NX, NY, 60, 4, 24, seed=3, inlet_clearance=64)


def _start(lbm, storage, mask):
    lat = lbm.Lattice(NX, NY, 1.0 / 0.56, lbm.EDGE_CHANNEL, storage)
    lat.set_inlet_velocity(0.08)
    lat.init_equilibrium(1.0, 0.08, 0.0, 1e-3, 7)
    lat.draw_mask(mask)
    return lat


@pytest.mark.parametrize("storage", [0, 1])
def test_gpu_steps_queued_before_a_stream_switch_come_first(lbm, cuda_ok, storage):
    import torch
    mask = _layout()
    ref = _start(lbm, storage, mask)
    ref.iterate(300)
    ref.iterate(7)
    want = ref.populations()
    ref.close()

    lat = _start(lbm, storage, mask)
    lat.iterate(300)  # ~10 ms queued on the handle's own stream
    s = torch.cuda.Stream()
    lat.set_stream(s.cuda_stream)
    lat.iterate(7)  # on the new stream: must follow the 300 steps
    np.testing.assert_array_equal(lat.populations(), want)
    lat.close()


@pytest.mark.parametrize("storage", [1, 2])
def test_gpu_rebase_queued_before_a_stream_switch_comes_first(lbm, cuda_ok, storage):
    """lbm_set_storage_reference re-expresses every stored word (one pass on
    the handle's stream); an initialisation queued on a new stream right
    after must not race it."""
    import torch
    mask = _layout()
    ref = lbm.Lattice(NX, NY, 1.0 / 0.56, lbm.EDGE_CHANNEL, storage)
    ref.set_storage_reference(True)
    ref.set_inlet_velocity(0.08)
    ref.init_equilibrium(1.0, 0.08, 0.0, 1e-3, 7)
    ref.draw_mask(mask)
    ref.iterate(20)
    want = ref.populations()
    ref.close()

    lat = lbm.Lattice(NX, NY, 1.0 / 0.56, lbm.EDGE_CHANNEL, storage)
    lat.iterate(100)  # keep the handle's own stream busy before the re-base
    lat.set_storage_reference(True)
    s = torch.cuda.Stream()
    lat.set_stream(s.cuda_stream)
    lat.set_inlet_velocity(0.08)
    lat.init_equilibrium(1.0, 0.08, 0.0, 1e-3, 7)
    lat.draw_mask(mask)
    lat.iterate(20)
    np.testing.assert_array_equal(lat.populations(), want)
    lat.close()


@pytest.mark.parametrize("storage,prec,sr", [(0, 0, False), (1, 1, False), (1, 1, True), (2, 2, True)])
def test_gpu_steps_in_a_callers_own_capture(lbm, cuda_ok, oracle_mod, storage, prec, sr):
    """lbm_step inside the caller's stream capture records plain launches;
    replaying the caller's graph three times advances the state by three
    times the recorded (even) steps, bit for bit with the oracle.  With
    stochastic rounding each replay reads fresh step indices from the
    device step clock, which the recorded graph advances itself."""
    import torch
    from test_gpu_parity import run_pair
    P = oracle_mod
    rng = np.random.default_rng(21)
    nx, ny = 200, 64
    mask = (rng.random((ny, nx)) < 0.08).astype(np.uint8)
    lat, o = run_pair(lbm, P, nx, ny, 1.0 / 0.6, 1, storage, prec, 2, mask, ux=0.07, noise=1e-2, seed=3,
                      sr_seed=44 if sr else None)
    s = torch.cuda.Stream()
    lat.set_stream(s.cuda_stream)
    lat.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s, capture_error_mode="thread_local"):
        lat.iterate(10)
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    o.step(30)
    pops, rho, _, _ = o.state()
    np.testing.assert_array_equal(lat.populations(), pops.astype(np.float32))
    np.testing.assert_array_equal(lat.field("rho"), rho.astype(np.float32))
    lat.close()
