"""lbm_conservation_noalloc against lbm_conservation, through the C ABI.

lbm_conservation_noalloc serves callers that cannot allocate device memory:
it takes device pointers to moment fields the caller already owns and keeps
its scratch (per-block partial sums) in a fixed array in the library's device
image.  This file is named so that pytest collects it last; it must pass both
alone in a fresh process and after every other test.  The two sums must agree
within the tolerance of the other conservation test (rtol 1e-12, atol 1e-9):
both add the same f32 values in f64, in different orders.  Against float64
numpy sums the bound also allows 1e-14 of the summed magnitudes, for the
large grids.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-12, 1e-9


def _noalloc(lbm, torch, rho, jx, jy, solid, out, nx=None):
    """Calls the entry point on (ny, pitch) device arrays; `nx` <= pitch
    columns of each row are cells (all of them by default)."""
    L = lbm.load_library()
    ny, pitch = rho.shape
    nx = pitch if nx is None else nx
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.lbm_conservation_noalloc(ctypes.c_void_p(rho.data_ptr()), ctypes.c_void_p(jx.data_ptr()),
                                    ctypes.c_void_p(jy.data_ptr()),
                                    ctypes.c_void_p(solid.data_ptr()) if solid is not None else None,
                                    nx, ny, pitch, ctypes.c_void_p(out.data_ptr()),
                                    ctypes.c_void_p(stream) if stream else None)
    assert rc == 0, L.lbm_last_error().decode()
    torch.cuda.synchronize()
    return out.cpu().numpy().copy()


def test_noalloc_matches_handle_reduction_on_two_calls(lbm, cuda_ok):
    import torch
    nx, ny = 300, 200
    rng = np.random.default_rng(11)
    mask = (rng.random((ny, nx)) < 0.1).astype(np.uint8)
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    with lbm.Lattice(nx, ny, 1.0 / 0.6, lbm.EDGE_CHANNEL, lbm.F32) as lat:
        lat.set_inlet_velocity(0.08)
        lat.init_equilibrium(1.0, 0.08, 0.0, 1e-3, 5)
        lat.draw_mask(mask)
        for steps in (20, 35):  # two calls in a row, on two different states
            lat.iterate(steps)
            want = lat.conservation()
            dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
            got = _noalloc(lbm, torch, dev(lat.field("rho")), dev(lat.field("jx")), dev(lat.field("jy")),
                           dev(lat.mask()), out)
            np.testing.assert_allclose(got, want, rtol=RTOL, atol=ATOL)


@pytest.mark.parametrize("nx,pitch,ny,with_solid", [(300, 320, 200, True), (300, 320, 200, False),
                                                   (1000, 1000, 700, False), (37, 64, 5, True),
                                                   (4096, 4224, 2048, True)])
def test_noalloc_matches_float64_sums_with_pitch_and_without_mask(lbm, cuda_ok, nx, pitch, ny, with_solid):
    """Against float64 numpy sums of the same f32 values: row pitch wider than
    the grid (the padding columns hold large values and solid flags that must
    be ignored), and solid = NULL (every cell counts).  Two calls in a row on
    different fields, the second after the scratch holds the first's sums."""
    import torch
    rng = np.random.default_rng(nx + ny)
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    for call in range(2):
        f = [rng.uniform(0.5, 1.5, (ny, pitch)).astype(np.float32),
             rng.normal(0.0, 0.1, (ny, pitch)).astype(np.float32),
             rng.normal(0.0, 0.1, (ny, pitch)).astype(np.float32)]
        for a in f:
            a[:, nx:] = 1e6 * (call + 1)  # padding: never summed
        solid = (rng.random((ny, pitch)) < 0.1).astype(np.uint8)
        solid[:, nx:] = rng.integers(0, 2, (ny, pitch - nx))
        keep = np.zeros((ny, pitch), bool)
        keep[:, :nx] = True
        if with_solid:
            keep &= solid == 0
        want = np.array([a.astype(np.float64)[keep].sum() for a in f])
        # float64 sums of the same values in two orders differ by rounding
        # only: bounded by 1e-14 of the sum of magnitudes at these sizes
        scale = np.array([np.abs(a.astype(np.float64)[keep]).sum() for a in f])
        dev = [torch.from_numpy(a).cuda() for a in f]
        got = _noalloc(lbm, torch, *dev, torch.from_numpy(solid).cuda() if with_solid else None, out, nx=nx)
        assert np.all(np.abs(got - want) <= np.maximum(ATOL, 1e-14 * scale) + RTOL * np.abs(want)), (got, want)


def test_noalloc_rejects_inputs_beyond_its_scratch(lbm, cuda_ok):
    import torch
    L = lbm.load_library()
    buf = torch.zeros(4, dtype=torch.float32, device="cuda")
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    rc = L.lbm_conservation_noalloc(p, p, p, None, 1 << 15, 1 << 14, 1 << 15, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 1
    assert b"exceed" in L.lbm_last_error()
