"""lbm_conservation_noalloc against lbm_conservation, through the C ABI.

lbm_conservation_noalloc serves callers that cannot allocate device memory:
it takes device pointers to moment fields the caller already owns and keeps
its scratch (per-block partial sums) in a fixed array in the library's device
image.  This file is named so that pytest collects it last; it must pass both
alone in a fresh process and after every other test.  The two sums must agree
within the tolerance of the other conservation test (rtol 1e-12, atol 1e-9):
both add the same f32 values in f64, in different orders.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-12, 1e-9


def _noalloc(lbm, torch, rho, jx, jy, solid, out):
    L = lbm.load_library()
    ny, nx = rho.shape
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.lbm_conservation_noalloc(ctypes.c_void_p(rho.data_ptr()), ctypes.c_void_p(jx.data_ptr()),
                                    ctypes.c_void_p(jy.data_ptr()),
                                    ctypes.c_void_p(solid.data_ptr()) if solid is not None else None,
                                    nx, ny, nx, ctypes.c_void_p(out.data_ptr()),
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


def test_noalloc_rejects_inputs_beyond_its_scratch(lbm, cuda_ok):
    import torch
    L = lbm.load_library()
    buf = torch.zeros(4, dtype=torch.float32, device="cuda")
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    rc = L.lbm_conservation_noalloc(p, p, p, None, 1 << 15, 1 << 14, 1 << 15, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 1
    assert b"exceed" in L.lbm_last_error()
