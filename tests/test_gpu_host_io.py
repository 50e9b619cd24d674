"""Host transfers through the C ABI with page-locked buffers.

A page-locked host buffer (torch's pinned memory here) is read or written by
the library's kernels directly over the host link, with no staging copy; other
host memory goes through a device staging buffer.  Both routes must move the
same bits: populations written either way step to the same state, and fields,
populations and masks read either way are identical.  The mask is bit-packed
on the device; reading it back (which rebuilds the host copy from the device
words) must return what was written.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage", [0, 1, 3])
@pytest.mark.parametrize("nx", [203, 204])  # 204: rows of whole 16-byte words, read and written four cells at a time
def test_gpu_pinned_and_pageable_transfers_agree(lbm, cuda_ok, storage, nx):
    import torch
    L = lbm.load_library()
    from lbm_gb300 import geometry
    ny = 77
    mask = geometry.random_layout(nx, ny, 0.08, 3, rmin=2.0, inlet_clearance=6)
    src = lbm.Lattice(nx, ny, 1.0 / 0.6, lbm.EDGE_CHANNEL, storage)
    src.set_inlet_velocity(0.06)
    src.init_equilibrium(1.0, 0.06, 0.0, 1e-3, 9)
    src.draw_mask(mask)
    src.iterate(17)
    pops = src.populations()
    src.close()
    out = {}
    for route in ("pageable", "pinned"):
        lat = lbm.Lattice(nx, ny, 1.0 / 0.6, lbm.EDGE_CHANNEL, storage)
        lat.set_inlet_velocity(0.06)
        if route == "pinned":
            p = torch.from_numpy(pops.reshape(-1).copy()).pin_memory()
            m = torch.from_numpy(mask.reshape(-1).astype(np.uint8)).pin_memory()
            lbm._check(L.lbm_write_populations(lat.handle, ctypes.c_void_p(p.data_ptr())))
            lbm._check(L.lbm_set_mask(lat.handle, ctypes.c_void_p(m.data_ptr())))
            p.zero_()  # the caller's buffers are free once the calls return
            m.zero_()
        else:
            lat.write_populations(pops)
            lat.draw_mask(mask)
        lat.iterate(11)
        fields = {}
        for name, code in (("rho", 0), ("ux", 3), ("curl", 5)):
            if route == "pinned":
                o = torch.full((ny * nx,), float("nan"), dtype=torch.float32).pin_memory()
                lbm._check(L.lbm_read_field(lat.handle, code, ctypes.c_void_p(o.data_ptr())))
                fields[name] = o.numpy().reshape(ny, nx).copy()
            else:
                fields[name] = lat.field(name)
        if route == "pinned":
            o = torch.empty(9 * nx * ny, dtype=torch.float32).pin_memory()
            lbm._check(L.lbm_read_populations(lat.handle, ctypes.c_void_p(o.data_ptr())))
            fields["pops"] = o.numpy().reshape(9, ny, nx).copy()
        else:
            fields["pops"] = lat.populations().reshape(9, ny, nx)
        fields["mask"] = lat.mask()
        lat.synchronize()
        lat.close()
        out[route] = fields
    for k in out["pageable"]:
        np.testing.assert_array_equal(out["pinned"][k], out["pageable"][k], err_msg=k)
    np.testing.assert_array_equal(out["pinned"]["mask"], (mask != 0).astype(np.uint8))


def test_gpu_mask_packed_on_device_then_edited(lbm, cuda_ok, oracle_mod):
    """A whole mask packed on the device, then single-cell barrier edits (which
    rebuild the host copy first): the state matches the oracle bit for bit."""
    nx, ny = 97, 45
    rng = np.random.default_rng(4)
    mask = (rng.random((ny, nx)) < 0.07).astype(np.uint8) * rng.integers(1, 255, (ny, nx)).astype(np.uint8)
    mask[:, 0] = 0
    lat = lbm.Lattice(nx, ny, 1.0 / 0.58, lbm.EDGE_CHANNEL, lbm.F32)
    o = oracle_mod.Oracle(nx, ny, float(np.float32(1.0 / 0.58)), oracle_mod.EDGE_CHANNEL, oracle_mod.P_F32)
    lat.set_inlet_velocity(0.05)
    o.set_inlet(float(np.float32(0.05)), apply=False)
    lat.init_equilibrium(1.0, 0.05, 0.0, 1e-3, 2)
    o.init_equilibrium(1.0, float(np.float32(0.05)), 0.0, float(np.float32(1e-3)), 2)
    lat.draw_mask(mask)
    o.set_mask((mask != 0).astype(np.uint8))
    lat.iterate(9)
    o.step(9)
    pairs = [3 + 20 * nx, 1, 40 + 30 * nx, 1, 50 + 10 * nx, 0]
    lat.draw_points(pairs)
    m2 = (mask != 0).astype(np.uint8)
    for i in range(0, len(pairs), 2):
        m2.reshape(-1)[pairs[i]] = pairs[i + 1]
    o.barrier_pairs(np.array(pairs, np.uint32))
    np.testing.assert_array_equal(lat.mask(), m2)
    lat.iterate(13)
    o.step(13)
    np.testing.assert_array_equal(lat.populations(), o.state()[0].astype(np.float32))
    lat.close()
