"""Checkpoint / resume: a lattice restored from a checkpoint continues bit for
bit as the saved one does, in every storage and edge mode and across the
fused representation's states (mid-run, just after an edit, with the closure
on); the file layout is the documented one; bad input is refused."""
import struct
import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [(0, 0, 3), (0, 1, 3), (1, 1, 8), (2, 1, 0), (3, 0, 0), (3, 1, 0), (0, 1, 1), (1, 0, 1)]


def make(lbm, nx, ny, edge, storage, kernel, seed=1):
    from lbm_gb300 import geometry
    mask = geometry.random_layout(nx, ny, 0.08, seed, rmin=2.0, inlet_clearance=6)
    if edge == 0:
        mask[0] = 1
        mask[-1] = 1
    lat = lbm.Lattice(nx, ny, 1.0 / 0.56, edge, storage)
    lat.set_tuning(8, kernel)
    lat.set_inlet_velocity(0.07)
    lat.init_equilibrium(1.0, 0.07, 0.0, 1e-2, seed)
    lat.draw_mask(mask)
    return lat


@pytest.mark.parametrize("storage,edge,kernel", CASES)
def test_gpu_resume_is_bitwise_identical(lbm, cuda_ok, tmp_path, storage, edge, kernel):
    nx, ny = 130, 70
    a = make(lbm, nx, ny, edge, storage, kernel)
    a.iterate(37)
    ck = a.checkpoint()
    path = tmp_path / "state.ck"
    a.save(str(path))
    assert path.read_bytes() == ck
    a.iterate(23)
    want = (a.populations(f64=storage == 3), a.field("rho"), a.field("jx"), a.get_compute_num())
    b = lbm.Lattice(nx, ny, 1.0, edge, storage)  # different omega and state: all restored
    b.set_tuning(8, kernel)
    b.load(str(path))
    assert b.get_compute_num() == 37
    b.iterate(23)
    got = (b.populations(f64=storage == 3), b.field("rho"), b.field("jx"), b.get_compute_num())
    np.testing.assert_array_equal(got[0], want[0])
    np.testing.assert_array_equal(got[1], want[1])
    np.testing.assert_array_equal(got[2], want[2])
    assert got[3] == want[3] == 60
    np.testing.assert_array_equal(b.mask(), a.mask())
    a.close()
    b.close()


def test_gpu_checkpoint_after_an_edit_and_with_the_closure(lbm, cuda_ok):
    import ctypes
    from lbm_gb300 import closure
    L = lbm.load_library()
    a = make(lbm, 96, 48, 1, lbm.F16, 8)
    a.iterate(10)
    a.draw_points([5 + 96 * 20, 1, 6 + 96 * 20, 1])  # an edit: the state is materialised
    w = closure.init_params(2)
    lbm._check(L.lbm_closure_set_weights(a.handle, w.ctypes.data_as(ctypes.c_void_p), w.size))
    lbm._check(L.lbm_closure_enable(a.handle, 0.5))
    lbm._check(L.lbm_closure_infer(a.handle))
    ck = a.checkpoint()
    a.iterate(15)
    want = a.populations()
    b = lbm.Lattice(96, 48, 1.0, 1, lbm.F16)
    b.set_tuning(8, 8)
    lbm._check(L.lbm_closure_set_weights(b.handle, w.ctypes.data_as(ctypes.c_void_p), w.size))
    b.restore(ck)
    b.iterate(15)
    np.testing.assert_array_equal(b.populations(), want)
    a.close()
    b.close()


def test_gpu_checkpoint_layout_and_refusals(lbm, cuda_ok):
    a = make(lbm, 50, 30, 1, lbm.F32, 3)
    a.iterate(5)
    ck = a.checkpoint()
    magic, version, nx, ny, edge, storage = struct.unpack_from("<8sIIIii", ck, 0)
    assert (magic, version, nx, ny, edge, storage) == (b"LBMGB3CK", 1, 50, 30, 1, 0)
    steps, = struct.unpack_from("<Q", ck, 40)
    payload, crc = struct.unpack_from("<QI", ck, 64)
    assert steps == 5 and payload == len(ck) - 96 == 50 * 30 * (1 + 17 * 4)
    assert crc == zlib.crc32(ck[96:]) & 0xFFFFFFFF
    mask = np.frombuffer(ck[96:96 + 1500], np.uint8).reshape(30, 50)
    np.testing.assert_array_equal(mask, a.mask())
    bad = bytearray(ck)
    bad[200] ^= 1
    with pytest.raises(lbm.LBMError):
        a.restore(bytes(bad))
    other = lbm.Lattice(50, 31, 1.0, 1, lbm.F32)
    with pytest.raises(lbm.LBMError):
        other.restore(ck)
    with pytest.raises(lbm.LBMError):
        lbm.Lattice(50, 30, 1.0, 1, lbm.F16).restore(ck)
    with pytest.raises(lbm.LBMError):
        a.restore(ck[:50])
    other.close()
    a.close()
