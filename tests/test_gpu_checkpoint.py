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


@pytest.mark.parametrize("storage", [1, 2])
def test_gpu_checkpoint_keeps_the_storage_reference(lbm, cuda_ok, storage):
    """16-bit words saved relative to the inlet equilibrium load into a
    lattice created with the default rest-weight reference: the setting is
    restored with the words, the run continues bit for bit, and the host-side
    inspection reports it."""
    a = make(lbm, 120, 64, 1, storage, 11)
    a.set_storage_reference(True)
    a.iterate(19)
    ck = a.checkpoint()
    info = lbm.checkpoint_info(ck)
    assert info["store_inlet"] == 1 and info["storage"] == storage and info["steps"] == 19
    a.iterate(11)
    want = a.populations()
    b = lbm.Lattice(120, 64, 1.0, 1, storage)
    assert not b.storage_reference
    b.set_tuning(8, 11)
    b.restore(ck)
    assert b.storage_reference
    b.iterate(11)
    np.testing.assert_array_equal(b.populations(), want)
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
    assert (magic, version, nx, ny, edge, storage) == (b"LBMGB3CK", 2, 50, 30, 1, 0)
    steps, = struct.unpack_from("<Q", ck, 40)
    payload, crc = struct.unpack_from("<QI", ck, 64)
    assert steps == 5 and payload == len(ck) - 96 == 50 * 30 * (1 + 17 * 4)
    assert crc == _crc(ck)
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
    bad = bytearray(ck)
    bad[84] ^= 1  # a reserved header word: the header is under the CRC too
    with pytest.raises(lbm.LBMError):
        a.restore(bytes(bad))
    other.close()
    a.close()


def _crc(ck):
    """The header's CRC-32: over the 96-byte header with its crc32 field
    (offset 72) zero, continued over the payload."""
    z = bytearray(ck[:96])
    z[72:76] = b"\0\0\0\0"
    return zlib.crc32(bytes(ck[96:]), zlib.crc32(bytes(z))) & 0xFFFFFFFF


def _forge(ck, fmt, offset, *values):
    """A copy of `ck` with header fields overwritten and the CRC redone, so
    that only the range checks can refuse it."""
    b = bytearray(ck)
    struct.pack_into(fmt, b, offset, *values)
    struct.pack_into("<I", b, 72, _crc(b))
    return bytes(b)


@pytest.mark.parametrize("field,fmt,offset,value", [
    ("cur", "<I", 48, 2), ("materialised", "<I", 52, 7), ("closure", "<I", 56, 2),
    ("omega", "<f", 28, float("nan")), ("omega", "<f", 28, 2.5), ("u_in", "<f", 32, float("inf")),
    ("drift", "<f", 36, float("nan")), ("drift", "<f", 36, -1.0), ("store_inlet", "<I", 76, 2),
    ("rounding", "<I", 80, 2), ("rounding", "<I", 80, 1)])
def test_gpu_checkpoint_header_fields_are_range_checked(lbm, cuda_ok, field, fmt, offset, value):
    """A header whose fields steer device work (the buffer index `cur`, the
    flags, omega, the inlet, the drift bound, the rounding mode: stochastic
    rounding of this f32 lattice included) is refused with LBM_ERR_ARG
    before anything is copied, even with a matching CRC."""
    a = make(lbm, 40, 20, 1, lbm.F32, 3)
    a.iterate(4)
    ck = a.checkpoint()
    want = a.populations()
    with pytest.raises(lbm.LBMError) as e:
        a.restore(_forge(ck, fmt, offset, value))
    assert e.value.code == 1 and "checkpoint header" in str(e.value)
    np.testing.assert_array_equal(a.populations(), want)  # the lattice is untouched
    a.restore(_forge(ck, "<I", 92, 5))  # the reserved word: accepted once the CRC matches
    a.close()


def test_gpu_rows_io_refuses_ranges_that_wrap(lbm, cuda_ok):
    """Row ranges are checked without a 32-bit sum that could wrap: y =
    0xFFFFFFF0 with 0x20 rows is refused, not copied."""
    import ctypes
    L = lbm.load_library()
    a = make(lbm, 40, 20, 1, lbm.F32, 3)
    buf = np.zeros(3 * 40 * 0x20, np.float32)
    p = buf.ctypes.data_as(ctypes.c_void_p)
    for y, n in ((0xFFFFFFF0, 0x20), (20, 1), (19, 2), (0, 0), (0, 0xFFFFFFFF)):
        assert L.lbm_rows_read(a.handle, y, n, 0x7, p, 0) == 1
        assert L.lbm_rows_write(a.handle, y, n, 0x7, p, 0) == 1
    assert L.lbm_rows_read(a.handle, 19, 1, 0x7, p, 0) == 0
    a.close()
