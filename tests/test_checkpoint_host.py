"""CPU: the checkpoint header checks, without a GPU (lbm_checkpoint_inspect).

lbm_checkpoint_load runs the same host-side checks before any device work,
so a header that would steer a launch out of bounds (a buffer index `cur` of
2, a NaN omega) is refused here already.  The checkpoints are built in the
test from the layout in include/lbm_checkpoint.h: a 96-byte little-endian
header, then the mask, both buffer sets, the rest plane and the optional
closure records, with zlib's CRC-32 over the header (crc32 field zero) and
the payload."""
import struct
import zlib

import numpy as np
import pytest

HEADER = struct.Struct("<8sIIIiifffQIIIIQIIIIi4x")  # through row_origin; the reserved word zero
assert HEADER.size == 96


def build(nx=12, ny=7, edge=1, storage=0, omega=1.2, u_in=0.05, drift=1.0, steps=42, cur=1, materialised=0,
          closure=0, store_inlet=1, rounding=0, rounding_seed=0, row_origin=0, payload=None, version=2, crc=None):
    es = {0: 4, 1: 2, 2: 2, 3: 8}[storage]
    cells = nx * ny
    n = cells + 17 * cells * es + (cells * 4 if closure else 0)
    if payload is None:
        payload = np.random.default_rng(nx * ny).integers(0, 256, n, dtype=np.uint8).tobytes()
    fields = [b"LBMGB3CK", version, nx, ny, edge, storage, omega, u_in, drift, steps, cur, materialised, closure, es,
              len(payload), 0, store_inlet, rounding, rounding_seed, row_origin]
    h = HEADER.pack(*fields)
    if crc is None:
        crc = zlib.crc32(payload, zlib.crc32(h)) & 0xFFFFFFFF
    fields[15] = crc
    return HEADER.pack(*fields) + payload


def test_a_valid_checkpoint_is_reported(lbm):
    info = lbm.checkpoint_info(build())
    assert (info["nx"], info["ny"], info["edge"], info["storage"], info["steps"]) == (12, 7, 1, 0, 42)
    assert info["omega"] == pytest.approx(1.2) and info["u_in"] == pytest.approx(0.05)
    assert info["closure"] == 0 and info["store_inlet"] == 1
    info = lbm.checkpoint_info(build(storage=1, closure=1, store_inlet=0))
    assert info["storage"] == 1 and info["closure"] == 1 and info["store_inlet"] == 0
    assert (info["rounding"], info["rounding_seed"], info["row_origin"]) == (0, 0, 0)
    info = lbm.checkpoint_info(build(storage=2, rounding=1, rounding_seed=0xDEADBEEF, row_origin=-3))
    assert (info["rounding"], info["rounding_seed"], info["row_origin"]) == (1, 0xDEADBEEF, -3)


@pytest.mark.parametrize("fields", [
    {"cur": 2}, {"materialised": 3}, {"closure": 2}, {"store_inlet": 5},
    {"omega": float("nan")}, {"omega": 2.0}, {"omega": 0.0}, {"u_in": float("inf")},
    {"drift": float("nan")}, {"drift": -1.0}, {"version": 1}, {"edge": 7}, {"storage": 9},
    {"rounding": 2}, {"rounding": 1, "storage": 0}, {"rounding": 1, "storage": 3}])
def test_headers_that_would_steer_device_work_are_refused(lbm, fields):
    """Each of these, with a CRC that matches, is refused with LBM_ERR_ARG."""
    kw = dict(fields)
    if kw.get("storage") == 9:  # a storage the engine does not know: the element size alone cannot be derived
        b = bytearray(build())
        struct.pack_into("<i", b, 24, 9)
        struct.pack_into("<I", b, 72, 0)
        struct.pack_into("<I", b, 72, zlib.crc32(bytes(b[96:]), zlib.crc32(bytes(b[:96]))) & 0xFFFFFFFF)
        data = bytes(b)
    else:
        data = build(**kw)
    with pytest.raises(lbm.LBMError) as e:
        lbm.checkpoint_info(data)
    assert e.value.code == 1


def test_crc_size_and_magic_are_checked(lbm):
    good = build()
    bad = bytearray(good)
    bad[200] ^= 1  # payload byte
    with pytest.raises(lbm.LBMError, match="CRC"):
        lbm.checkpoint_info(bytes(bad))
    bad = bytearray(good)
    bad[92] ^= 1  # the reserved header word: under the CRC too
    with pytest.raises(lbm.LBMError, match="CRC"):
        lbm.checkpoint_info(bytes(bad))
    with pytest.raises(lbm.LBMError):
        lbm.checkpoint_info(good[:-1])  # payload cut short
    with pytest.raises(lbm.LBMError):
        lbm.checkpoint_info(good[:50])  # header cut short
    with pytest.raises(lbm.LBMError):
        lbm.checkpoint_info(build(payload=b"\0" * 10))  # payload size not the grid's
    with pytest.raises(lbm.LBMError):
        lbm.checkpoint_info(b"NOTACKPT" + good[8:])
