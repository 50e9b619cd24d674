"""The CPU oracle against the reference's own shader arithmetic.

Two pins: (1) the committed golden fixtures, generated by
tests/golden/make_golden.py from the reference's WGSL shaders translated to C++
(oracle/wgsl2cpp.py + oracle/ref_host.cpp); (2) live runs of that translation
when it can be built here (the reference tree is present).  Both must agree
with the oracle restatement bit for bit in f32.
"""
import hashlib

import numpy as np
import pytest

from conftest import golden

CASES = ["cfg0_256x128_1000", "small_64x32_300", "odd_33x17_200", "tiny_8x6_50"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_fixture(oracle_mod, name):
    P = oracle_mod
    g = golden(name)
    nx, ny = int(g["nx"]), int(g["ny"])
    o = P.Oracle(nx, ny, float(g["omega"]), P.EDGE_REF, P.P_F32)
    o.init_equilibrium(1.0, float(g["ux"]), 0.0, float(g["noise"]), int(g["seed"]))
    p0, _, _, _ = o.state()
    assert sha(p0.astype(np.float32)) == str(g["init_sha"])
    o.set_mask(g["mask"])
    o.step(int(g["steps"]))
    pops, rho, jx, jy = o.state()
    assert sha(pops.astype(np.float32)) == str(g["pops_sha"])
    if "pops" in g:
        np.testing.assert_array_equal(pops.astype(np.float32), g["pops"])
    np.testing.assert_array_equal(rho.astype(np.float32), g["rho"])
    np.testing.assert_array_equal(jx.astype(np.float32), g["jx"])
    np.testing.assert_array_equal(jy.astype(np.float32), g["jy"])
    curl = o.curl_ref().astype(np.float32)
    inner = np.zeros((ny, nx), bool)
    inner[: ny - 1, 1:] = True
    np.testing.assert_array_equal(curl[inner], g["curl"][inner])


def test_oracle_matches_reference_edits_fixture(oracle_mod):
    P = oracle_mod
    g = golden("edits_48x24")
    nx, ny = int(g["nx"]), int(g["ny"])
    o = P.Oracle(nx, ny, float(g["omega"]), P.EDGE_REF, P.P_F32)
    o.init_equilibrium(1.0, 0.1, 0.0, 1e-3, 21)
    o.set_mask(g["mask"])
    o.step(40)
    o.barrier_pairs(g["draw"])
    o.step(25)
    o.set_omega(float(g["omega2"]))
    o.step(35)
    pops, rho, jx, jy = o.state()
    np.testing.assert_array_equal(o.mask(), g["barrier_after"].astype(np.uint8))
    np.testing.assert_array_equal(pops.astype(np.float32), g["pops"])
    np.testing.assert_array_equal(rho.astype(np.float32), g["rho"])


def test_oracle_matches_reference_single_cell_fixture(oracle_mod):
    P = oracle_mod
    g = golden("single_cell_40x20")
    nx, ny = int(g["nx"]), int(g["ny"])
    for d in range(9):
        o = P.Oracle(nx, ny, float(g["omega"]), P.EDGE_REF, P.P_F32)
        o.single_cell(d)
        o.step(int(g["steps"]))
        pops, _, _, _ = o.state()
        np.testing.assert_array_equal(pops.astype(np.float32), g["pops_%d" % d])


def _live_ref(P):
    if not P.ref_available():
        pytest.skip("translated reference shaders not built (reference tree absent)")


@pytest.mark.parametrize("nx,ny,seed", [(8, 6, 1), (33, 17, 2), (40, 9, 3), (17, 31, 4)])
def test_oracle_matches_live_reference_random(oracle_mod, nx, ny, seed):
    P = oracle_mod
    _live_ref(P)
    rng = np.random.default_rng(seed)
    omega = float(np.float32(rng.uniform(0.6, 1.9)))
    o = P.Oracle(nx, ny, omega, P.EDGE_REF, P.P_F32)
    o.init_equilibrium(1.0, rng.uniform(0.0, 0.15), 0.0, 1e-2, seed)
    mask = (rng.random((ny, nx)) < 0.2).astype(np.uint8)
    mask[0] = 1
    if seed % 2:
        mask[-1] = 1  # otherwise the last row is fluid but still never streamed
    o.set_mask(mask)
    p0, _, _, _ = o.state()
    r = P.RefShaders(nx, ny, np.float32(omega))
    r.put_state(p0.astype(np.float32))
    r.set_barrier(mask)
    for chunk in (3, 10, 1):
        o.step(chunk)
        r.iterate(chunk)
        pairs = np.stack([rng.integers(0, nx * ny + 3, 5), rng.integers(0, 2, 5)], 1).astype(np.uint32)
        o.barrier_pairs(pairs)
        r.draw_points(pairs)
    po, ro, jxo, jyo = o.state()
    pr, rr, jxr, jyr = r.state()
    np.testing.assert_array_equal(po.astype(np.float32), pr)
    np.testing.assert_array_equal(ro.astype(np.float32), rr)
    np.testing.assert_array_equal(jxo.astype(np.float32), jxr)
    np.testing.assert_array_equal(jyo.astype(np.float32), jyr)
    np.testing.assert_array_equal(o.mask(), r.barrier().astype(np.uint8))
