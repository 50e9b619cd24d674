"""Generate the golden fixtures in this folder from the reference's own shaders.

The reference (PPLUSCHT/LBM) ships no tests or vectors for its step, and its
GPU path cannot run here.  Its per-cell arithmetic lives in WGSL compute
shaders, which oracle/wgsl2cpp.py translates mechanically to C++ and
oracle/ref_host.cpp dispatches in the reference's pass order.  This script runs
that translation (oracle/_ref/libref.so, built by `make -C oracle ref` from the
reference tree) on small seeded cases and stores its outputs, so that parity
checks still have reference outputs where the reference tree is absent.

Initial states come from the oracle's restatement of set_equil (lbm.rs:611-643;
Rust host code, not a shader) and are uploaded to both buffer sets, as
custom_speed does.  Run:  python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as P  # noqa: E402
from lbm_gb300 import geometry  # noqa: E402

# name: (nx, ny, tau, ux, noise, seed, steps, shape)
CASES = {
    "cfg0_256x128_1000": (256, 128, 0.6, 0.1, 1e-4, 0, 1000, ("circle", 64, 64, 12)),
    "small_64x32_300": (64, 32, 0.55, 0.08, 1e-3, 3, 300, ("circle", 20, 15, 5)),
    "odd_33x17_200": (33, 17, 0.7, 0.05, 1e-3, 5, 200, ("random", 0.15, 11)),
    "tiny_8x6_50": (8, 6, 0.9, 0.1, 1e-2, 9, 50, ("random", 0.2, 13)),
}


def initial_state(nx, ny, tau, ux, noise, seed):
    o = P.Oracle(nx, ny, 1.0 / tau, P.EDGE_REF, P.P_F32)
    o.init_equilibrium(1.0, ux, 0.0, noise, seed)
    pops, _, _, _ = o.state()
    return pops.astype(np.float32)


def make_mask(nx, ny, shape):
    if shape[0] == "circle":
        m = geometry.single_circle(nx, ny, shape[1], shape[2], shape[3])
    else:
        rng = np.random.default_rng(shape[2])
        m = (rng.random((ny, nx)) < shape[1]).astype(np.uint8)
    m[0, :] = 1
    m[-1, :] = 1
    return m


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_case(name, nx, ny, tau, ux, noise, seed, steps, shape):
    pops0 = initial_state(nx, ny, tau, ux, noise, seed)
    mask = make_mask(nx, ny, shape)
    r = P.RefShaders(nx, ny, np.float32(1.0 / tau))
    r.put_state(pops0)
    r.set_barrier(mask)
    r.iterate(steps)
    pops, rho, jx, jy = r.state()
    curl = r.summary(0)
    out = dict(nx=nx, ny=ny, tau=tau, omega=np.float32(1.0 / tau), ux=ux, noise=noise, seed=seed, steps=steps,
               mask=mask, init_sha=sha(pops0), pops_sha=sha(pops), rho=rho, jx=jx, jy=jy, curl=curl)
    if pops.size <= 9 * 64 * 32:
        out["pops"] = pops
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def run_edit_case():
    """Barrier edits and a viscosity change between iterate calls."""
    nx, ny, tau = 48, 24, 0.6
    pops0 = initial_state(nx, ny, tau, 0.1, 1e-3, 21)
    mask = make_mask(nx, ny, ("circle", 14, 12, 4))
    r = P.RefShaders(nx, ny, np.float32(1.0 / tau))
    r.put_state(pops0)
    r.set_barrier(mask)
    r.iterate(40)
    draw = np.array([[30 + 10 * nx, 1], [31 + 10 * nx, 1], [30 + 11 * nx, 1], [14 + 12 * nx, 0],
                     [nx * ny + 5, 1]], np.uint32)  # last one clamps to the last cell
    r.draw_points(draw)
    r.iterate(25)
    omega2 = np.float32(1.0 / (3.0 * 0.05 + 0.5))
    r.set_omega(omega2)
    r.iterate(35)
    pops, rho, jx, jy = r.state()
    np.savez_compressed(os.path.join(HERE, "edits_48x24.npz"), nx=nx, ny=ny, tau=tau, omega=np.float32(1.0 / tau),
                        omega2=omega2, mask=mask, draw=draw, init_sha=sha(pops0), pops=pops, rho=rho, jx=jx, jy=jy,
                        barrier_after=r.barrier())


def run_single_cell_cases():
    """single_cell presets (lbm.rs:1482-1500) under near-pure streaming
    (update_viscosity(1e7): omega = 1/(3e7 + 0.5), tutorial StreamDemo)."""
    nx, ny = 40, 20
    omega = np.float32(1.0 / (3.0 * 1e7 + 0.5))
    res = {}
    for d in range(9):
        o = P.Oracle(nx, ny, float(omega), P.EDGE_REF, P.P_F32)
        o.single_cell(d)
        pops0, _, _, _ = o.state()
        r = P.RefShaders(nx, ny, omega)
        r.put_state(pops0.astype(np.float32))
        r.iterate(7)
        pops, rho, _, _ = r.state()
        res["pops_%d" % d] = pops
    np.savez_compressed(os.path.join(HERE, "single_cell_40x20.npz"), nx=nx, ny=ny, omega=omega, steps=7, **res)


def main():
    if not P.build(ref=True):
        raise SystemExit("the reference's shaders are not available: cannot regenerate fixtures")
    for name, args in CASES.items():
        run_case(name, *args)
    run_edit_case()
    run_single_cell_cases()
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
