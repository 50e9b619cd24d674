"""CPU: the oracle's restatement of stochastic rounding (lbm_set_rounding).

The conversions are pinned to known answers of the GPU's own cvt.rs
instructions (tests/golden/cvt_rs.npz, made by tests/golden/make_cvt_rs.py
on a GB300); the hash that feeds them random bits is checked against a
second, Python restatement; the rounding is unbiased by construction: over
all 2^k random words a value's roundings average to the value exactly."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_conversions_match_the_gpu_known_answers(oracle_mod):
    P = oracle_mod
    g = np.load(os.path.join(HERE, "golden", "cvt_rs.npz"))
    a, b, r = g["a"], g["b"], g["rbits"]
    f16, bf16 = g["f16x2"], g["bf16x2"]
    assert len(a) == 4096
    for i in range(len(a)):
        ri = int(r[i])
        # a rounds to the high half with the upper random field, b to the low half
        assert P.half_rs(a[i], (ri >> 16) & 0x1FFF) == int(f16[i]) >> 16, i
        assert P.half_rs(b[i], ri & 0x1FFF) == int(f16[i]) & 0xFFFF, i
        assert P.bf16_rs(a[i], ri >> 16) == int(bf16[i]) >> 16, i
        assert P.bf16_rs(b[i], ri & 0xFFFF) == int(bf16[i]) & 0xFFFF, i
    # the fixture spans the input classes the storage meets
    ab = np.abs(np.concatenate([a, b]).astype(np.float64))
    assert (ab < 2.0 ** -14).sum() > 300 and (ab > 65504).sum() > 100 and (ab == 0).sum() > 10


def _fmix32(h):
    h ^= h >> 16
    h = (h * 0x85EBCA6B) & 0xFFFFFFFF
    h ^= h >> 13
    h = (h * 0xC2B2AE35) & 0xFFFFFFFF
    return h ^ (h >> 16)


def _sr_mul(q):
    m = 0xFFFFFFFFFFFFFFFF
    z = ((q + 1) * 0x9E3779B97F4A7C15) & m
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
    z ^= z >> 31
    return (z >> 32) | 1


def _bits(seed, t, y, x, q):
    st = _fmix32(seed ^ ((t * 0x9E3779B1) & 0xFFFFFFFF))
    ky = _fmix32((st + (y * 0x85EBCA77)) & 0xFFFFFFFF)
    kp = _fmix32(ky ^ (((x >> 1) * 0xC2B2AE3D) & 0xFFFFFFFF))
    return (kp * _sr_mul(q)) & 0xFFFFFFFF


def test_hash_restated_twice_agrees(oracle_mod):
    P = oracle_mod
    rng = np.random.default_rng(3)
    for _ in range(2000):
        seed, t = int(rng.integers(1 << 32)), int(rng.integers(1 << 40))
        y, x, q = int(rng.integers(-50, 1 << 20)), int(rng.integers(0, 1 << 20)), int(rng.integers(9))
        assert P.sr_bits(seed, t, y, x, q) == _bits(seed, t & 0xFFFFFFFF, y & 0xFFFFFFFF, x, q)
    # a column pair shares one word; every other coordinate changes it
    assert P.sr_bits(1, 5, 7, 10, 3) == P.sr_bits(1, 5, 7, 11, 3)
    base = P.sr_bits(1, 5, 7, 10, 3)
    for other in [(2, 5, 7, 10, 3), (1, 6, 7, 10, 3), (1, 5, 8, 10, 3), (1, 5, 7, 12, 3), (1, 5, 7, 10, 4)]:
        assert P.sr_bits(*other) != base


def test_hash_bits_are_close_to_uniform(oracle_mod):
    """The 13-bit fields the binary16 rounding reads, over a row of cells and
    over steps of one cell: every 1/16 of the range within 15 % of its share."""
    P = oracle_mod
    for vals in ([P.sr_bits(9, 1, 3, x, q) for x in range(0, 8192, 2) for q in range(9)],
                 [P.sr_bits(9, t, 3, 100, 5) for t in range(20000)]):
        v = np.array(vals, np.uint64)
        for field in (v & 0x1FFF, (v >> 16) & 0x1FFF):
            h = np.bincount((field >> 9).astype(np.int64), minlength=16)
            assert np.all(np.abs(h / h.mean() - 1) < 0.15), h


@pytest.mark.parametrize("v", [1.0 + 2.0 ** -11, -0.0371, 3.14159e-3, 0.40123, -1.7e-2, 2.0 ** -13 * 1.37,
                               6.1e-6, -3.3e-7])
def test_rounding_is_unbiased_over_all_random_words(oracle_mod, v):
    """sum_r floor(q + r / 2^k) over the 2^k words r equals floor(2^k q): the
    roundings of an f32 value (k = 13 dropped bits for binary16, 16 for
    bfloat16) average to the value itself, subnormal binary16 included
    down to its 2^-37 resolution."""
    P = oracle_mod
    f = np.float32(v)
    h = np.array([P.half_rs(f, r) for r in range(1 << 13)], np.uint16).view(np.float16).astype(np.float64)
    want = float(f) if abs(float(f)) >= 2.0 ** -14 else np.trunc(float(f) * 2.0 ** 37) / 2.0 ** 37
    assert h.mean() == pytest.approx(want, rel=0, abs=1e-18)
    bb = np.array([P.bf16_rs(f, r) for r in range(1 << 16)], np.uint32)
    bv = (bb << 16).view(np.float32).astype(np.float64)
    assert bv.mean() == float(f)


def test_oracle_runs_are_seeded_and_differ_from_nearest(oracle_mod):
    P = oracle_mod
    nx, ny = 48, 24
    rng = np.random.default_rng(2)
    mask = (rng.random((ny, nx)) < 0.1).astype(np.uint8)

    def run(mode, seed, prec=P.P_F16):
        o = P.Oracle(nx, ny, 1.0 / 0.6, P.EDGE_CHANNEL, prec)
        o.set_inlet(0.08, apply=False)
        o.init_equilibrium(1.0, 0.08, 0.0, 1e-2, 5)
        o.set_mask(mask)
        o.set_rounding(mode, seed)
        o.step(40)
        return o.state()[0]

    a, b, c, d = run(1, 7), run(1, 7), run(1, 8), run(0, 7)
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, c) and not np.array_equal(a, d)
    # f32 storage ignores the request (the engine refuses it)
    np.testing.assert_array_equal(run(1, 7, P.P_F32), run(0, 7, P.P_F32))


def test_stochastic_rounding_cuts_the_steady_error_in_the_oracle(oracle_mod):
    """The mechanism behind stochastic rounding, on the CPU: a steady cylinder
    wake (192 x 64, r 6, tau 0.8, u 0.05, 6000 steps) run in f64, and in f16
    and bf16 (f - w words) with each rounding.  Round-to-nearest gives each
    cell the same error every step and the flow accumulates it; unbiased
    rounding removes that, so the velocity error against f64 falls at least
    3x (measured 4.9e-3 -> 1.1e-3 in f16, 2.0e-2 -> 3.3e-3 in bf16)."""
    from lbm_gb300 import geometry
    P = oracle_mod
    nx, ny, steps = 192, 64, 6000
    mask = geometry.single_circle(nx, ny, 48, 32, 6)
    fl = mask == 0
    fl[:, 0] = False

    def velocity(prec, sr):
        o = P.Oracle(nx, ny, float(np.float32(1 / 0.8)), P.EDGE_CHANNEL, prec)
        o.set_inlet(float(np.float32(0.05)), apply=False)
        o.init_equilibrium(1.0, float(np.float32(0.05)), 0.0, 0.0, 0)
        o.set_mask(mask)
        if sr:
            o.set_rounding(1, 7)
        o.step(steps)
        _, rho, jx, jy = o.state()
        return np.stack([jx / rho, jy / rho])

    ref = velocity(P.P_F64, False)

    def err(u):
        return float(np.linalg.norm((u - ref)[:, fl]) / np.linalg.norm(ref[:, fl]))

    for prec in (P.P_F16, P.P_BF16):
        rn, sr = err(velocity(prec, False)), err(velocity(prec, True))
        print(prec, rn, sr)
        assert 3 * sr < rn, (prec, rn, sr)
