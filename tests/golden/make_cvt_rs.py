"""Known-answer vectors of the GPU's stochastic-rounding conversions
(cvt.rs.f16x2.f32, cvt.rs.bf16x2.f32), which the 16-bit storage rounds with
under lbm_set_rounding(..., LBM_ROUND_STOCHASTIC).

Needs a GB300 (sm_103a) and nvcc: builds cvt_rs_probe.cu, runs it (2^20
seeded input pairs and random-bit words) and keeps a seeded selection of 4096
cases, the 1024 single-bit / structured random words first, then 3072 drawn
across the input classes, in cvt_rs.npz:
  a, b     float32 inputs (a goes to the high half of each result word)
  rbits    uint32 random bits
  f16x2    uint32 result of cvt.rs.f16x2.f32 d, a, b, rbits
  bf16x2   uint32 result of cvt.rs.bf16x2.f32 d, a, b, rbits

    python tests/golden/make_cvt_rs.py [--from-dump probe.bin]
"""
import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
N = 1 << 20


def run_probe(path):
    exe = os.path.join(tempfile.mkdtemp(), "cvt_rs_probe")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-o", exe,
                    os.path.join(HERE, "cvt_rs_probe.cu")], check=True)
    subprocess.run([exe, path], check=True)


def select(dump):
    d = np.fromfile(dump, dtype=np.uint32)
    assert d.size == 7 * N, d.size
    a, b, r, f16, bf16 = d[0:N], d[N:2 * N], d[2 * N:3 * N], d[3 * N:4 * N], d[4 * N:5 * N]
    first = np.arange(1024)
    rng = np.random.default_rng(20261204)
    rest = np.sort(rng.choice(np.arange(4096, N), size=3072, replace=False))
    idx = np.concatenate([first, rest])
    return dict(a=a[idx].view(np.float32), b=b[idx].view(np.float32), rbits=r[idx], f16x2=f16[idx],
                bf16x2=bf16[idx])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--from-dump", help="an earlier output of cvt_rs_probe instead of running it")
    args = ap.parse_args()
    dump = args.from_dump
    if not dump:
        dump = os.path.join(tempfile.mkdtemp(), "cvt_rs_probe.bin")
        run_probe(dump)
    np.savez_compressed(os.path.join(HERE, "cvt_rs.npz"), **select(dump))
    print("wrote", os.path.join(HERE, "cvt_rs.npz"))


if __name__ == "__main__":
    sys.exit(main())
