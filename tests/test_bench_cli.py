"""bench.py's command line (CPU only): the run-length and implementation
flags, the section switches and the small profiling cases all parse; nothing
is run."""
import subprocess
import sys

from conftest import ROOT


def test_bench_flags():
    out = subprocess.run([sys.executable, "bench.py", "--help"], cwd=ROOT, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr
    for flag in ("--gpus", "--steps", "--warmup", "--impl", "--no-batched", "--no-closure", "--no-precision",
                 "--no-variants", "--no-cpu-baseline", "--kernel-only", "--case", "--precision-steps",
                 "--batched-steps", "--cpu-seconds", "--min-seconds", "--slab", "--no-slab"):
        assert flag in out.stdout, flag
