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


def test_flags_for_the_storage_options():
    out = subprocess.run([sys.executable, "bench.py", "--help"], cwd=ROOT, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr
    for flag in ("--inlet-reference", "--stochastic", "--batched-split"):
        assert flag in out.stdout, flag


class _FakeLattice:
    """Counts steps and launches as the engine reports them."""

    def __init__(self):
        self.steps, self.launches, self.inits = 0, 0, 0

    def get_compute_num(self):
        return self.steps

    def launch_count(self):
        return self.launches

    def init_equilibrium(self, *a):
        self.steps, self.inits = 0, self.inits + 1
        self.launches += 1

    def iterate(self, n):
        self.steps += n
        self.launches += n

    def synchronize(self):
        pass


def test_restarter_keeps_timed_runs_inside_the_finite_horizon():
    """The timed calls restart (untimed) before a call would pass
    RESTART_STEPS; the restart's own launches are counted apart, so the
    launches per timed call stay exact."""
    sys.path.insert(0, ROOT)
    import bench
    lat = _FakeLattice()
    k = 3000
    rs = bench.restarter(lat, k)
    timed_launches = 0
    for _ in range(20):
        rs()
        assert lat.steps + k <= bench.RESTART_STEPS
        before = lat.launches
        lat.iterate(k)  # the timed call
        timed_launches += lat.launches - before
    assert rs.restarts == lat.inits >= 1
    assert timed_launches == 20 * k
    assert rs.launches == lat.launches - timed_launches  # init + its one step, per restart
    # short calls restart only when they would cross the horizon
    lat2 = _FakeLattice()
    rs2 = bench.restarter(lat2, 20)
    for _ in range(bench.RESTART_STEPS // 20):
        rs2()
        lat2.iterate(20)
    assert rs2.restarts == 0
    rs2()
    assert rs2.restarts == 1 and lat2.steps == 1
