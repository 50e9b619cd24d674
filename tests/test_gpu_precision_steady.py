"""16-bit storage precision over a long run that does not shed vortices.

On the benchmark workload the wakes shed vortices, so any rounding
difference grows into a different vortex sequence and the long-run error of
every storage format (f32 included) measures chaos as much as storage.  This
case separates the two: flow past one cylinder at Reynolds number 24 (a wake
that does not shed), 20,000 steps, each storage against the f64 run of the
same state.  The differences then grow smoothly (f32 linearly, from the
rounding of the reference's own f32 arithmetic), not chaotically.  Bars
(relative L2 velocity error over fluid cells, final and second-half
average): f32 <= 2e-3; 16-bit words against the rest weights (the default)
f16 <= 3e-2, bf16 <= 8e-2; against the inlet equilibrium f16 <= 8e-3,
bf16 <= 4e-2, and f16 at least 3x below its rest-weight error.  Measured:
f32 7.1e-4 / 5.5e-4; rest weights f16 2.2e-2 / 1.6e-2, bf16 6.1e-2 /
5.0e-2; inlet equilibrium f16 4.6e-3 / 3.7e-3, bf16 2.4e-2 / 1.7e-2.

With stochastic rounding (lbm_set_rounding) round-to-nearest's bias, which
the steady flow accumulates, is gone: f16 with the default f - w words meets
the 1e-3 target (measured 4.8e-4 / 1.8e-4), bf16 <= 8e-3 (4.3e-3 /
2.6e-3); with the inlet reference both reach the f32 arithmetic's own floor
(f16 7.6e-4 / 6.1e-4, bf16 1.9e-3 / 1.6e-3; bars 2e-3 and 4e-3).  Each
default form improves at least 10x (f16) and 5x (bf16).
"""
import os
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_gpu_storage_error_on_a_steady_wake(lbm, cuda_ok):
    sys.path.insert(0, ROOT)
    import bench
    r = bench.steady_precision(lbm, steps=20000)
    print(r)
    for name, bar in (("f32", 2e-3), ("f16", 3e-2), ("bf16", 8e-2), ("f16_inlet", 8e-3), ("bf16_inlet", 4e-2),
                      ("f16_sr", 1e-3), ("bf16_sr", 8e-3), ("f16_inlet_sr", 2e-3), ("bf16_inlet_sr", 4e-3)):
        for k in ("rel_err_final_velocity", "rel_err_time_avg_velocity"):
            v = r[name][k]
            assert isinstance(v, float) and v <= bar, (name, k, v)
    for k in ("rel_err_final_velocity", "rel_err_time_avg_velocity"):
        assert 3 * r["f16_inlet"][k] <= r["f16"][k], k
        assert 10 * r["f16_sr"][k] <= r["f16"][k], k
        assert 5 * r["bf16_sr"][k] <= r["bf16"][k], k
