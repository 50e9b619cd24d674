"""Flow observables of a run: drag / lift series, drag coefficient, Strouhal
number and conservation drift.

The reference computes none of these.  The force comes from the engine
(`Lattice.force`, momentum exchange on the bounce-back links, f64); the rest is
host-side analysis of its time series, so the same functions apply to any
run, GPU or CPU.
"""
import numpy as np


def force_series(lat, steps, every):
    """Advance `steps` steps, sampling (drag, lift) every `every` steps.
    Returns (step_index[k], forces[k, 2])."""
    if every < 1 or steps < every:
        raise ValueError("need 1 <= every <= steps")
    idx, out = [], []
    done = 0
    while done + every <= steps:
        lat.iterate(every)
        done += every
        idx.append(lat.get_compute_num())
        out.append(lat.force())
    return np.asarray(idx), np.asarray(out)


def drag_coefficient(mean_drag, u, diameter, rho=1.0):
    """C_d = 2 F / (rho u^2 D) per unit depth."""
    return 2.0 * mean_drag / (rho * u * u * diameter)


def zero_crossing_period(signal, dt=1.0):
    """Mean period of an oscillating signal from its upward crossings of the
    mean, located by linear interpolation between samples.  Returns NaN with
    fewer than two crossings."""
    s = np.asarray(signal, dtype=np.float64)
    s = s - s.mean()
    up = np.nonzero((s[:-1] < 0.0) & (s[1:] >= 0.0))[0]
    if up.size < 2:
        return float("nan")
    t = up + (-s[up]) / (s[up + 1] - s[up])  # fractional crossing positions
    return float((t[-1] - t[0]) / (up.size - 1) * dt)


def strouhal(lift, sample_every, diameter, u):
    """St = f D / u from the lift signal sampled every `sample_every` steps."""
    period = zero_crossing_period(lift, dt=sample_every)
    return float(diameter / (period * u)) if np.isfinite(period) else float("nan")


def drift(series):
    """Relative drift of a conservation sum: (last - first) / |first|."""
    s = np.asarray(series, dtype=np.float64)
    return float((s[-1] - s[0]) / abs(s[0])) if s.size and s[0] != 0 else float("nan")
