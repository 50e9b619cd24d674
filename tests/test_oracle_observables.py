"""Observables of the CPU oracle: momentum-exchange force and Strouhal analysis."""
import numpy as np
import pytest


def test_zero_crossing_period_of_a_sine():
    from lbm_gb300 import observables as ob
    t = np.arange(0, 5000, 10.0)
    s = 0.3 + 0.01 * np.sin(2 * np.pi * t / 823.0 + 0.4)
    assert ob.zero_crossing_period(s, dt=10.0) == pytest.approx(823.0, rel=2e-3)
    assert ob.strouhal(s, 10, 18, 0.08) == pytest.approx(18 / (823.0 * 0.08), rel=2e-3)


def test_force_is_zero_without_solids_and_positive_drag_on_a_cylinder(oracle_mod):
    P = oracle_mod
    from lbm_gb300 import geometry
    o = P.Oracle(80, 40, 1.0 / 0.6, P.EDGE_CHANNEL, P.P_F64)
    o.set_inlet(0.05, apply=False)
    o.init_equilibrium(1.0, 0.05, 0.0)
    with pytest.raises(RuntimeError):
        o.force()
    o.step(5)
    assert np.abs(o.force()).max() == 0.0
    o.set_mask(geometry.single_circle(80, 40, 25, 19.5, 5))
    o.step(300)
    drag, lift = o.force()
    assert drag > 0 and abs(lift) < 0.05 * drag  # symmetric body: small lift before shedding


def test_drag_equals_momentum_given_to_a_wall_pulse(oracle_mod):
    """A single east pulse of excess 2 hitting a one-cell solid at rest: the
    momentum exchanged in the bounce step is 2 * f * c."""
    P = oracle_mod
    nx, ny = 20, 7
    o = P.Oracle(nx, ny, 1.0 / (3 * 1e7 + 0.5), P.EDGE_CHANNEL, P.P_F64)
    w = np.array([1 / 36, 1 / 9, 1 / 36, 1 / 9, 4 / 9, 1 / 9, 1 / 36, 1 / 9, 1 / 36])
    pops = np.broadcast_to(w[:, None, None], (9, ny, nx)).copy()
    pops[5, 3, 9] += 2.0  # east pulse at (9, 3)
    o.put_state(pops)
    mask = np.zeros((ny, nx), np.uint8)
    mask[3, 11] = 1
    o.set_mask(mask)
    o.step(1)  # the pulse streams to (10, 3), next to the solid (11, 3)
    o.step(1)  # its collision is the last one: (10, 3) will take its own e back as w
    fx, fy = o.force()
    # the rest-state links around the solid cancel pairwise; the pulse's excess 2 adds 2 * 2 along +x
    assert fx == pytest.approx(2.0 * 2.0, rel=1e-6)
    assert abs(fy) < 1e-12
