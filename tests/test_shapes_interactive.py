"""Barrier shapes, presets and the interactive frame loop (host logic, no GPU).

Line pixels follow a restatement of the line_drawing crate's Bresenham, which
no reference test pins; the tests check the properties the reference's code
relies on (end points included, 8-connected, one cell per major-axis step)
and the shape constructions around it (thickening, diagonal fill, presets,
undo history) against the reference's rules."""
import numpy as np
import pytest

from lbm_gb300 import SummaryStat, ColorMap
from lbm_gb300 import shapes as S
from lbm_gb300 import interactive as I


@pytest.mark.parametrize("p0,p1", [((0, 0), (7, 3)), ((5, 5), (1, 9)), ((3, 8), (3, 0)), ((2, 2), (9, 9)),
                                   ((10, 1), (0, 4)), ((4, 4), (4, 4)), ((0, 6), (2, 0))])
def test_bresenham_properties(p0, p1):
    pts = S.bresenham(p0, p1)
    assert pts[0] == p0 and pts[-1] == p1
    assert len(pts) == max(abs(p1[0] - p0[0]), abs(p1[1] - p0[1])) + 1
    for a, b in zip(pts, pts[1:]):
        assert max(abs(a[0] - b[0]), abs(a[1] - b[1])) == 1
    # every cell lies within one cell of the exact segment along the minor axis
    # (the crate's error term starts at dy - dx, so cells may trail the line by
    # up to one cell rather than half)
    (x0, y0), (x1, y1) = p0, p1
    if abs(x1 - x0) >= abs(y1 - y0) and x1 != x0:
        for x, y in pts:
            assert abs(y - (y0 + (y1 - y0) * (x - x0) / (x1 - x0))) < 1.0


def test_bresenham_first_octant_cells():
    assert S.bresenham((0, 0), (4, 1)) == [(0, 0), (1, 0), (2, 0), (3, 0), (4, 1)]
    assert S.bresenham((0, 0), (4, 3)) == [(0, 0), (1, 0), (2, 1), (3, 2), (4, 3)]
    assert S.bresenham((0, 0), (7, 3)) == [(0, 0), (1, 0), (2, 0), (3, 1), (4, 1), (5, 2), (6, 2), (7, 3)]


def test_line_is_three_cells_thick_and_diagonals_are_filled():
    ln = S.Line((10, 5), (10, 15), 40, 30)
    cells = {(x, y) for x, y, v in ln.points}
    assert all(v for _, _, v in ln.points)
    # vertical line: the centre column plus one neighbour column on each side of the construction
    assert {(10, y) for y in range(5, 16)} <= cells
    d = S.Line((2, 2), (12, 12), 40, 30)
    dc = {(x, y) for x, y, _ in d.points}
    for x, y in S.bresenham((12, 12), (2, 2)):
        assert (x, y) in dc
    # a 45-degree walk fills both corner cells of every diagonal step, so the barrier is 4-connected
    for x, y in S.bresenham((12, 12), (2, 2))[1:]:
        assert (x + 1, y) in dc and (x, y + 1) in dc
    with pytest.raises(ValueError):
        S.Line((0, 0), (40, 3), 40, 30)


def test_erased_line_and_blob_join_override():
    e = S.Line((20, 10), (30, 20), 64, 48, erased=True)
    assert e.points and not any(v for _, _, v in e.points)
    assert len({(x, y) for x, y, _ in e.points}) > 10 * len(S.Line((20, 10), (30, 20), 64, 48).points) // 3
    b = S.Blob()
    b.join(S.Line((20, 10), (30, 20), 64, 48))
    b.join(e)  # erase wins where they overlap
    assert (25, 15, True) not in b.points and (25, 15, False) in b.points


def test_points_vector_indices():
    ln = S.Line((3, 2), (6, 2), 10, 8)
    pv = np.array(S.points_vector(ln, 10)).reshape(-1, 2)
    got = {(i % 10, i // 10) for i, v in pv}
    assert got == {(x, y) for x, y, _ in ln.points}
    assert (pv[:, 1] == 1).all()


@pytest.mark.parametrize("x,y", [(200, 100), (513, 287), (1000, 400)])
def test_presets_stay_inside_the_grid(x, y):
    for name, fn in S.PRESETS.items():
        for shape in fn(x, y):
            for px, py, v in shape.points:
                assert 0 <= px < x and 0 <= py < y and v
    curl = {(px, py) for px, py, _ in S.curl_barrier(x, y)[0].points}
    assert (4 * x // 10, y // 4) in curl and (4 * x // 10, y // 2) in curl
    w = S.welcome_barrier(x, y)[0]
    assert len(w.points) > 10 * (y // 4)


def test_calculate_dimensions():
    x, y, px = I.calculate_dimensions(230400, 1920, 1080)
    assert x == 640 and y == 360 and px == pytest.approx(3.0)


class FakeLattice:
    """Records the calls the frame loop makes."""

    def __init__(self, x, y):
        self.x, self.y = x, y
        self.calls = []
        self.steps = 0

    def __getattr__(self, name):
        def rec(*a):
            self.calls.append((name,) + a)
            if name == "iterate":
                self.steps += a[0]
            if name == "render":
                return np.zeros((a[1], a[0], 3), np.float32)
        return rec


def names(lat):
    return [c[0] for c in lat.calls]


def test_frame_loop_order_pause_and_step_mode():
    lat = FakeLattice(64, 32)
    app = I.App(lat)
    f = app.redraw()  # first frame: output_changed is initially set
    assert f is not None and lat.steps == 15
    assert names(lat) == ["set_summary", "iterate", "render"]
    lat.calls.clear()
    app.toggle_pause()
    assert app.redraw() is None and lat.calls == []
    app.set_color_map(ColorMap.Viridis)
    assert app.redraw() is not None and names(lat) == ["set_color_map", "render"] and lat.steps == 15
    app.toggle_pause()
    app.set_step_mode()
    lat.calls.clear()
    assert app.redraw() is None and lat.steps == 15
    app.take_step()
    assert app.redraw() is not None and lat.steps == 16
    assert app.redraw() is None
    app.release_step_mode()
    app.update_compute_rate(7)
    app.update_viscosity(0.05)
    app.set_output(SummaryStat.Speed)
    lat.calls.clear()
    app.redraw()
    assert names(lat) == ["set_summary", "update_omega_buffer", "iterate", "render"]
    assert lat.calls[1][1] == pytest.approx(1.0 / (3.0 * 0.05 + 0.5))
    assert lat.steps == 23


def test_presets_and_fluid_presets_in_the_loop():
    lat = FakeLattice(100, 50)
    app = I.App(lat)
    app.redraw()
    lat.calls.clear()
    app.change_barrier_preset(I.BarrierPreset.Chaos)
    app.change_fluid_preset(I.FluidPreset.SingleEast)
    app.redraw()
    n = names(lat)
    assert n[0] == "reset_barrier" and n.count("draw_points") == 4
    assert ("single_cell", 5) in lat.calls
    lat.calls.clear()
    app.update_flow_speed(0.07)
    app.redraw()
    assert ("custom_speed", 0.07) in lat.calls


def test_drawing_and_undo_restore_the_barrier():
    lat = FakeLattice(80, 40)
    app = I.App(lat)
    app.redraw()
    app.set_draw_type(I.ClickType.Line)
    app.press((10, 10))
    app.release()
    app.press((30, 20))
    app.release()
    lat.calls.clear()
    app.redraw()
    drawn = [c for c in lat.calls if c[0] == "draw_points"]
    assert len(drawn) == 1
    pv = np.array(drawn[0][1]).reshape(-1, 2)
    assert (pv[:, 1] == 1).all() and len(pv) == len(S.Line((10, 10), (30, 20), 80, 40).points)
    app.undo()
    lat.calls.clear()
    app.redraw()
    undone = [c for c in lat.calls if c[0] == "draw_points"]
    assert len(undone) == 1
    pu = np.array(undone[0][1]).reshape(-1, 2)
    assert sorted(pu[:, 0]) == sorted(pv[:, 0]) and (pu[:, 1] == 0).all()
