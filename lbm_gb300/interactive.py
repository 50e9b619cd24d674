"""The reference's interactive frame loop as a host-side driver over a lattice.

lbm-wgpu keeps its user interface in static flags that the browser sets
(WASMInteraction, lib.rs:447-537) and that the winit loop consumes on each
redraw (lib.rs:108-204), with mouse strokes turned into barrier shapes by a
click handler with an undo history (lib.rs:218-426).  `App` restates that
state machine without a window: the setters record the same flags, and
`redraw()` applies them in the reference's order (barrier preset, undo,
fluid preset, output, colour map, pending strokes, viscosity, then
`compute_per_render` steps, a single step in step mode, or nothing when
paused) and returns the frame as a headless RGB buffer (or None when the
reference would not have re-rendered).  `press`, `move` and `release` stand
in for the mouse events (lib.rs:80-106).  Any object with the `Lattice`
methods used here can be driven, so the logic is testable without a GPU.
"""
from . import ColorMap, SummaryStat
from .shapes import PRESETS, Blob, Curve, CurveCollection, Line, points_vector


class ClickType:
    Line, Erase, Draw, Inactive = 0, 1, 2, 3


class FluidPreset:
    Equilibrium, CustomSpeed, SingleNorth, SingleOrigin, SingleEast, SingleNorthEast = range(6)


class BarrierPreset:
    Welcome, Tunnel, Curl, Chaos = range(4)


_PRESET_NAMES = {BarrierPreset.Welcome: "Welcome", BarrierPreset.Tunnel: "Tunnel", BarrierPreset.Curl: "Curl",
                 BarrierPreset.Chaos: "Chaos"}


def calculate_dimensions(res_cells, width, height):
    """Grid size and pixel size for a window (lib.rs:547-555): res_cells is
    the Resolution value (cell budget)."""
    import math
    aspect = height / width
    x = int(math.floor(math.sqrt(res_cells / aspect)))
    pixel = width / x
    y = int(math.floor(height / pixel))
    return x, y, pixel


class ClickHandler:
    def __init__(self, x, y):
        self.x, self.y = x, y
        self.current_type = ClickType.Draw
        self.line_points = []
        self.current_blob = Blob()
        self.current_curve = Curve()
        self.contiguous_curve = CurveCollection()
        self.undo_stack = []
        self.history = {}

    def clear_barrier(self):
        self.current_curve = Curve()
        self.contiguous_curve = CurveCollection()
        self.undo_stack.clear()
        self.history.clear()
        self.current_blob.empty()
        self.line_points.clear()

    def _segment(self, loc, erase, ydim=None):
        if erase:
            self.current_curve.erase_segment(loc, self.x, self.y if ydim is None else ydim)
        else:
            self.current_curve.add_segment(loc, self.x, self.y)

    def handle_movement(self, loc):
        if self.current_type in (ClickType.Erase, ClickType.Draw):
            self._segment(loc, self.current_type == ClickType.Erase)

    def handle_release(self):
        if self.current_type in (ClickType.Erase, ClickType.Draw):
            self.current_blob.join(self.current_curve)
            temp, self.current_curve = self.current_curve, Curve()
            self.contiguous_curve.add_curve(temp)
            temp, self.contiguous_curve = self.contiguous_curve, CurveCollection()
            self._add_to_history(temp)

    def empty_all(self):
        self.current_blob.empty()
        self.current_curve.empty()

    def handle_click(self, loc):
        if self.current_type == ClickType.Line:
            self.line_points.append(loc)
            if len(self.line_points) >= 2:
                shape = Line(self.line_points[0], self.line_points[1], self.x, self.y)
                self.current_blob.join(shape)
                self._add_to_history(shape)
                self.line_points.clear()
        elif self.current_type in (ClickType.Erase, ClickType.Draw):
            self._segment(loc, self.current_type == ClickType.Erase)

    def switch_click_type(self, t):
        self.current_type = t
        self.line_points.clear()

    def update(self, pressed, loc, click_type):
        self.current_blob.empty()
        if pressed and click_type in (ClickType.Draw, ClickType.Erase):
            temp, self.current_curve = self.current_curve, Curve()
            self.contiguous_curve.add_curve(temp)
            # the reference passes the grid width as both dimensions when erasing (lib.rs:362)
            self._segment(loc, click_type == ClickType.Erase, ydim=self.x)

    def undo(self):
        if self.current_blob.is_empty() and self.current_curve.is_empty():
            return self._remove_shape(self.undo_stack.pop()) if self.undo_stack else None
        self.current_blob.empty()
        self.current_curve.empty()
        return None

    def validate_click(self, loc):
        cx = self.x + loc[0] if loc[0] < 0 else (self.x - 1 if loc[0] >= self.x else loc[0])
        cy = self.y + loc[1] if loc[1] < 0 else (self.y - 1 if loc[1] >= self.y else loc[1])
        return cx, cy

    def _add_to_history(self, shape):
        for x, y, v in shape.points:
            self.history.setdefault((x, y), []).append(v)
        self.undo_stack.append(shape)

    def _remove_shape(self, shape):
        pts = []
        for x, y, v in shape.points:
            vec = self.history.get((x, y))
            if vec is not None:
                vec.pop()
                pts.append((x, y, vec[-1] if vec else False))
                if not vec:
                    del self.history[(x, y)]
            else:
                pts.append((x, y, False))
        pts.sort()
        b = Blob()
        b.add(pts, self.x, self.y)
        return b


class App:
    """Headless frame loop over `lattice` (an lbm_gb300.Lattice or a stand-in)."""

    def __init__(self, lattice, width=None, height=None):
        self.lat = lattice
        self.x, self.y = lattice.x, lattice.y
        self.width, self.height = width or self.x, height or self.y
        self.click = ClickHandler(self.x, self.y)
        self.pressed = False
        self.position = (0, 0)
        # flags of lib.rs:13-33 with their initial values
        self.current_output = SummaryStat.Curl
        self.output_changed = True
        self.click_type = ClickType.Inactive
        self.click_type_changed = True
        self.color_map = ColorMap.Jet
        self.color_changed = False
        self.paused = False
        self.compute_per_render = 15
        self.viscosity = 0.1
        self.viscosity_changed = False
        self.fluid_preset = FluidPreset.Equilibrium
        self.fluid_preset_changed = False
        self.fluid_speed = 0.1
        self.barrier_preset = BarrierPreset.Tunnel
        self.barrier_preset_changed = False
        self.undo_count = 0
        self.undo_changed = False
        self.step_mode = False
        self.step_taken = False
        self.frames = 0

    # ---- WASMInteraction setters ------------------------------------------------
    def set_output(self, stat):
        self.current_output, self.output_changed = stat, True

    def set_draw_type(self, t):
        self.click_type, self.click_type_changed = t, True

    def set_color_map(self, cmap):
        self.color_map, self.color_changed = cmap, True

    def toggle_pause(self):
        self.paused = not self.paused

    def update_compute_rate(self, rate):
        self.compute_per_render = int(rate)

    def update_viscosity(self, nu):
        self.viscosity, self.viscosity_changed = float(nu), True

    def update_flow_speed(self, speed):
        self.fluid_preset_changed = True
        self.fluid_preset = FluidPreset.CustomSpeed
        self.fluid_speed = float(speed)

    def undo(self):
        self.undo_count += 1
        self.undo_changed = True

    def set_step_mode(self):
        self.step_mode = True

    def release_step_mode(self):
        self.step_mode = False

    def take_step(self):
        self.step_taken = True

    def change_fluid_preset(self, f):
        self.fluid_preset_changed, self.fluid_preset = True, f

    def change_barrier_preset(self, b):
        self.barrier_preset_changed, self.barrier_preset = True, b

    # ---- mouse (lib.rs:80-106) ---------------------------------------------------------
    def _mouse_input(self):
        if self.click_type_changed:
            self.click.switch_click_type(self.click_type)
            self.click_type_changed = False

    def press(self, loc):
        self.position = self.click.validate_click(loc)
        self._mouse_input()
        self.pressed = True
        self.click.handle_click(self.position)

    def move(self, loc):
        self.position = self.click.validate_click(loc)
        if self.pressed:
            self.click.handle_movement(self.position)

    def release(self):
        self._mouse_input()
        self.pressed = False
        self.click.handle_release()

    # ---- one redraw (lib.rs:108-204) ---------------------------------------------------
    def _draw(self, shape):
        if not shape.is_empty():
            self.lat.draw_points(points_vector(shape, self.x))

    def redraw(self):
        lat = self.lat
        barrier_redraw = not self.click.current_blob.is_empty() or not self.click.current_curve.is_empty()
        if self.barrier_preset_changed:
            lat.reset_barrier()
            for s in PRESETS[_PRESET_NAMES[self.barrier_preset]](self.x, self.y):
                self._draw(s)
            self.click.clear_barrier()
            barrier_redraw = False
            self.undo_count = 0
            self.undo_changed = False
        if self.undo_changed:
            blob = Blob()
            for _ in range(self.undo_count):
                u = self.click.undo()
                if u is not None:
                    blob.join(u)
            self._draw(blob)
            self.click.empty_all()
            barrier_redraw = False
            self.undo_count = 0
        if self.fluid_preset_changed:
            f = self.fluid_preset
            if f == FluidPreset.Equilibrium:
                lat.reset_to_equilibrium()
            elif f == FluidPreset.CustomSpeed:
                lat.custom_speed(self.fluid_speed)
            else:
                lat.single_cell({FluidPreset.SingleNorth: 1, FluidPreset.SingleOrigin: 4,
                                 FluidPreset.SingleEast: 5, FluidPreset.SingleNorthEast: 2}[f])
        if self.output_changed:
            lat.set_summary(self.current_output)
        if self.color_changed:
            lat.set_color_map(self.color_map)
        if barrier_redraw:
            self.click.current_blob.join(self.click.current_curve)
            self._draw(self.click.current_blob)
            self.click.update(self.pressed, self.position, self.click_type)
        if self.viscosity_changed:
            lat.update_omega_buffer(1.0 / (3.0 * self.viscosity + 0.5))
            self.viscosity_changed = False
        frame = None
        if not self.paused and not self.step_mode:
            lat.iterate(self.compute_per_render)
            frame = lat.render(self.width, self.height)
        elif self.step_mode and self.step_taken:
            lat.iterate(1)
            frame = lat.render(self.width, self.height)
            self.step_taken = False
        elif (self.output_changed or barrier_redraw or self.color_changed or self.fluid_preset_changed
              or self.undo_changed or self.barrier_preset_changed):
            frame = lat.render(self.width, self.height)
        self.undo_changed = self.output_changed = self.color_changed = False
        self.fluid_preset_changed = self.barrier_preset_changed = False
        if frame is not None:
            self.frames += 1
        return frame
