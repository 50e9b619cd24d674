"""Barrier shapes and presets of the reference, restated on the host.

The reference builds barriers on the host as sets of (x, y, solid) points and
uploads them as (index, value) u32 pairs (barrier_shapes/*.rs,
merge_shapes.rs:13-21; lbm.rs:1337-1356); the engine takes the same pairs
through `Lattice.draw_points` / lbm_set_barrier.

* `bresenham` restates the line iteration of the line_drawing crate 1.0.0
  (Cargo.lock pins it; it is not vendored): the line is mapped into the first
  octant by reflections and an x / y swap, walked from the start point with
  an error term initialised to dy - dx that steps y whenever it is >= 0, and
  mapped back.  Its exact pixels on ties are not pinned by any reference
  test or fixture.
* `Line` is line.rs:23-58 (three parallel Bresenham lines, diagonal steps
  filled) and line.rs:60-95 (the erasing variant, 2 x 29 parallel lines);
  `Curve`, `Blob`, `CurveCollection`, `merge` and `points_vector` follow
  curve.rs, blob.rs, curve_collection.rs and merge_shapes.rs.
* `curl_barrier`, `chaos_barrier` and `welcome_barrier` are the presets of
  lbm.rs:1367-1480, with Rust's integer semantics (u32 division of the grid
  size, isize division truncating toward zero).

Sets of points are Python sets; the reference's HashSet order (which decides
the upload order of the pairs) is unspecified, and so is the order here.
"""


def _tdiv(a, b):
    """Integer division truncating toward zero (Rust / C semantics)."""
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b >= 0) else -q


def bresenham(start, end):
    """Cells of the line from start to end, both included, in walking order."""
    x0, y0 = start
    dx, dy = end[0] - x0, end[1] - y0
    sx = 1 if dx >= 0 else -1
    sy = 1 if dy >= 0 else -1
    ax, ay = abs(dx), abs(dy)
    steep = ay > ax
    if steep:
        ax, ay = ay, ax
    err = ay - ax
    pts = []
    u = v = 0
    while u <= ax:
        pts.append((x0 + sx * v, y0 + sy * u) if steep else (x0 + sx * u, y0 + sy * v))
        if err >= 0:
            v += 1
            err -= ax
        u += 1
        err += ay
    return pts


def _valid(p, q, xdim, ydim):
    return all(0 <= a < xdim for a in (p[0], q[0])) and all(0 <= b < ydim for b in (p[1], q[1]))


def _order(p1, p2):
    return (p1, p2) if p1[0] > p2[0] else (p2, p1)


class Shape:
    def __init__(self, points=None):
        self.points = set(points or ())

    def is_empty(self):
        return not self.points

    def negate(self):
        return Blob({(x, y, not v) for x, y, v in self.points})


class Line(Shape):
    """Thick line between two in-grid end points; raises ValueError for end
    points outside the grid (the reference returns an error)."""

    def __init__(self, p1, p2, xdim, ydim, erased=False):
        super().__init__()
        if not _valid(p1, p2, xdim, ydim):
            raise ValueError("Endpoints (%d,%d) (%d,%d) are invalid with dimensions %d and %d"
                             % (p1[0], p1[1], p2[0], p2[1], xdim, ydim))
        value = not erased
        for a, b in (self._endpoints_variable(p1, p2, 30) if erased else self._endpoints(p1, p2)):
            if not _valid(a, b, xdim, ydim):
                continue
            prev = a
            for i in bresenham(a, b):
                self.points.add((i[0], i[1], value))
                if prev[0] != i[0] and prev[1] != i[1]:  # diagonal step: fill both corners
                    d = (i[0] - prev[0], i[1] - prev[1])
                    self.points.add((i[0] - d[0], i[1], value))
                    self.points.add((i[0], i[1] - d[1], value))
                prev = i

    @staticmethod
    def _endpoints(p1, p2):
        a, b = _order(p1, p2)
        if a[1] > b[1]:
            left = ((a[0], a[1] - 1), (a[0] + 1, a[1]))
        else:
            left = ((a[0], a[1] + 1), (a[0] + 1, a[1]))
        right = ((b[0] - 1, b[1]), (b[0], b[1] - 1))
        return [(a, b), (left[0], right[0]), (left[1], right[1])]

    @staticmethod
    def _endpoints_variable(p1, p2, thickness):
        a, b = _order(p1, p2)
        out = [(a, b)]
        for i in range(1, thickness):
            if a[1] > b[1]:
                left = ((a[0], a[1] - i), (a[0] + i, a[1]))
            else:
                left = ((a[0], a[1] + i), (a[0] + i, a[1]))
            right = ((b[0] - i, b[1]), (b[0], b[1] - i))
            out.append((left[0], right[0]))
            out.append((left[1], right[1]))
        return out


class Blob(Shape):
    def add(self, points, xdim, ydim):
        for x, y, v in points:
            if (x & 0xFFFFFFFF) < xdim and (y & 0xFFFFFFFF) < ydim:
                self.points.discard((x, y, not v))
                self.points.add((x, y, v))

    def join(self, shape):
        for x, y, v in list(shape.points):
            self.points.discard((x, y, not v))
            self.points.add((x, y, v))

    def empty(self):
        self.points.clear()


class Curve(Shape):
    def __init__(self):
        super().__init__()
        self.last_point = None

    def add_segment(self, nxt, xdim, ydim, erased=False):
        if self.last_point is not None:
            self.points |= Line(self.last_point, nxt, xdim, ydim, erased=erased).points
        else:
            self.points.add((nxt[0], nxt[1], not erased))
        self.last_point = nxt

    def erase_segment(self, nxt, xdim, ydim):
        self.add_segment(nxt, xdim, ydim, erased=True)

    def empty(self):
        self.points.clear()
        self.last_point = None


class CurveCollection(Shape):
    def __init__(self):
        super().__init__()
        self.last_point = None

    def add_curve(self, curve):
        self.last_point = curve.last_point
        self.points |= curve.points


def merge(s1, s2):
    b = Blob()
    b.join(s1)
    b.join(s2)
    return b


def points_vector(shape, xdim):
    """(index, value) pairs as the reference uploads them: index = x + y * xdim
    in u32 arithmetic, value 1 for solid."""
    out = []
    for x, y, v in shape.points:
        out += [((x & 0xFFFFFFFF) + (y & 0xFFFFFFFF) * xdim) & 0xFFFFFFFF, 1 if v else 0]
    return out


# ---- presets (lbm.rs:1367-1480); each returns the shapes in drawing order ----------

def curl_barrier(x, y):
    return [Line((4 * x // 10, y // 4), (4 * x // 10, y // 2), x, y)]


def chaos_barrier(x, y):
    return [Line((x // 2, 9 * y // 20), (x // 2, 0), x, y),
            Line((x // 2, 11 * y // 20), (x // 2, y - 1), x, y),
            Line((3 * x // 5, y // 2), (3 * x // 4, 3 * y // 4), x, y),
            Line((3 * x // 5, y // 2), (3 * x // 4, y // 4), x, y)]


def welcome_barrier(x, y):
    def line(p1, p2):
        return Line(p1, p2, x, y)

    blob = Blob()
    height = -(y // 4)
    bottom = y // 2
    space = x // 50
    cx = x // 5
    lw = x // 13
    h2, h4 = _tdiv(height, 2), _tdiv(height, 4)
    # W
    parts = [line((cx, bottom + height), (cx, bottom)),
             line((cx, bottom), (cx + lw // 2, bottom + h2))]
    cx += lw // 2
    parts.append(line((cx, bottom + h2), (cx + lw // 2, bottom)))
    cx += lw // 2
    parts.append(line((cx, bottom + height), (cx, bottom)))
    cx += space

    def letter_e(cx):
        return [line((cx, bottom + h2), (cx, bottom)), line((cx, bottom), (cx + lw, bottom)),
                line((cx, bottom + h4), (cx + lw, bottom + h4)),
                line((cx + lw, bottom + h2), (cx + lw, bottom + h4)),
                line((cx, bottom + h2), (cx + lw, bottom + h2))]

    parts += letter_e(cx)  # e
    cx += lw + space
    parts.append(line((cx, bottom), (cx, bottom + height)))  # l
    cx += space
    parts += [line((cx, bottom + h2), (cx, bottom)), line((cx, bottom), (cx + lw, bottom)),
              line((cx, bottom + h2), (cx + lw, bottom + h2))]  # c
    cx += lw + space
    parts += [line((cx, bottom + h2), (cx, bottom)), line((cx, bottom), (cx + lw, bottom)),
              line((cx, bottom + h2), (cx + lw, bottom + h2)),
              line((cx + lw, bottom + h2), (cx + lw, bottom))]  # o
    cx += lw + space
    parts += [line((cx, bottom + h2), (cx, bottom)), line((cx, bottom + h2), (cx + lw, bottom + h2)),
              line((cx + lw, bottom + h2), (cx + lw, bottom)),
              line((cx + lw // 2, bottom), (cx + lw // 2, bottom + h2))]  # m
    cx += lw + space
    parts += letter_e(cx)  # e
    cx += lw + space
    parts += [line((cx, _tdiv(height, 10) + bottom), (cx, bottom)),
              line((cx, _tdiv(height, 5) + bottom), (cx, bottom + height))]  # !
    for p in parts:
        blob.join(p)
    return [blob]


PRESETS = {"Welcome": welcome_barrier, "Tunnel": lambda x, y: [], "Curl": curl_barrier, "Chaos": chaos_barrier}
