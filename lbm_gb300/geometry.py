"""Seeded barrier geometry for the benchmark workloads.

The reference draws barriers from mouse strokes as thick Bresenham lines
(lbm-wgpu/src/barrier_shapes/line.rs); the workloads here use solid circles
and rectangles instead, rasterised with a cell-centre-inside rule: cell (x, y)
(integer coordinates) is solid when (x - cx)^2 + (y - cy)^2 <= r^2, or when it
lies in [x0, x1) x [y0, y1) for a rectangle.  Randomness comes from a
splitmix64 stream, so layouts are identical on every machine.
"""
import numpy as np

MASK64 = (1 << 64) - 1


class SplitMix64:
    """splitmix64 generator (Steele, Lea, Flood 2014): state += golden gamma, then mix."""

    def __init__(self, seed):
        self.state = seed & MASK64

    def next_u64(self):
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0):
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / 9007199254740992.0))

    def randint(self, lo, hi):
        """Integer in [lo, hi]."""
        return lo + int(self.uniform() * (hi - lo + 1)) if hi > lo else lo


def disk(mask, cx, cy, r, value=1):
    """Rasterise one solid circle into mask[y, x] in place."""
    ny, nx = mask.shape
    x0, x1 = max(int(np.floor(cx - r)), 0), min(int(np.ceil(cx + r)), nx - 1)
    y0, y1 = max(int(np.floor(cy - r)), 0), min(int(np.ceil(cy + r)), ny - 1)
    if x1 < x0 or y1 < y0:
        return mask
    yy, xx = np.mgrid[y0:y1 + 1, x0:x1 + 1]
    inside = (xx - cx) ** 2 + (yy - cy) ** 2 <= r * r
    sub = mask[y0:y1 + 1, x0:x1 + 1]
    sub[inside] = value
    return mask


def rect(mask, x0, y0, x1, y1, value=1):
    ny, nx = mask.shape
    mask[max(y0, 0):min(y1, ny), max(x0, 0):min(x1, nx)] = value
    return mask


def single_circle(nx, ny, cx, cy, r):
    """One circle (the 256 x 128 workload: r = 12 at (64, 64))."""
    return disk(np.zeros((ny, nx), np.uint8), cx, cy, r)


def random_circles(nx, ny, count, rmin, rmax, seed, inlet_clearance=64, target_fraction=None,
                   outlet_clearance=None):
    """`count` seeded circles with radii uniform in [rmin, rmax] and centres
    uniform over the grid, none within `inlet_clearance` cells of the inlet
    (centre x - r >= clearance).  With `outlet_clearance` none comes within
    that many cells of the outflow column either (centre x + r <= nx - 1 -
    clearance); without it circles may reach the outflow edge.  If
    target_fraction is given, drawing stops once that solid fraction is
    reached."""
    rng = SplitMix64(seed)
    m = np.zeros((ny, nx), np.uint8)
    placed = 0
    solid = 0  # running count of solid cells (only the disk's bounding box changes)
    while placed < count:
        r = rng.uniform(rmin, rmax)
        hi = nx - 1 if outlet_clearance is None else nx - 1 - outlet_clearance - r
        cx = rng.uniform(inlet_clearance + r, hi)
        cy = rng.uniform(0, ny - 1)
        y0, y1 = max(int(np.floor(cy - r)), 0), min(int(np.ceil(cy + r)), ny - 1) + 1
        x0, x1 = max(int(np.floor(cx - r)), 0), min(int(np.ceil(cx + r)), nx - 1) + 1
        before = int(m[y0:y1, x0:x1].sum())
        disk(m, cx, cy, r)
        solid += int(m[y0:y1, x0:x1].sum()) - before
        placed += 1
        if target_fraction is not None and solid >= target_fraction * m.size:
            break
    return m


def random_layout(nx, ny, fraction, seed, rmin=2.0, rmax=None, rect_share=0.5, inlet_clearance=None,
                  outlet_clearance=0):
    """Circles and rectangles until the solid fraction reaches `fraction`;
    no solid within `inlet_clearance` columns of the inlet or
    `outlet_clearance` columns of the outflow edge."""
    rng = SplitMix64(seed)
    m = np.zeros((ny, nx), np.uint8)
    rmax = rmax or max(rmin + 1.0, min(nx, ny) / 8.0)
    clear = inlet_clearance if inlet_clearance is not None else max(4, nx // 8)
    xend = nx - 2 - outlet_clearance  # last column a shape may cover
    guard = 0
    while m.mean() < fraction and guard < 100000:
        guard += 1
        if rng.uniform() < rect_share:
            w = rng.randint(2, max(2, int(2 * rmax)))
            h = rng.randint(2, max(2, int(2 * rmax)))
            x0 = rng.randint(clear, max(clear, xend - w))
            y0 = rng.randint(1, max(1, ny - 1 - h))
            rect(m, x0, y0, min(x0 + w, xend + 1), y0 + h)
        else:
            r = rng.uniform(rmin, rmax)
            cx = rng.uniform(clear + r, max(clear + r, xend - r))
            cy = rng.uniform(0, ny - 1)
            disk(m, cx, cy, r)
    if outlet_clearance:
        m[:, max(xend + 1, 0):] = 0
    return m
