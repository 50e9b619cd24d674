"""A small float64 numpy channel lattice with the engine's step semantics,
used by the CPU tests of the y-slab decomposition (test infrastructure).

State P: the populations the next step pulls from.  A step replaces P by
C(pull(P)) for fluid cells off the inlet column (pull: upstream cell
(x - cx, y - cy) with x clamped to the grid and y periodic; a solid upstream
cell bounces the cell's own opposite population back), or by C(P) right
after a state upload.  Inlet column and solids keep their populations."""
import numpy as np

CX = np.array([q % 3 - 1 for q in range(9)])
CY = np.array([q // 3 - 1 for q in range(9)])
W9 = np.array([1 / 36, 1 / 9, 1 / 36, 1 / 9, 4 / 9, 1 / 9, 1 / 36, 1 / 9, 1 / 36])
SLOTS = [0, 1, 2, 3, 5, 6, 7, 8]  # slot -> direction


class NumpyLattice:
    storage_dtype = np.float64

    def __init__(self, x, y, omega):
        self.x, self.y, self.omega = x, y, omega
        self.P = np.zeros((9, y, x))
        self.mask = np.zeros((y, x), np.uint8)
        self.materialised = True

    def draw_mask(self, m):
        self.mask = np.asarray(m, np.uint8).copy()

    def write_populations(self, p):
        self.P = np.array(p, np.float64)
        self.materialised = True

    def populations(self, f64=True):
        return self.P.copy()

    def field(self, name):
        rho = self.P.sum(0)
        return {"rho": rho, "jx": np.tensordot(CX, self.P, 1)}[name]

    def _rows_target(self):
        return self.pending if getattr(self, "pending", None) is not None else self.P

    def read_rows(self, y, n, slots):
        return np.stack([self._rows_target()[SLOTS[s], y:y + n] for s in slots])

    def write_rows(self, y, slots, words):
        for k, s in enumerate(slots):
            self._rows_target()[SLOTS[s], y:y + words.shape[1]] = words[k]

    def iterate(self, n):
        for _ in range(n):
            self._step()

    def step_rows(self, y0, y1, complete=False, moments=False):
        """Rows [y0, y1) of the next step into a pending state that reads and
        writes of rows address until `complete` (the engine's lbm_step_rows);
        rows no call covers keep the previous values."""
        if getattr(self, "pending", None) is None:
            self.pending = self.P.copy()
            self.pending_mat = self.materialised
        keep, mat = self.P, self.materialised
        self.materialised = self.pending_mat
        self._step()
        self.pending[:, y0:y1] = self.P[:, y0:y1]
        self.P, self.materialised = keep, mat
        if complete:
            self.P, self.pending = self.pending, None
            self.materialised = False

    def _step(self):
        P, m = self.P, self.mask.astype(bool)
        Y, X = m.shape
        if self.materialised:
            f = P.copy()
            self.materialised = False
        else:
            f = np.empty_like(P)
            yy, xx = np.mgrid[0:Y, 0:X]
            for q in range(9):
                ux = np.clip(xx - CX[q], 0, X - 1)
                uy = (yy - CY[q]) % Y
                pulled = P[q][uy, ux]
                f[q] = np.where(m[uy, ux], P[8 - q], pulled)
        rho = f.sum(0)
        ux = np.tensordot(CX, f, 1) / rho
        uy = -np.tensordot(CY, f, 1) / rho
        usq = ux * ux + uy * uy
        out = f.copy()
        for q in range(9):
            cu = CX[q] * ux - CY[q] * uy
            feq = W9[q] * rho * (1 + 3 * cu + 4.5 * cu * cu - 1.5 * usq)
            out[q] = f[q] + self.omega * (feq - f[q])
        frozen = m.copy()
        frozen[:, 0] = True
        self.P = np.where(frozen[None], P, out)
