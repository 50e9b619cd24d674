"""GB300 D2Q9 lattice-Boltzmann engine: Python host side over the C ABI.

`Lattice` mirrors the simulation surface of the reference's engine
(lbm-wgpu/src/lbm.rs, `impl LBM`) with the same names and argument meaning:

    reference (lbm.rs)                     here
    LBM::new(driver, omega, x, y)  :726    Lattice(x, y, omega, edge=..., storage=...)
    draw_shape(driver, shape)      :1337   draw_points(pairs) / draw_mask(...)
    reset_barrier(driver)          :1362   reset_barrier()
    update_omega_buffer(driver, w) :1358   update_omega_buffer(w)
    custom_speed(driver, ux)       :1090   custom_speed(ux)
    reset_to_equilibrium(driver)   :1076   reset_to_equilibrium()
    single_cell(driver, index)     :1502   single_cell(index)
    iterate(driver, n)             :1065   iterate(n)  (compute part; returns nothing)
    set_summary(stat) + draw       :1061   summary(stat) -> numpy array; render(w, h) -> frame
    get_compute_num()              :1170   get_compute_num()

Errors raise `LBMError` with the library's message.  The compute path is the
CUDA library liblbm_gb300.so; there is no CPU fallback: importing works
without a GPU, but creating a Lattice needs the library and a CUDA device.
"""
import ctypes
import os

import numpy as np

__all__ = ["Lattice", "LBMError", "load_library", "EDGE_REF", "EDGE_CHANNEL", "F32", "F16", "BF16", "F64",
           "ROUND_NEAREST", "ROUND_STOCHASTIC",
           "SummaryStat", "ColorMap", "FIELD"]

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblbm_gb300.so")

EDGE_REF, EDGE_CHANNEL = 0, 1
F32, F16, BF16, F64 = 0, 1, 2, 3
ROUND_NEAREST, ROUND_STOCHASTIC = 0, 1
FIELD = {"rho": 0, "jx": 1, "jy": 2, "ux": 3, "uy": 4, "curl": 5, "vorticity": 6, "speed": 7}


class SummaryStat:
    """The reference's SummaryStat enum (lbm.rs:10-16): Curl, Ux, Uy, Rho, Speed."""
    Curl, Ux, Uy, Rho, Speed = 0, 1, 2, 3, 4


class ColorMap:
    """The reference's ColorMap enum (lbm.rs:20-24): Inferno, Viridis, Jet."""
    Inferno, Viridis, Jet = 0, 1, 2


class LBMError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("lbm error %d: %s" % (code, msg))
        self.code = code


_lib = None

# (name, restype, argtypes) of every entry point declared in include/*.h
_P = ctypes.c_void_p
_SIGS = [
    ("lbm_last_error", ctypes.c_char_p, []),
    ("lbm_version", ctypes.c_char_p, []),
    ("lbm_create", ctypes.c_int, [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, ctypes.c_int, ctypes.c_int,
                                  ctypes.POINTER(_P)]),
    ("lbm_destroy", ctypes.c_int, [_P]),
    ("lbm_get_info", ctypes.c_int, [_P, _P, _P, _P, _P]),
    ("lbm_set_stream", ctypes.c_int, [_P, _P]),
    ("lbm_get_stream", ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    ("lbm_set_tuning", ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int]),
    ("lbm_set_barrier", ctypes.c_int, [_P, _P, ctypes.c_size_t]),
    ("lbm_reset_barrier", ctypes.c_int, [_P]),
    ("lbm_set_mask", ctypes.c_int, [_P, _P]),
    ("lbm_get_mask", ctypes.c_int, [_P, _P]),
    ("lbm_set_omega", ctypes.c_int, [_P, ctypes.c_float]),
    ("lbm_set_viscosity", ctypes.c_int, [_P, ctypes.c_float]),
    ("lbm_set_inlet_velocity", ctypes.c_int, [_P, ctypes.c_float, ctypes.c_int]),
    ("lbm_set_storage_reference", ctypes.c_int, [_P, ctypes.c_int]),
    ("lbm_init_equilibrium_noise", ctypes.c_int, [_P, ctypes.c_float, ctypes.c_float, ctypes.c_float, _P]),
    ("lbm_get_storage_reference", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
    ("lbm_set_rounding", ctypes.c_int, [_P, ctypes.c_int, ctypes.c_uint32]),
    ("lbm_get_rounding", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_uint32)]),
    ("lbm_set_row_origin", ctypes.c_int, [_P, ctypes.c_int32]),
    ("lbm_get_row_origin", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int32)]),
    ("lbm_reset_to_equilibrium", ctypes.c_int, [_P]),
    ("lbm_init_equilibrium", ctypes.c_int, [_P, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                            ctypes.c_uint64]),
    ("lbm_single_cell", ctypes.c_int, [_P, ctypes.c_int]),
    ("lbm_step", ctypes.c_int, [_P, ctypes.c_uint32]),
    ("lbm_step_rows", ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int]),
    ("lbm_set_graphs", ctypes.c_int, [_P, ctypes.c_int]),
    ("lbm_synchronize", ctypes.c_int, [_P]),
    ("lbm_read_field", ctypes.c_int, [_P, ctypes.c_int, _P]),
    ("lbm_read_field_device", ctypes.c_int, [_P, ctypes.c_int, _P]),
    ("lbm_read_populations", ctypes.c_int, [_P, _P]),
    ("lbm_read_populations_f64", ctypes.c_int, [_P, _P]),
    ("lbm_read_populations_device", ctypes.c_int, [_P, _P]),
    ("lbm_write_populations", ctypes.c_int, [_P, _P]),
    ("lbm_write_populations_f64", ctypes.c_int, [_P, _P]),
    ("lbm_step_count", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint64)]),
    ("lbm_launch_count", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint64)]),
    ("lbm_conservation", ctypes.c_int, [_P, _P]),
    ("lbm_read_force", ctypes.c_int, [_P, _P]),
    ("lbm_conservation_noalloc", ctypes.c_int, [_P, _P, _P, _P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                                _P, _P]),
    ("lbm_rows_read", ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _P, ctypes.c_int]),
    ("lbm_rows_write", ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _P, ctypes.c_int]),
    ("lbm_storage_bytes", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint32)]),
    # include/lbm_render.h
    ("lbm_summary", ctypes.c_int, [_P, ctypes.c_int, _P]),
    ("lbm_render", ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, _P, _P,
                                  ctypes.c_int]),
    ("lbm_render_device", ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, _P]),
    # include/lbm_checkpoint.h
    ("lbm_checkpoint_size", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    ("lbm_checkpoint_save", ctypes.c_int, [_P, _P, ctypes.c_size_t]),
    ("lbm_checkpoint_load", ctypes.c_int, [_P, _P, ctypes.c_size_t]),
    ("lbm_checkpoint_write", ctypes.c_int, [_P, ctypes.c_char_p]),
    ("lbm_checkpoint_read", ctypes.c_int, [_P, ctypes.c_char_p]),
    ("lbm_checkpoint_inspect", ctypes.c_int, [_P, ctypes.c_size_t, _P]),
    # include/lbm_cnn.h
    ("lbm_cnn_conv_forward", ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P,
                                            ctypes.c_int, ctypes.c_int, _P, _P]),
    ("lbm_cnn_conv_backward_data", ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                  _P, ctypes.c_int, _P, _P]),
    ("lbm_cnn_conv_backward_weight", ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                    ctypes.c_int, ctypes.c_int, _P, _P, _P, ctypes.c_size_t, _P]),
    ("lbm_cnn_weight_scratch_bytes", ctypes.c_size_t, [ctypes.c_int, ctypes.c_int]),
    ("lbm_cnn_closure_loss", ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                            _P, _P, _P, _P]),
    ("lbm_cnn_adam", ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                    ctypes.c_float, ctypes.c_float, _P]),
    ("lbm_cnn_closure_sample", ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P, _P,
                                              _P]),
    ("lbm_closure_set_weights", ctypes.c_int, [_P, _P, ctypes.c_size_t]),
    ("lbm_closure_enable", ctypes.c_int, [_P, ctypes.c_float]),
    ("lbm_closure_disable", ctypes.c_int, [_P]),
    ("lbm_closure_infer", ctypes.c_int, [_P]),
    ("lbm_closure_set_inference", ctypes.c_int, [_P, ctypes.c_int]),
    ("lbm_closure_read", ctypes.c_int, [_P, _P, _P]),
    ("lbm_closure_fallback_count", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.c_int]),
    # include/lbm_batch.h
    ("lbm_batch_create", ctypes.c_int, [ctypes.c_uint32, _P, _P, _P, _P, ctypes.c_int, ctypes.POINTER(_P)]),
    ("lbm_batch_destroy", ctypes.c_int, [_P]),
    ("lbm_batch_info", ctypes.c_int, [_P, _P, _P, _P]),
    ("lbm_batch_get_stream", ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    ("lbm_batch_set_mask", ctypes.c_int, [_P, ctypes.c_uint32, _P]),
    ("lbm_batch_init_equilibrium", ctypes.c_int, [_P, ctypes.c_float, ctypes.c_uint64]),
    ("lbm_batch_step", ctypes.c_int, [_P, ctypes.c_uint32]),
    ("lbm_batch_synchronize", ctypes.c_int, [_P]),
    ("lbm_batch_read_field", ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_int, _P]),
    ("lbm_batch_read_populations", ctypes.c_int, [_P, ctypes.c_uint32, _P]),
    ("lbm_batch_conservation", ctypes.c_int, [_P, _P]),
    ("lbm_batch_set_schedule", ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, _P]),
    ("lbm_batch_set_rounding", ctypes.c_int, [_P, ctypes.c_int, ctypes.c_uint32]),
    ("lbm_batch_get_rounding", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_uint32)]),
    ("lbm_batch_autotune", ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_char_p, ctypes.c_size_t]),
]


class CheckpointInfo(ctypes.Structure):
    """lbm_checkpoint_info (include/lbm_checkpoint.h)."""
    _fields_ = [("nx", ctypes.c_uint32), ("ny", ctypes.c_uint32), ("edge", ctypes.c_int), ("storage", ctypes.c_int),
                ("omega", ctypes.c_float), ("u_in", ctypes.c_float), ("drift", ctypes.c_float),
                ("steps", ctypes.c_uint64), ("closure", ctypes.c_int), ("store_inlet", ctypes.c_int),
                ("rounding", ctypes.c_int), ("rounding_seed", ctypes.c_uint32), ("row_origin", ctypes.c_int32)]


def checkpoint_info(buf):
    """Check a checkpoint (bytes) on the host, as loading it would, and return
    its header fields as a dict; raises LBMError if any check fails.  Needs
    no GPU and no lattice."""
    load_library()
    b = np.frombuffer(buf, np.uint8)
    info = CheckpointInfo()
    _check(_lib.lbm_checkpoint_inspect(ctypes.c_void_p(b.ctypes.data), b.size, ctypes.byref(info)))
    return {name: getattr(info, name) for name, _ in CheckpointInfo._fields_}


def load_library(path=None):
    """Load liblbm_gb300.so (built by lbm_gb300/build.py) and declare its ABI."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError("%s is missing: build it with `python lbm_gb300/build.py` "
                                "(or __graft_entry__.build())" % p)
    L = ctypes.CDLL(p)
    for name, res, args in _SIGS:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise LBMError(rc, _lib.lbm_last_error().decode())


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


class Lattice:
    """One nx x ny D2Q9 lattice on the current CUDA device."""

    def __init__(self, x, y, omega=1.0 / (0.5 + 0.3), edge=EDGE_REF, storage=F32):
        L = load_library()
        h = ctypes.c_void_p()
        _check(L.lbm_create(int(x), int(y), float(omega), int(edge), int(storage), ctypes.byref(h)))
        self._h = h
        self.x, self.y, self.edge, self.storage = int(x), int(y), int(edge), int(storage)
        self.summary_stat = SummaryStat.Curl

    # -- lifetime ---------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            _lib.lbm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    # -- barrier ------------------------------------------------------------
    def draw_points(self, pairs):
        """draw_barrier_updates: (location, value) u32 pairs, value 1 = solid."""
        p = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1)
        if p.size % 2:
            raise ValueError("pairs must have an even number of entries")
        _check(_lib.lbm_set_barrier(self._h, _ptr(p), p.size // 2))

    def draw_shape(self, shape):
        """draw_shape (lbm.rs:1337-1339): upload a shape's (index, value) pairs."""
        from .shapes import points_vector
        if not shape.is_empty():
            self.draw_points(points_vector(shape, self.x))

    def draw_mask(self, mask):
        """Upload a whole [y, x] mask (nonzero = solid)."""
        m = np.ascontiguousarray(mask, dtype=np.uint8).reshape(-1)
        if m.size != self.x * self.y:
            raise ValueError("mask has %d cells, lattice %d" % (m.size, self.x * self.y))
        _check(_lib.lbm_set_mask(self._h, _ptr(m)))

    def mask(self):
        m = np.zeros(self.x * self.y, np.uint8)
        _check(_lib.lbm_get_mask(self._h, _ptr(m)))
        return m.reshape(self.y, self.x)

    def reset_barrier(self):
        _check(_lib.lbm_reset_barrier(self._h))

    # -- parameters -------------------------------------------------------
    def update_omega_buffer(self, omega):
        _check(_lib.lbm_set_omega(self._h, float(omega)))

    def update_viscosity(self, nu):
        _check(_lib.lbm_set_viscosity(self._h, float(nu)))

    def custom_speed(self, ux):
        _check(_lib.lbm_set_inlet_velocity(self._h, float(ux), 1))

    def set_inlet_velocity(self, ux, reset_field=False):
        _check(_lib.lbm_set_inlet_velocity(self._h, float(ux), 1 if reset_field else 0))

    def set_storage_reference(self, inlet):
        """16-bit storage: keep the words relative to the rest weights (False,
        the default: f - w) or to the inlet equilibrium (True: smaller words,
        and several times less rounding error, in a flow near the inlet
        velocity; a few per cent slower).  The stored state is re-expressed;
        f32 / f64 storage is unaffected."""
        _check(_lib.lbm_set_storage_reference(self._h, 1 if inlet else 0))

    @property
    def storage_reference(self):
        v = ctypes.c_int()
        _check(_lib.lbm_get_storage_reference(self._h, ctypes.byref(v)))
        return bool(v.value)

    def set_rounding(self, mode, seed=0):
        """Rounding of the words each step stores: ROUND_NEAREST (the
        default) or ROUND_STOCHASTIC (16-bit storage only: each word rounds
        up or down with probabilities set by its distance to the two
        neighbouring 16-bit values, from a seeded hash of step, cell and
        direction; rounding then adds no bias that a steady flow would
        accumulate)."""
        _check(_lib.lbm_set_rounding(self._h, int(mode), int(seed) & 0xFFFFFFFF))

    @property
    def rounding(self):
        """(mode, seed)."""
        m, sd = ctypes.c_int(), ctypes.c_uint32()
        _check(_lib.lbm_get_rounding(self._h, ctypes.byref(m), ctypes.byref(sd)))
        return m.value, sd.value

    def set_row_origin(self, y0):
        """Row y of this lattice hashes as y + y0 in the stochastic rounding
        (a slab of a larger lattice sets its first row's index)."""
        _check(_lib.lbm_set_row_origin(self._h, int(y0)))

    @property
    def row_origin(self):
        v = ctypes.c_int32()
        _check(_lib.lbm_get_row_origin(self._h, ctypes.byref(v)))
        return v.value

    def reset_to_equilibrium(self):
        _check(_lib.lbm_reset_to_equilibrium(self._h))

    def init_equilibrium(self, rho=1.0, ux=0.1, uy=0.0, noise=0.0, seed=0):
        _check(_lib.lbm_init_equilibrium(self._h, rho, ux, uy, noise, seed))

    def init_equilibrium_noise(self, rho, ux, uy, noise):
        """set_equil per cell at (rho, ux + noise[0], uy + noise[1]) with the
        caller's float32 noise of shape (2, ny, nx); None for no noise."""
        if noise is None:
            _check(_lib.lbm_init_equilibrium_noise(self._h, rho, ux, uy, None))
            return
        n = np.ascontiguousarray(noise, np.float32)
        if n.shape != (2, self.y, self.x):
            raise ValueError("noise must have shape (2, %d, %d)" % (self.y, self.x))
        _check(_lib.lbm_init_equilibrium_noise(self._h, rho, ux, uy, _ptr(n)))

    def single_cell(self, index):
        _check(_lib.lbm_single_cell(self._h, int(index)))

    def set_tuning(self, rows_per_thread=8, kernel=1):
        _check(_lib.lbm_set_tuning(self._h, int(rows_per_thread), int(kernel)))

    def set_stream(self, stream_ptr):
        """Queue work on a cudaStream_t given as an integer (0 = the legacy default stream)."""
        _check(_lib.lbm_set_stream(self._h, ctypes.c_void_p(stream_ptr) if stream_ptr else None))

    def get_stream(self):
        v = ctypes.c_void_p()
        _check(_lib.lbm_get_stream(self._h, ctypes.byref(v)))
        return v.value or 0

    # -- stepping -----------------------------------------------------------
    def iterate(self, n):
        _check(_lib.lbm_step(self._h, int(n)))

    def step_rows(self, y0, y1, complete=False, moments=False):
        """Rows [y0, y1) of the next step (lbm_step_rows); `complete` ends the step."""
        _check(_lib.lbm_step_rows(self._h, int(y0), int(y1), (1 if complete else 0) | (2 if moments else 0)))

    def synchronize(self):
        _check(_lib.lbm_synchronize(self._h))

    def get_compute_num(self):
        v = ctypes.c_uint64()
        _check(_lib.lbm_step_count(self._h, ctypes.byref(v)))
        return v.value

    def launch_count(self):
        v = ctypes.c_uint64()
        _check(_lib.lbm_launch_count(self._h, ctypes.byref(v)))
        return v.value

    # -- readback -----------------------------------------------------------
    def field(self, name):
        code = FIELD[name] if isinstance(name, str) else int(name)
        out = np.zeros(self.x * self.y, np.float32)
        _check(_lib.lbm_read_field(self._h, code, _ptr(out)))
        return out.reshape(self.y, self.x)

    def set_summary(self, stat):
        self.summary_stat = stat

    def summary(self, stat=None):
        """The reference's summary output for a SummaryStat (summary_stats/*.wgsl):
        curl, raw momenta for Ux / Uy, the display-scaled rho and speed."""
        stat = self.summary_stat if stat is None else stat
        out = np.zeros(self.x * self.y, np.float32)
        _check(_lib.lbm_summary(self._h, int(stat), _ptr(out)))
        return out.reshape(self.y, self.x)

    def set_color_map(self, cmap):
        self.color_map = cmap

    def render(self, width=None, height=None, stat=None, cmap=None, rgba=False, srgb=False):
        """Headless frame of the current state (lbm_render): [height, width, 3]
        float32 RGB, or [height, width, 4] uint8 with rgba=True."""
        stat = self.summary_stat if stat is None else stat
        cmap = getattr(self, "color_map", ColorMap.Jet) if cmap is None else cmap
        w = self.x if width is None else int(width)
        h = self.y if height is None else int(height)
        if rgba:
            out = np.zeros(w * h * 4, np.uint8)
            _check(_lib.lbm_render(self._h, int(stat), int(cmap), w, h, None, _ptr(out), 1 if srgb else 0))
            return out.reshape(h, w, 4)
        out = np.zeros(w * h * 3, np.float32)
        _check(_lib.lbm_render(self._h, int(stat), int(cmap), w, h, _ptr(out), None, 0))
        return out.reshape(h, w, 3)

    def populations(self, f64=False):
        out = np.zeros(9 * self.x * self.y, np.float64 if f64 else np.float32)
        fn = _lib.lbm_read_populations_f64 if f64 else _lib.lbm_read_populations
        _check(fn(self._h, _ptr(out)))
        return out.reshape(9, self.y, self.x)

    def write_populations(self, pops):
        a = np.asarray(pops)
        if a.dtype == np.float64:
            a = np.ascontiguousarray(a).reshape(-1)
            fn = _lib.lbm_write_populations_f64
        else:
            a = np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
            fn = _lib.lbm_write_populations
        if a.size != 9 * self.x * self.y:
            raise ValueError("need 9*x*y values")
        _check(fn(self._h, _ptr(a)))

    def conservation(self):
        """FP64 (sum rho, sum jx, sum jy) over fluid cells."""
        out = np.zeros(3, np.float64)
        _check(_lib.lbm_conservation(self._h, _ptr(out)))
        return out

    # -- halo rows (y-slab decomposition) ------------------------------------------
    @property
    def storage_dtype(self):
        return {F32: np.float32, F16: np.uint16, BF16: np.uint16, F64: np.float64}[self.storage]

    def read_rows(self, y, nrows, slots):
        """Rows y .. y+nrows-1 of the given moving-population slots of the state
        the next step pulls from, as storage words [len(slots), nrows, x]."""
        mask = sum(1 << s for s in slots)
        out = np.zeros((len(slots), nrows, self.x), self.storage_dtype)
        _check(_lib.lbm_rows_read(self._h, int(y), int(nrows), mask, _ptr(out), 0))
        return out

    def read_rows_device(self, y, nrows, slots, ptr):
        """The same rows into device memory at `ptr` (an integer address),
        queued on the lattice's stream."""
        _check(_lib.lbm_rows_read(self._h, int(y), int(nrows), sum(1 << s for s in slots), ctypes.c_void_p(ptr), 1))

    def write_rows_device(self, y, nrows, slots, ptr):
        """Rows from device memory at `ptr`, queued on the lattice's stream."""
        _check(_lib.lbm_rows_write(self._h, int(y), int(nrows), sum(1 << s for s in slots), ctypes.c_void_p(ptr), 1))

    def write_rows(self, y, slots, words):
        mask = sum(1 << s for s in slots)
        a = np.ascontiguousarray(words, dtype=self.storage_dtype)
        if list(slots) != sorted(slots) or a.shape[0] != len(slots) or a.shape[2] != self.x:
            raise ValueError("rows must be [len(slots) ascending, nrows, x]")
        _check(_lib.lbm_rows_write(self._h, int(y), a.shape[1], mask, _ptr(a), 0))

    # -- checkpoint / resume ------------------------------------------------------
    def checkpoint(self):
        """The exact device state as bytes (include/lbm_checkpoint.h layout)."""
        n = ctypes.c_size_t()
        _check(_lib.lbm_checkpoint_size(self._h, ctypes.byref(n)))
        buf = np.zeros(n.value, np.uint8)
        _check(_lib.lbm_checkpoint_save(self._h, _ptr(buf), n.value))
        return buf.tobytes()

    def restore(self, data):
        buf = np.frombuffer(data, np.uint8)
        _check(_lib.lbm_checkpoint_load(self._h, ctypes.c_void_p(buf.ctypes.data), buf.size))

    def save(self, path):
        _check(_lib.lbm_checkpoint_write(self._h, os.fsencode(path)))

    def load(self, path):
        _check(_lib.lbm_checkpoint_read(self._h, os.fsencode(path)))

    def force(self):
        """(drag, lift) on the solid cells by momentum exchange, f64."""
        out = np.zeros(2, np.float64)
        _check(_lib.lbm_read_force(self._h, _ptr(out)))
        return out
