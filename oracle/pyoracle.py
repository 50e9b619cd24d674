"""ctypes wrappers around the CPU oracles.  TEST INFRASTRUCTURE ONLY.

`Oracle` wraps liboracle.so (the C++ restatement, lbm_oracle.cpp) and `RefShaders`
wraps _ref/libref.so (the reference's WGSL translated by wgsl2cpp.py and driven
by ref_host.cpp).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline use them; the product package lbm_gb300 never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")

EDGE_REF, EDGE_CHANNEL = 0, 1
P_F32, P_F16, P_BF16, P_F64 = 0, 1, 2, 3

_c_u8p = ctypes.POINTER(ctypes.c_uint8)
_c_u32p = ctypes.POINTER(ctypes.c_uint32)
_c_f32p = ctypes.POINTER(ctypes.c_float)
_c_f64p = ctypes.POINTER(ctypes.c_double)


# Where the reference tree is read from when its shaders are translated:
# LBM_REFERENCE_ROOT, else the build container's copy.  Without either, an
# earlier translation (_ref/ref_shaders.inc) is compiled as it is.
REFERENCE_ROOT = os.environ.get("LBM_REFERENCE_ROOT") or "/root/reference"


def build(ref=True):
    """Compile liboracle.so and, when possible, the translated reference."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref:
        root = REFERENCE_ROOT if os.path.isdir(REFERENCE_ROOT) else ""
        r = subprocess.run(["make", "-s", "-C", HERE, "ref", "REF_ROOT=" + root], capture_output=True, text=True)
        return r.returncode == 0
    return os.path.exists(REF_SO)


def _ptr(a, t):
    return a.ctypes.data_as(t) if a is not None else None


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        L = ctypes.CDLL(ORACLE_SO)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_set_threads.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_set_omega.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.orc_set_inlet.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.orc_set_storage_reference.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_set_rounding.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32]
        L.orc_set_row_origin.argtypes = [ctypes.c_void_p, ctypes.c_long]
        L.orc_half_rs.restype = ctypes.c_uint16
        L.orc_half_rs.argtypes = [ctypes.c_float, ctypes.c_uint32]
        L.orc_bf16_rs.restype = ctypes.c_uint16
        L.orc_bf16_rs.argtypes = [ctypes.c_float, ctypes.c_uint32]
        L.orc_sr_bits.restype = ctypes.c_uint32
        L.orc_sr_bits.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_long, ctypes.c_long, ctypes.c_int]
        L.orc_init_equilibrium.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_uint64]
        L.orc_init_equilibrium_noise.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                                 ctypes.c_double, ctypes.c_void_p]
        L.orc_single_cell.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_apply_inlet.argtypes = [ctypes.c_void_p]
        L.orc_set_mask.argtypes = [ctypes.c_void_p, _c_u8p]
        L.orc_get_mask.argtypes = [ctypes.c_void_p, _c_u8p]
        L.orc_apply_barrier_pairs.argtypes = [ctypes.c_void_p, _c_u32p, ctypes.c_size_t]
        L.orc_reset_barrier.argtypes = [ctypes.c_void_p]
        L.orc_step.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.orc_step_count.restype = ctypes.c_uint64
        L.orc_step_count.argtypes = [ctypes.c_void_p]
        L.orc_get_state.argtypes = [ctypes.c_void_p, _c_f64p, _c_f64p, _c_f64p, _c_f64p]
        L.orc_get_raw_state.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_put_state.argtypes = [ctypes.c_void_p, _c_f64p]
        L.orc_curl_ref.argtypes = [ctypes.c_void_p, _c_f64p]
        L.orc_force.restype = ctypes.c_int
        L.orc_force.argtypes = [ctypes.c_void_p, _c_f64p]
        L.orc_float_to_half.restype = ctypes.c_uint16
        L.orc_float_to_half.argtypes = [ctypes.c_float]
        L.orc_half_to_float.restype = ctypes.c_float
        L.orc_half_to_float.argtypes = [ctypes.c_uint16]
        L.orc_float_to_bf16.restype = ctypes.c_uint16
        L.orc_float_to_bf16.argtypes = [ctypes.c_float]
        L.orc_recip_newton.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.orc_noise_u01.restype = ctypes.c_double
        L.orc_noise_u01.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int]
        _lib = L
    return _lib


class Oracle:
    """The C++ restatement of the reference step (8 passes, reference order)."""

    def __init__(self, nx, ny, omega, edge=EDGE_REF, prec=P_F32, threads=None):
        self.nx, self.ny, self.n = nx, ny, nx * ny
        self.prec = prec
        self.h = lib().orc_create(nx, ny, omega, edge, prec)
        if not self.h:
            raise ValueError("orc_create failed")
        lib().orc_set_threads(self.h, threads or os.cpu_count() or 1)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def set_threads(self, t):
        lib().orc_set_threads(self.h, t)

    def set_omega(self, w):
        lib().orc_set_omega(self.h, w)

    def set_inlet(self, u, apply=True):
        lib().orc_set_inlet(self.h, u)
        if apply:
            lib().orc_apply_inlet(self.h)

    def set_storage_reference(self, inlet):
        """16-bit words relative to the inlet equilibrium (True) or the rest weights."""
        lib().orc_set_storage_reference(self.h, 1 if inlet else 0)

    def set_rounding(self, mode, seed=0):
        """Rounding of the collided 16-bit words: 0 nearest, 1 stochastic (seeded)."""
        lib().orc_set_rounding(self.h, int(mode), int(seed) & 0xFFFFFFFF)

    def set_row_origin(self, y0):
        """Row y hashes as y + y0 in the stochastic rounding."""
        lib().orc_set_row_origin(self.h, int(y0))

    def init_equilibrium(self, rho=1.0, ux=0.1, uy=0.0, noise=0.0, seed=0):
        lib().orc_init_equilibrium(self.h, rho, ux, uy, noise, seed)

    def init_equilibrium_noise(self, rho, ux, uy, noise):
        """The caller's per-cell velocity noise: float32 (2, ny, nx) (ux, uy), or None."""
        if noise is None:
            lib().orc_init_equilibrium_noise(self.h, rho, ux, uy, None)
            return
        n = np.ascontiguousarray(noise, np.float32)
        lib().orc_init_equilibrium_noise(self.h, rho, ux, uy, n.ctypes.data_as(ctypes.c_void_p))

    def single_cell(self, d):
        lib().orc_single_cell(self.h, d)

    def set_mask(self, mask):
        m = np.ascontiguousarray(mask, dtype=np.uint8).reshape(-1)
        assert m.size == self.n
        lib().orc_set_mask(self.h, _ptr(m, _c_u8p))

    def mask(self):
        m = np.zeros(self.n, np.uint8)
        lib().orc_get_mask(self.h, _ptr(m, _c_u8p))
        return m.reshape(self.ny, self.nx)

    def barrier_pairs(self, pairs):
        p = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1)
        lib().orc_apply_barrier_pairs(self.h, _ptr(p, _c_u32p), p.size // 2)

    def reset_barrier(self):
        lib().orc_reset_barrier(self.h)

    def step(self, n=1):
        lib().orc_step(self.h, n)

    @property
    def step_count(self):
        return lib().orc_step_count(self.h)

    def state(self):
        """(pops[9, ny, nx], rho, jx, jy) as float64 arrays."""
        p = np.zeros(9 * self.n)
        r, jx, jy = np.zeros(self.n), np.zeros(self.n), np.zeros(self.n)
        lib().orc_get_state(self.h, _ptr(p, _c_f64p), _ptr(r, _c_f64p), _ptr(jx, _c_f64p), _ptr(jy, _c_f64p))
        s = (self.ny, self.nx)
        return p.reshape(9, *s), r.reshape(s), jx.reshape(s), jy.reshape(s)

    def raw_state(self):
        """Raw storage words of the current set and the other set, [9, ny, nx] each."""
        dt = {P_F32: np.float32, P_F64: np.float64, P_F16: np.uint16, P_BF16: np.uint16}[self.prec]
        a = np.zeros(9 * self.n, dt)
        b = np.zeros(9 * self.n, dt)
        lib().orc_get_raw_state(self.h, a.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p))
        return a.reshape(9, self.ny, self.nx), b.reshape(9, self.ny, self.nx)

    def put_state(self, pops9):
        p = np.ascontiguousarray(pops9, dtype=np.float64).reshape(-1)
        lib().orc_put_state(self.h, _ptr(p, _c_f64p))

    def curl_ref(self):
        out = np.zeros(self.n)
        lib().orc_curl_ref(self.h, _ptr(out, _c_f64p))
        return out.reshape(self.ny, self.nx)

    def force(self):
        """(drag, lift) by momentum exchange on the last post-collision state."""
        out = np.zeros(2)
        if lib().orc_force(self.h, _ptr(out, _c_f64p)):
            raise RuntimeError("no collision yet")
        return out


_ref = None


def half_rs(v, r13):
    """binary16 bits of float32 `v` rounded stochastically with 13 random bits."""
    return lib().orc_half_rs(float(v), int(r13))


def bf16_rs(v, r16):
    """bfloat16 bits of float32 `v` rounded stochastically with 16 random bits."""
    return lib().orc_bf16_rs(float(v), int(r16))


def sr_bits(seed, t, y, x, q):
    """The 32 random bits of direction q for the column pair of cell (x, y) at step t."""
    return lib().orc_sr_bits(int(seed) & 0xFFFFFFFF, int(t), int(y), int(x), int(q))


def ref_available():
    return os.path.exists(REF_SO)


def ref_lib():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            raise FileNotFoundError(REF_SO)
        L = ctypes.CDLL(REF_SO)
        L.ref_create.restype = ctypes.c_void_p
        L.ref_create.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float]
        L.ref_destroy.argtypes = [ctypes.c_void_p]
        L.ref_set_threads.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.ref_set_omega.argtypes = [ctypes.c_void_p, ctypes.c_float]
        L.ref_put_state.argtypes = [ctypes.c_void_p, _c_f32p]
        L.ref_set_barrier_buffer.argtypes = [ctypes.c_void_p, _c_u32p]
        L.ref_get_barrier_buffer.argtypes = [ctypes.c_void_p, _c_u32p]
        L.ref_draw_points.argtypes = [ctypes.c_void_p, _c_u32p, ctypes.c_uint32]
        L.ref_iterate.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.ref_compute_step.restype = ctypes.c_uint64
        L.ref_compute_step.argtypes = [ctypes.c_void_p]
        L.ref_get_state.argtypes = [ctypes.c_void_p, _c_f32p, _c_f32p, _c_f32p, _c_f32p]
        L.ref_get_sets.argtypes = [ctypes.c_void_p, _c_f32p, _c_f32p]
        L.ref_summary.argtypes = [ctypes.c_void_p, ctypes.c_int, _c_f32p]
        L.ref_color_map.argtypes = [ctypes.c_void_p, ctypes.c_int, _c_f32p]
        _ref = L
    return _ref


class RefShaders:
    """The reference's WGSL step, translated to C++ and run on the CPU (f32)."""

    def __init__(self, nx, ny, omega, threads=None):
        self.nx, self.ny, self.n = nx, ny, nx * ny
        self.h = ref_lib().ref_create(nx, ny, omega)
        ref_lib().ref_set_threads(self.h, threads or os.cpu_count() or 1)

    def __del__(self):
        if getattr(self, "h", None):
            ref_lib().ref_destroy(self.h)
            self.h = None

    def set_threads(self, t):
        ref_lib().ref_set_threads(self.h, t)

    def set_omega(self, w):
        ref_lib().ref_set_omega(self.h, w)

    def put_state(self, pops9):
        p = np.ascontiguousarray(pops9, dtype=np.float32).reshape(-1)
        ref_lib().ref_put_state(self.h, _ptr(p, _c_f32p))

    def set_barrier(self, mask):
        b = np.ascontiguousarray(mask, dtype=np.uint32).reshape(-1)
        ref_lib().ref_set_barrier_buffer(self.h, _ptr(b, _c_u32p))

    def barrier(self):
        b = np.zeros(self.n, np.uint32)
        ref_lib().ref_get_barrier_buffer(self.h, _ptr(b, _c_u32p))
        return b.reshape(self.ny, self.nx)

    def draw_points(self, pairs):
        p = np.ascontiguousarray(pairs, dtype=np.uint32).reshape(-1)
        ref_lib().ref_draw_points(self.h, _ptr(p, _c_u32p), p.size // 2)

    def iterate(self, n):
        ref_lib().ref_iterate(self.h, n)

    @property
    def step_count(self):
        return ref_lib().ref_compute_step(self.h)

    def state(self):
        p = np.zeros(9 * self.n, np.float32)
        r, jx, jy = (np.zeros(self.n, np.float32) for _ in range(3))
        ref_lib().ref_get_state(self.h, _ptr(p, _c_f32p), _ptr(r, _c_f32p), _ptr(jx, _c_f32p), _ptr(jy, _c_f32p))
        s = (self.ny, self.nx)
        return p.reshape(9, *s), r.reshape(s), jx.reshape(s), jy.reshape(s)

    def sets(self):
        a = np.zeros(9 * self.n, np.float32)
        b = np.zeros(9 * self.n, np.float32)
        ref_lib().ref_get_sets(self.h, _ptr(a, _c_f32p), _ptr(b, _c_f32p))
        return a.reshape(9, self.ny, self.nx), b.reshape(9, self.ny, self.nx)

    def summary(self, stat):
        out = np.zeros(self.n, np.float32)
        ref_lib().ref_summary(self.h, stat, _ptr(out, _c_f32p))
        return out.reshape(self.ny, self.nx)

    def color_map(self, cmap):
        """Colours of the current output buffer (after summary()), [ny, nx, 3]."""
        out = np.zeros(3 * self.n, np.float32)
        ref_lib().ref_color_map(self.h, cmap, _ptr(out, _c_f32p))
        return out.reshape(self.ny, self.nx, 3)
