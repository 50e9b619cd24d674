"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/*.h declares.  No compute calls (runs without a GPU)."""
import ctypes
import glob
import os
import re

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names.update(re.findall(r"^\s*(?:const\s+)?\w+\s*\**\s*(lbm\w*)\s*\(", src, flags=re.M))
    return names


def test_header_declares_the_surface():
    names = declared_symbols()
    for must in ["lbm_create", "lbm_destroy", "lbm_set_barrier", "lbm_reset_barrier", "lbm_set_omega",
                 "lbm_set_viscosity", "lbm_set_inlet_velocity", "lbm_step", "lbm_read_field", "lbm_step_count",
                 "lbm_last_error"]:
        assert must in names


def test_library_exports_every_declared_symbol(lbm):
    lib = ctypes.CDLL(lbm.LIB_PATH)
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_mirror_binds_every_symbol(lbm):
    bound = {name for name, _, _ in lbm._SIGS}
    assert declared_symbols() <= bound


def test_error_path_without_device(lbm):
    """Argument validation happens before any device work."""
    L = lbm.load_library()
    h = ctypes.c_void_p()
    assert L.lbm_create(2, 2, 1.0, 0, 0, ctypes.byref(h)) == 1
    assert b"must be >= 3" in L.lbm_last_error()
    assert L.lbm_create(16, 16, 1.0, 7, 0, ctypes.byref(h)) == 1
    assert L.lbm_step(None, 1) == 1


def test_limits_and_null_arguments_without_device(lbm):
    """Grids past the size limits, unknown storage, null outputs and null
    handles are refused with LBM_ERR_ARG (1) before any device work; so are
    the rounding entry points without a lattice or without outputs."""
    L = lbm.load_library()
    h = ctypes.c_void_p()
    assert L.lbm_create(1 << 20, 1 << 15, 1.0, 0, 0, ctypes.byref(h)) == 1  # 8 planes past 2^32 cells
    assert b"too large" in L.lbm_last_error()
    assert L.lbm_create(64, 70000, 1.0, 0, 0, ctypes.byref(h)) == 1  # more rows than the limit
    assert L.lbm_create(64, 64, 1.0, 0, 9, ctypes.byref(h)) == 1
    assert b"storage" in L.lbm_last_error()
    assert L.lbm_create(64, 64, 1.0, 0, 0, None) == 1
    mode, seed, origin = ctypes.c_int(), ctypes.c_uint32(), ctypes.c_int32()
    assert L.lbm_set_rounding(None, 1, 5) == 1
    assert L.lbm_get_rounding(None, ctypes.byref(mode), ctypes.byref(seed)) == 1
    assert L.lbm_set_row_origin(None, 3) == 1
    assert L.lbm_get_row_origin(None, ctypes.byref(origin)) == 1
    assert L.lbm_batch_set_rounding(None, 1, 5) == 1
    assert L.lbm_batch_get_rounding(None, ctypes.byref(mode), ctypes.byref(seed)) == 1


def test_library_is_built_for_sm_103a(lbm):
    """ptxas reports every kernel compiled for sm_103a (the build keeps its log)."""
    logs = glob.glob(os.path.join(ROOT, "lbm_gb300", "_build", "*.ptxas.txt"))
    assert logs
    text = "".join(open(f).read() for f in logs)
    targets = set(re.findall(r"for '(sm_\w+)'", text))
    assert targets == {"sm_103a"}, targets
