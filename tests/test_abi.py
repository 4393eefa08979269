"""The C-ABI library builds for sm_103a, loads, and exports every symbol include/*.h declares."""
import ctypes
import glob
import os
import re

from tisphi_gb300 import build_native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(tsg_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("tsg_create", "tsg_upload", "tsg_sort", "tsg_kernel_corr", "tsg_init_tmp", "tsg_one_step",
                 "tsg_advect", "tsg_substep", "tsg_step", "tsg_field", "tsg_reduce_diag", "tsg_last_error",
                 "tsg_destroy", "tsg_neighbors", "tsg_grid"):
        assert must in names


def test_library_exports_all_declared_symbols():
    lib_path = build_native.build()
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_status_strings_without_gpu():
    lib = ctypes.CDLL(build_native.build())
    lib.tsg_status_string.restype = ctypes.c_char_p
    assert lib.tsg_status_string(0) == b"ok"
    assert b"argument" in lib.tsg_status_string(-1)
    # creating with a NULL config is rejected before any CUDA call
    assert lib.tsg_create(None, None) == -1
