"""The C ABI library builds, loads without a GPU, and exports every function
declared in include/pmmoto_gb300.h (no device work is done here)."""

import ctypes
import os
import re

from pmmoto_gb300 import _build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "pmmoto_gb300.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pmg_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared()
    for must in ("pmg_edt3d", "pmg_edt3d_noalloc", "pmg_edt2d", "pmg_morph", "pmg_cc_label", "pmg_cc_select",
                 "pmg_spheres", "pmg_porosimetry", "pmg_drainage", "pmg_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_build.build())
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_last_error_and_version_without_gpu():
    lib = ctypes.CDLL(_build.build())
    lib.pmg_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.pmg_version()
    buf = ctypes.create_string_buffer(64)
    assert lib.pmg_last_error(buf, 64) == 0
