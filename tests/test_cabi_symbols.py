"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/*.h declares (no GPU needed: nothing is called)."""
import ctypes
import glob
import os
import re

from mpm_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        syms.update(re.findall(r"\b(mpm_(?:gpu|ns|nn)_\w+)\s*\(", text))
    return syms


def test_library_exports_every_declared_symbol():
    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    syms = declared_symbols()
    assert len(syms) >= 16
    missing = [s for s in sorted(syms) if not hasattr(lib, s)]
    assert not missing, missing


def test_status_strings_without_gpu():
    lib = ctypes.CDLL(build.build())
    lib.mpm_gpu_status_string.restype = ctypes.c_char_p
    assert lib.mpm_gpu_status_string(0) == b"ok"
    assert b"grid" in lib.mpm_gpu_status_string(4)
