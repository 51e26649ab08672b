"""The C-ABI library builds, loads and exports every entry point declared in
include/*.h (no GPU needed: nothing is called that touches a device)."""
import ctypes
import glob
import os
import re

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(sq_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("sq_create", "sq_build", "sq_trace", "sq_radix_sort_pairs", "sq_morton_codes",
                 "sq_bvh_export_node1", "sq_bvh_import_node1"):
        assert must in names


def test_library_exports_every_declared_symbol(lib_built):
    lib = ctypes.CDLL(lib_built)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version(lib_built):
    lib = ctypes.CDLL(lib_built)
    lib.sq_abi_version.restype = ctypes.c_uint32
    assert lib.sq_abi_version() == 2


def test_struct_sizes():
    import numpy as np
    import sequoia_gb300 as sq
    assert sq.NODE1.itemsize == 32
    assert sq.HIT.itemsize == 12
    assert ctypes.sizeof(sq._RaySource) == 4 * 3 + 12 * 3 + 4 + 4 + 8 + 4 + 4  # with padding
