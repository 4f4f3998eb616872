"""The C-ABI library loads and exports every function include/*.h declares
(no compute calls: runs without a GPU)."""
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for hdr in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(hdr).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(lbm_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_entry_points():
    names = declared_functions()
    for required in ("lbm_create", "lbm_init", "lbm_step", "lbm_get_macro", "lbm_destroy",
                     "lbm_macro_norms", "lbm_status", "lbm_build_flags"):
        assert required in names


def test_library_exports_every_declared_symbol(native_lib):
    missing = [n for n in declared_functions() if not hasattr(native_lib, n)]
    assert not missing, missing
    assert native_lib.lbm_version() >= 1
