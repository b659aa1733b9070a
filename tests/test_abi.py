"""The C ABI library loads and exports every entry point include/*.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import glob
import os
import re

from conftest import ROOT


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names.update(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(crt_\w+)\s*\(", src, flags=re.M))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("crt_scene_create", "crt_bvh_build", "crt_bvh_refit", "crt_trace_closest", "crt_trace_shadow",
                 "crt_render", "crt_sort_pairs", "crt_morton", "crt_last_error_string"):
        assert must in names


def test_library_exports_every_declared_symbol(built):
    import crt
    lib = crt.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"
    assert b"sm_103a" in lib.crt_version()


def test_library_is_in_tree_and_built_for_sm103a(built):
    import crt.build as b
    assert os.path.exists(b.LIB) and b.LIB.startswith(ROOT)
    assert "arch=compute_103a,code=sm_103a" in " ".join(b.ARCH)
    assert "-fmad=false" in b.FLAGS
