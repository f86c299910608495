"""The C-ABI library loads and exports every function include/psy_gpu.h
declares (no compute calls: runs without a GPU)."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for f in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ \*]*?\b(psy_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("psy_scene_create", "psy_scene_destroy", "psy_trace", "psy_render_bucket", "psy_render_image"):
        assert n in names


def test_library_exports_declared_symbols(gpu_lib):
    for n in declared_functions():
        assert hasattr(gpu_lib, n), n


def test_version_and_error_without_gpu_work(gpu_lib):
    assert b"psychopath_gb300" in gpu_lib.psy_version()
    # invalid argument paths return codes, never abort
    import ctypes as C
    from psychopath_gb300 import abi
    h = C.c_void_p()
    assert gpu_lib.psy_scene_create(None, None, C.byref(h)) == abi.PSY_E_INVALID
    assert gpu_lib.psy_scene_destroy(None) == 0
    assert gpu_lib.psy_last_error() != b""


def test_abi_struct_sizes():
    import ctypes as C
    from psychopath_gb300 import abi
    assert C.sizeof(abi.PsyRay) == 40
    assert C.sizeof(abi.PsyHit) == 32
    assert C.sizeof(abi.PsySurfaceHit) == 80
    assert abi.ray_dtype().itemsize == 40
    assert abi.hit_dtype().itemsize == 32
    assert abi.surface_hit_dtype().itemsize == 80
