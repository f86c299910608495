"""The C-ABI library loads and exports every function include/psy_gpu.h
declares (no compute calls: runs without a GPU)."""
import os
import re

import pytest

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


def test_ctypes_layout_matches_header(tmp_path):
    """Every ctypes mirror in abi.py has the size and field offsets the C
    compiler gives the header's struct (compiled with gcc, no GPU)."""
    import ctypes as C
    import shutil
    import subprocess
    import pytest
    from psychopath_gb300 import abi
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = [n for n in dir(abi) if n.startswith("Psy") and isinstance(getattr(abi, n), type)
               and issubclass(getattr(abi, n), C.Structure)]
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "psy_gpu.h"', "int main(void) {"]
    for n in structs:
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (n, n))
        for f in getattr(abi, n)._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (n, f[0], n, f[0]))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = dict(l.rsplit(" ", 1) for l in out if l.strip())
    for n in structs:
        T = getattr(abi, n)
        assert int(got[n]) == C.sizeof(T), n
        for f in T._fields_:
            assert int(got["%s.%s" % (n, f[0])]) == getattr(T, f[0]).offset, (n, f[0])


def test_ctypes_constants_match_header():
    """Every integer constant abi.py mirrors has the value the header's
    #define gives it."""
    import re
    from psychopath_gb300 import abi
    text = open(os.path.join(ROOT, "include", "psy_gpu.h")).read()
    defs = {m.group(1): int(m.group(2), 0)
            for m in re.finditer(r"^#define\s+(PSY_\w+)\s+\(?(-?(?:0x[0-9A-Fa-f]+|\d+))[uU]?\)?\s*(?:/\*.*)?$", text, re.M)}
    mirrored = [n for n in dir(abi) if n.startswith("PSY_") and isinstance(getattr(abi, n), int)]
    checked = [n for n in mirrored if n in defs]
    assert len(checked) >= 10
    for n in checked:
        assert getattr(abi, n) == defs[n], n


def _gpu_present():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_gpu_present(), reason="passes placeholder device pointers: run only where no GPU exists")
def test_compact_entry_points_validate_before_any_gpu_work(gpu_lib):
    """Argument errors of the codec calls come back as PSY_E_INVALID (the
    reference panics or cannot express them) before any launch.  Some calls
    pass placeholder pointers that the host-side checks must reject, so the
    test runs only on machines without a GPU."""
    import ctypes as C
    from psychopath_gb300 import abi, gpu
    gpu.lib()  # binds the argument types
    L = gpu_lib
    size = C.c_uint32()
    for fmt, want in ((abi.PSY_COMPACT_FLUV32, 4), (abi.PSY_COMPACT_OCT32_PRECISE, 4),
                      (abi.PSY_COMPACT_UNSIGNED40, 5), (abi.PSY_COMPACT_SIGNED48, 6)):
        assert L.psy_compact_element_size(fmt, C.byref(size)) == abi.PSY_OK and size.value == want
    assert L.psy_compact_element_size(99, C.byref(size)) == abi.PSY_E_INVALID
    assert L.psy_compact_encode(99, None, 4, None, None, None) == abi.PSY_E_INVALID
    assert L.psy_compact_decode(99, None, 4, None, None) == abi.PSY_E_INVALID
    assert L.psy_compact_encode(abi.PSY_COMPACT_FLUV32, None, 0, None, None, None) == abi.PSY_OK  # empty batch
    assert L.psy_compact_encode(abi.PSY_COMPACT_FLUV32, None, 4, None, None, None) == abi.PSY_E_INVALID
    assert L.psy_compact_encode(abi.PSY_COMPACT_FLUV32, 16, 4, 16, 2, None) == abi.PSY_E_INVALID  # counter
    assert L.psy_closure_compress(16, 1, 5, 16, None, None) == abi.PSY_E_INVALID  # stride below 6
    assert L.psy_closure_compress(18, 1, 10, 16, None, None) == abi.PSY_E_INVALID  # misaligned records
    assert L.psy_closure_decompress(16, 1, 10, 18, None, None) == abi.PSY_E_INVALID
    assert L.psy_color_compress(None, 1, None, None, None) == abi.PSY_E_INVALID
    assert b"compact" in L.psy_last_error() or b"closure" in L.psy_last_error() or b"color" in L.psy_last_error()
