"""Oracle (test infrastructure only): a CPU restatement of Psychopath's
tracing path, used by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline as the checker.  The product package never imports this.

Two builds of the same sources: libpsy_oracle.so computes in f32 as the
reference does; libpsy_oracle64.so (-DPSYO_F64) is the FP64 oracle, the same
algorithm with every f32 operation done in f64 (same samples, same
constants, same scene data), used to state each form's rounding error."""
import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libpsy_oracle.so")
LIB64_PATH = os.path.join(BUILD_DIR, "libpsy_oracle64.so")
SOURCES = ["psy_oracle.cpp", "oracle_sobol.cpp", "oracle_halton.cpp", "oracle_compact.cpp"]
HEADERS = ["psy_oracle.h", "oracle_math.h", "oracle_shading.h"]


def build(force=False):
    """Compile both oracle builds with g++ (strict IEEE: no contraction, no
    fast-math), in parallel."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, h) for h in HEADERS] + [
        os.path.join(HERE, "..", "include", "psy_gpu.h"),
        os.path.join(HERE, "..", "psychopath_gb300", "csrc", "spectra_tables.inc")]
    procs = []
    for path, defs in ((LIB_PATH, []), (LIB64_PATH, ["-DPSYO_F64"])):
        if not force and os.path.exists(path):
            t = os.path.getmtime(path)
            if all(os.path.getmtime(d) <= t for d in deps):
                continue
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
               "-Wall", "-Wno-unused-function"] + defs + ["-o", path + ".tmp"] + srcs + ["-lpthread"]
        procs.append((path, subprocess.Popen(cmd)))
    for path, p in procs:
        if p.wait() != 0:
            raise RuntimeError("oracle build failed: %s" % path)
        os.replace(path + ".tmp", path)
    return LIB_PATH


_lib = None
_lib64 = None


def _bind_scene_calls(L):
    vp, u32 = C.c_void_p, C.c_uint32
    L.psyo_scene_create.restype = vp
    L.psyo_scene_create.argtypes = [vp]
    L.psyo_scene_destroy.argtypes = [vp]
    L.psyo_trace.argtypes = [vp, vp, u32, vp, vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), u32]
    L.psyo_render.argtypes = [vp, u32, u32, vp, u32, vp, vp]
    L.psyo_render_sampled.argtypes = [vp, u32, u32, vp, u32, u32, vp, vp]
    L.psyo_render_paths.argtypes = [vp, vp, vp, vp, vp]
    L.psyo_mesh_bvh_info.argtypes = [vp, u32, vp, C.POINTER(u32)]
    L.psyo_light_tree_info.argtypes = [vp, C.POINTER(u32), C.POINTER(u32), C.POINTER(u32)]


def lib64():
    """The FP64 oracle (scene, trace and render calls only)."""
    global _lib64
    if _lib64 is None:
        build()
        L = C.CDLL(LIB64_PATH)
        _bind_scene_calls(L)
        _lib64 = L
    return _lib64


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp, u32, f32, fp, up = C.c_void_p, C.c_uint32, C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_uint32)
        _bind_scene_calls(L)
        L.psyo_hash_u32.restype = u32
        L.psyo_hash_u32.argtypes = [u32, u32]
        L.psyo_hash_u64.restype = C.c_uint64
        L.psyo_hash_u64.argtypes = [C.c_uint64, C.c_uint64]
        L.psyo_hash_u32_to_f32.restype = f32
        L.psyo_hash_u32_to_f32.argtypes = [u32, u32]
        L.psyo_get_sample_4d.argtypes = [u32, u32, u32, u32, u32, fp]
        L.psyo_golden_ratio_sample.restype = f32
        L.psyo_golden_ratio_sample.argtypes = [u32, u32]
        L.psyo_wavelengths.argtypes = [u32, u32, u32, u32, fp]
        L.psyo_probit.restype = f32
        L.psyo_probit.argtypes = [f32, f32]
        L.psyo_fast_exp.restype = f32
        L.psyo_fast_exp.argtypes = [f32]
        L.psyo_hilbert_d2xy.argtypes = [u32, up, up]
        L.psyo_hilbert_xy2d.restype = u32
        L.psyo_hilbert_xy2d.argtypes = [u32, u32]
        L.psyo_traversal_table.argtypes = [vp]
        for n in ("psyo_xf_mul",):
            getattr(L, n).argtypes = [fp, fp, fp]
        L.psyo_xf_inverse.argtypes = [fp, fp]
        L.psyo_xf_lerp.argtypes = [fp, fp, f32, fp]
        L.psyo_xf_point.argtypes = [fp, fp, fp]
        L.psyo_xf_normal.argtypes = [fp, fp, fp]
        L.psyo_xf_vector.argtypes = [fp, fp, fp]
        L.psyo_lerp3.argtypes = [fp, fp, f32, fp]
        L.psyo_lerp.restype = f32
        L.psyo_lerp.argtypes = [f32, f32, f32]
        L.psyo_lerp_slice.restype = f32
        L.psyo_lerp_slice.argtypes = [fp, u32, f32]
        L.psyo_xyz_to_spectrum.argtypes = [fp, f32, fp]
        L.psyo_spectrum_to_xyz.argtypes = [fp, f32, fp]
        L.psyo_rec709_e_to_xyz.argtypes = [fp, fp]
        L.psyo_rec709_to_xyz.argtypes = [fp, fp]
        L.psyo_xyz_to_srgb8.argtypes = [fp, C.c_uint32, C.c_uint32, C.c_void_p]
        L.psyo_intersect_triangle.restype = C.c_int
        L.psyo_intersect_triangle.argtypes = [fp, fp, f32, fp, fp, fp, fp]
        L.psyo_quick_select_ints.restype = u32
        L.psyo_quick_select_ints.argtypes = [C.POINTER(C.c_int32), u32, u32]
        L.psyo_increment_ulp_check.restype = C.c_int
        L.psyo_halton_sample.restype = C.c_int
        L.psyo_halton_sample.argtypes = [u32, u32, fp]
        for n in ("psyo_compact_encode", "psyo_color_compress", "psyo_color_decompress"):
            getattr(L, n).argtypes = [u32, vp, u32, vp, vp] if n == "psyo_compact_encode" else [vp, u32, vp, vp]
        L.psyo_compact_decode.argtypes = [u32, vp, u32, vp]
        L.psyo_signed48_decode_u64.argtypes = [C.c_uint64, fp]
        L.psyo_fluv32_decode_yuv.argtypes = [vp, u32, vp]
        L.psyo_f16_from_f32.restype = u32
        L.psyo_f16_from_f32.argtypes = [f32]
        L.psyo_f16_to_f32.restype = f32
        L.psyo_f16_to_f32.argtypes = [u32]
        L.psyo_closure_compress.argtypes = [vp, u32, u32, vp, vp]
        L.psyo_closure_decompress.argtypes = [vp, u32, u32, vp, vp]
        _lib = L
    return _lib
