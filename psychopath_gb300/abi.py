"""ctypes mirror of include/psy_gpu.h (the C ABI of the tracing path)."""
import ctypes as C

PSY_OK = 0
PSY_E_INVALID = -1
PSY_E_CUDA = -2
PSY_E_NOMEM = -3
PSY_E_UNSUPPORTED = -4
PSY_E_TIMEOUT = -5
PSY_E_BUSY = -6
PSY_E_NOTFOUND = -7
PSY_E_CANCELLED = -8
PSY_E_OVERFLOW = -9

PSY_COLOR_XYZ, PSY_COLOR_BLACKBODY, PSY_COLOR_TEMPERATURE = 0, 1, 2
PSY_SHADER_EMIT, PSY_SHADER_LAMBERT, PSY_SHADER_GGX = 0, 1, 2
PSY_OBJ_MESH, PSY_OBJ_RECT_LIGHT, PSY_OBJ_SPHERE_LIGHT = 0, 1, 2
PSY_BOUNDS_FP32, PSY_BOUNDS_FP16 = 0, 1
PSY_SHADING_F64, PSY_SHADING_F32 = 0, 1
PSY_RAY_ORDER_AS_GIVEN, PSY_RAY_ORDER_BINNED = 0, 1
PSY_BVH_SAH, PSY_BVH_GPU = 0, 1
PSY_RAY_OCCLUSION = 1
PSY_NOALLOC_MAX_SAMPLES = 262144
PSY_HIT_MISS, PSY_HIT_OCCLUDE, PSY_HIT_SURFACE, PSY_HIT_LIGHT = 0, 1, 2, 3
PSY_REQ_QUEUED, PSY_REQ_RUNNING, PSY_REQ_DONE, PSY_REQ_CANCELLED, PSY_REQ_FAILED = 0, 1, 2, 3, 4
PSY_SCHED_FIFO, PSY_SCHED_SHORTEST = 0, 1
PSY_TUNE_GRID_RESIDENT = 0xFFFFFFFF
PSY_COMPACT_FLUV32, PSY_COMPACT_OCT32, PSY_COMPACT_OCT32_PRECISE = 0, 1, 2
PSY_COMPACT_UNSIGNED32, PSY_COMPACT_UNSIGNED40, PSY_COMPACT_SIGNED48 = 3, 4, 5

_fp = C.POINTER(C.c_float)
_up = C.POINTER(C.c_uint32)


class PsyColor(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("v", C.c_float * 3)]


class PsyShaderDesc(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("color", PsyColor), ("roughness", C.c_float), ("fresnel", C.c_float)]


class PsyYuv(C.Structure):
    _fields_ = [("y", C.c_float), ("u", C.c_uint8), ("v", C.c_uint8), ("pad", C.c_uint8 * 2)]


def color_dtype():
    """numpy mirror of PsyColor (16 bytes)."""
    import numpy as np
    return np.dtype([("kind", "<u4"), ("v", "<f4", (3,))])


def shader_dtype():
    """numpy mirror of PsyShaderDesc (28 bytes)."""
    import numpy as np
    return np.dtype([("kind", "<u4"), ("color", color_dtype()), ("roughness", "<f4"), ("fresnel", "<f4")])


def yuv_dtype():
    """numpy mirror of PsyYuv (8 bytes)."""
    import numpy as np
    return np.dtype([("y", "<f4"), ("u", "u1"), ("v", "u1"), ("pad", "u1", (2,))])


class PsyObjectDesc(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("time_samples", C.c_uint32), ("num_verts", C.c_uint32),
                ("num_tris", C.c_uint32), ("verts", _fp), ("normals", _fp), ("indices", _up),
                ("dims", _fp), ("colors", C.POINTER(PsyColor))]


class PsyInstanceDesc(C.Structure):
    _fields_ = [("object", C.c_uint32), ("shader", C.c_int32), ("xform_start", C.c_uint32),
                ("xform_count", C.c_uint32)]


class PsyTransform(C.Structure):
    _fields_ = [("m", C.c_float * 12)]


class PsyCameraDesc(C.Structure):
    _fields_ = [("num_transforms", C.c_uint32), ("transforms", C.POINTER(PsyTransform)),
                ("num_fovs", C.c_uint32), ("fovs", _fp),
                ("num_aperture_radii", C.c_uint32), ("aperture_radii", _fp),
                ("num_focus_distances", C.c_uint32), ("focus_distances", _fp)]


class PsyDistantLightDesc(C.Structure):
    _fields_ = [("num_keys", C.c_uint32), ("radii", _fp), ("directions", _fp),
                ("colors", C.POINTER(PsyColor))]


class PsySceneDesc(C.Structure):
    _fields_ = [("num_objects", C.c_uint32), ("objects", C.POINTER(PsyObjectDesc)),
                ("num_shaders", C.c_uint32), ("shaders", C.POINTER(PsyShaderDesc)),
                ("num_instances", C.c_uint32), ("instances", C.POINTER(PsyInstanceDesc)),
                ("num_xforms", C.c_uint32), ("xforms", C.POINTER(PsyTransform)),
                ("camera", PsyCameraDesc), ("background", PsyColor),
                ("num_distant_lights", C.c_uint32), ("distant_lights", C.POINTER(PsyDistantLightDesc)),
                ("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_uint32),
                ("seed", C.c_uint32), ("max_bounces", C.c_uint32)]


class PsySceneOptions(C.Structure):
    _fields_ = [("bounds_precision", C.c_uint32), ("shading_precision", C.c_uint32), ("ray_order", C.c_uint32),
                ("bvh_build", C.c_uint32), ("reserved", C.c_uint32 * 4)]


class PsyRay(C.Structure):
    _fields_ = [("orig", C.c_float * 3), ("dir", C.c_float * 3), ("max_t", C.c_float),
                ("time", C.c_float), ("wavelength", C.c_float), ("flags", C.c_uint32)]


class PsyHit(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("prim", C.c_uint32), ("inst", C.c_uint32), ("t", C.c_float),
                ("b0", C.c_float), ("b1", C.c_float), ("b2", C.c_float), ("pad", C.c_float)]


class PsySurfaceHit(C.Structure):
    _fields_ = [("hit", PsyHit), ("pos", C.c_float * 3), ("pos_err", C.c_float), ("nor", C.c_float * 3),
                ("sample_pdf", C.c_float), ("nor_g", C.c_float * 3), ("shader", C.c_int32)]


class PsyBucket(C.Structure):
    _fields_ = [("x", C.c_uint32), ("y", C.c_uint32), ("w", C.c_uint32), ("h", C.c_uint32)]


class PsyRenderStats(C.Structure):
    _fields_ = [("trace_time", C.c_double), ("initial_ray_generation_time", C.c_double),
                ("ray_generation_time", C.c_double), ("sample_writing_time", C.c_double),
                ("total_time", C.c_double), ("ray_count", C.c_uint64), ("accel_node_visits", C.c_uint64),
                ("samples", C.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PsyServerOptions(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("wave_paths", C.c_uint32), ("max_active", C.c_uint32),
                ("use_graphs", C.c_uint32), ("waves_in_flight", C.c_uint32), ("policy", C.c_uint32),
                ("aging_ms", C.c_uint32), ("reserved", C.c_uint32 * 2)]


class PsyRequest(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_uint32),
                ("seed", C.c_uint32), ("reserved", C.c_uint32), ("xyz_out", C.c_void_p), ("d_xyz_out", C.c_void_p)]


class PsyRequestStatus(C.Structure):
    _fields_ = [("state", C.c_uint32), ("error", C.c_int32), ("samples", C.c_uint64), ("queued_s", C.c_double),
                ("latency_s", C.c_double), ("waves", C.c_uint32), ("shared_waves", C.c_uint32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PsyServerStats(C.Structure):
    _fields_ = [("requests_done", C.c_uint64), ("samples_done", C.c_uint64), ("waves", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("hbm_used_bytes", C.c_uint64), ("hbm_peak_bytes", C.c_uint64), ("hbm_budget_bytes", C.c_uint64),
                ("queued", C.c_uint32), ("active", C.c_uint32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PsyTuneOptions(C.Structure):
    _fields_ = [("probe_paths", C.c_uint32), ("repeats", C.c_uint32), ("max_wave_mib", C.c_uint32),
                ("reserved", C.c_uint32 * 5)]


class PsyTuneResult(C.Structure):
    _fields_ = [("trace_mode", C.c_uint32), ("minb", C.c_uint32), ("stack", C.c_uint32), ("grid", C.c_uint32),
                ("sort_bits", C.c_uint32), ("wave_paths", C.c_uint32), ("use_graph", C.c_uint32),
                ("shade_minb", C.c_uint32), ("candidates", C.c_uint32), ("default_s", C.c_double), ("best_s", C.c_double),
                ("resident_tail", C.c_uint32), ("reserved", C.c_uint32)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        if d["grid"] == PSY_TUNE_GRID_RESIDENT:
            d["grid"] = -1  # each wavefront kernel's resident blocks
        return d


# numpy structured dtypes with the same layout (for bulk ray / hit buffers)
def ray_dtype():
    import numpy as np
    return np.dtype([("orig", "<f4", 3), ("dir", "<f4", 3), ("max_t", "<f4"), ("time", "<f4"),
                     ("wavelength", "<f4"), ("flags", "<u4")])


def hit_dtype():
    import numpy as np
    return np.dtype([("kind", "<u4"), ("prim", "<u4"), ("inst", "<u4"), ("t", "<f4"), ("b0", "<f4"),
                     ("b1", "<f4"), ("b2", "<f4"), ("pad", "<f4")])


def surface_hit_dtype():
    import numpy as np
    return np.dtype([("hit", hit_dtype()), ("pos", "<f4", 3), ("pos_err", "<f4"), ("nor", "<f4", 3),
                     ("sample_pdf", "<f4"), ("nor_g", "<f4", 3), ("shader", "<i4")])


assert C.sizeof(PsyRay) == 40
assert C.sizeof(PsyHit) == 32
assert C.sizeof(PsySurfaceHit) == 80
assert C.sizeof(PsyServerOptions) == 40
assert C.sizeof(PsyRequest) == 40
assert C.sizeof(PsyRequestStatus) == 40
