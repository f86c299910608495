"""Python binding of the C ABI (include/psy_gpu.h), mirroring the
reference's Tracer / Renderer interface for this path:

    scene = Scene(scene_data)                  # AssemblyBuilder::build + Camera::new
    tracer = Tracer(scene)                     # Tracer::from_assembly
    hits = tracer.trace(rays)                  # Tracer::trace
    tracer.rays_traced()                       # Tracer::rays_traced
    img, stats = Renderer(scene).render()      # Renderer::render

The CUDA library is required: loading fails loudly when it is missing or no
GPU is present; there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

from . import abi

_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libpsy_gpu.so")
_lib = None

EXPORTED = [
    "psy_scene_create", "psy_scene_destroy", "psy_scene_device_bytes", "psy_trace", "psy_trace_device",
    "psy_rays_traced", "psy_render_bucket", "psy_render_image_device", "psy_render_image", "psy_last_error",
    "psy_version", "psy_render_bucket_noalloc", "psy_server_create", "psy_server_add_scene", "psy_submit",
    "psy_poll", "psy_wait", "psy_cancel", "psy_server_stats", "psy_server_destroy", "psy_autotune",
    "psy_xyz_to_srgb8", "psy_halton_samples", "psy_render_rows_device", "psy_compact_element_size",
    "psy_compact_encode", "psy_compact_decode", "psy_fluv32_decode_yuv", "psy_color_compress",
    "psy_color_decompress", "psy_closure_compress", "psy_closure_decompress",
]


class PsyError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("psy error %d: %s" % (code, msg))
        self.code = code


def lib(path=None):
    """Load libpsy_gpu.so (built by psychopath_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or _LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("libpsy_gpu.so not built (run psychopath_gb300.build.build()): %s" % p)
    L = C.CDLL(p)
    vp, u32 = C.c_void_p, C.c_uint32
    L.psy_scene_create.argtypes = [vp, vp, C.POINTER(vp)]
    L.psy_scene_destroy.argtypes = [vp]
    L.psy_scene_device_bytes.argtypes = [vp, C.POINTER(C.c_uint64)]
    L.psy_trace.argtypes = [vp, vp, u32, vp, vp, vp]
    L.psy_trace_device.argtypes = [vp, vp, u32, vp, vp]
    L.psy_rays_traced.argtypes = [vp, C.POINTER(C.c_uint64)]
    L.psy_render_bucket.argtypes = [vp, vp, u32, u32, vp, vp]
    L.psy_render_image_device.argtypes = [vp, vp, vp, vp, vp]
    L.psy_render_image.argtypes = [vp, vp, vp, vp]
    L.psy_render_bucket_noalloc.argtypes = [vp, vp, u32, u32, vp, vp]
    L.psy_render_rows_device.argtypes = [vp, u32, u32, vp, vp, vp]
    L.psy_last_error.restype = C.c_char_p
    L.psy_version.restype = C.c_char_p
    L.psy_debug_mesh_bvh_info.argtypes = [vp, u32, vp, C.POINTER(u32)]
    L.psy_debug_scene_info.argtypes = [vp, C.POINTER(u32), C.POINTER(u32), C.POINTER(u32)]
    L.psy_debug_set_launch.argtypes = [vp, C.c_int, u32]
    L.psy_debug_set_resident_tail.argtypes = [vp, C.c_int]
    L.psy_debug_color_spectra.argtypes = [vp, u32, vp, vp, vp, C.POINTER(u32)]
    L.psy_debug_counters.argtypes = [vp, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    L.psy_debug_set_trace.argtypes = [vp, C.c_int, C.c_int]
    L.psy_debug_set_sort.argtypes = [vp, C.c_int]
    L.psy_debug_set_shade.argtypes = [vp, C.c_int]
    L.psy_debug_host_build.argtypes = [vp, vp, u32, vp, C.POINTER(u32), C.POINTER(u32)]
    L.psy_debug_set_graph.argtypes = [vp, C.c_int]
    L.psy_debug_set_ray_order.argtypes = [vp, C.c_int]
    L.psy_debug_ray_order.argtypes = [vp, vp, u32, vp, vp, vp]
    L.psy_debug_render_sized.argtypes = [vp, u32, u32, u32, u32, vp, vp]
    L.psy_debug_push_tables.argtypes = [vp, vp, vp]
    L.psy_debug_scene_flags.argtypes = [vp, C.POINTER(u32)]
    L.psy_debug_host_nodes.argtypes = [vp, vp, C.c_int, vp, C.POINTER(u32), vp, C.POINTER(u32)]
    L.psy_debug_host_nodes_h.argtypes = [vp, vp, vp, C.POINTER(u32)]
    L.psy_debug_render_paths.argtypes = [vp, vp, u32, u32, vp, vp]
    L.psy_debug_samplers.argtypes = [C.c_int, vp, u32, vp, vp]
    L.psy_server_create.argtypes = [vp, C.POINTER(vp)]
    L.psy_server_add_scene.argtypes = [vp, vp, C.POINTER(u32)]
    L.psy_submit.argtypes = [vp, vp, C.POINTER(C.c_uint64)]
    L.psy_poll.argtypes = [vp, C.c_uint64, vp]
    L.psy_wait.argtypes = [vp, C.c_uint64, C.c_double, vp]
    L.psy_cancel.argtypes = [vp, C.c_uint64]
    L.psy_server_stats.argtypes = [vp, vp]
    L.psy_server_destroy.argtypes = [vp]
    L.psy_autotune.argtypes = [vp, vp, vp]
    L.psy_xyz_to_srgb8.argtypes = [vp, u32, u32, vp, vp]
    L.psy_halton_samples.argtypes = [u32, vp, u32, vp, vp]
    L.psy_compact_element_size.argtypes = [u32, C.POINTER(u32)]
    L.psy_compact_encode.argtypes = [u32, vp, u32, vp, vp, vp]
    L.psy_compact_decode.argtypes = [u32, vp, u32, vp, vp]
    L.psy_fluv32_decode_yuv.argtypes = [vp, u32, vp, vp]
    L.psy_color_compress.argtypes = [vp, u32, vp, vp, vp]
    L.psy_color_decompress.argtypes = [vp, u32, vp, vp, vp]
    L.psy_closure_compress.argtypes = [vp, u32, u32, vp, vp, vp]
    L.psy_closure_decompress.argtypes = [vp, u32, u32, vp, vp, vp]
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise PsyError(rc, lib().psy_last_error().decode())


def host_build_info(scene_data, obj, bounds="fp32"):
    """Run only the host-side scene build (no GPU needed): the mesh object's
    triangle order after the BVH build, its BVH4 node count and the scene's
    worst-case traversal stack depth."""
    desc = scene_data.desc()
    opts = abi.PsySceneOptions()
    opts.bounds_precision = abi.PSY_BOUNDS_FP16 if bounds == "fp16" else abi.PSY_BOUNDS_FP32
    n = scene_data.objects[obj]["indices"].shape[0] if scene_data.objects[obj]["kind"] == abi.PSY_OBJ_MESH else 0
    order = np.zeros(max(1, n), dtype=np.uint32)
    nc, ms = C.c_uint32(), C.c_uint32()
    _check(lib().psy_debug_host_build(C.byref(desc), C.byref(opts), obj, order.ctypes.data, C.byref(nc), C.byref(ms)))
    return order[:n], nc.value, ms.value


def host_nodes(scene_data, serial=False, bounds="fp32"):
    """Host-side build only (no GPU needed): the scene's BVH4 node records and
    motion bounds as raw bytes (128 and 96 bytes per entry)."""
    desc = scene_data.desc()
    opts = abi.PsySceneOptions()
    opts.bounds_precision = abi.PSY_BOUNDS_FP16 if bounds == "fp16" else abi.PSY_BOUNDS_FP32
    nc, ec = C.c_uint32(), C.c_uint32()
    _check(lib().psy_debug_host_nodes(C.byref(desc), C.byref(opts), 1 if serial else 0, None, C.byref(nc), None,
                                      C.byref(ec)))
    nodes = np.zeros(nc.value * 128, dtype=np.uint8)
    ext = np.zeros(max(1, ec.value) * 96, dtype=np.uint8)
    _check(lib().psy_debug_host_nodes(C.byref(desc), C.byref(opts), 1 if serial else 0, nodes.ctypes.data,
                                      C.byref(nc), ext.ctypes.data, C.byref(ec)))
    return nodes, ext[:ec.value * 96]


def host_nodes_h(scene_data):
    """Host-side build only (no GPU needed): the FP16 node copies of the
    scene's BVH4 nodes as raw bytes, 96 per node."""
    desc = scene_data.desc()
    opts = abi.PsySceneOptions()
    opts.bounds_precision = abi.PSY_BOUNDS_FP16
    nc = C.c_uint32()
    _check(lib().psy_debug_host_nodes_h(C.byref(desc), C.byref(opts), None, C.byref(nc)))
    nodes = np.zeros(nc.value * 96, dtype=np.uint8)
    _check(lib().psy_debug_host_nodes_h(C.byref(desc), C.byref(opts), nodes.ctypes.data, C.byref(nc)))
    return nodes


def halton_samples_device(dimension, d_indices_ptr, n, d_out_ptr, stream=None):
    """psy_halton_samples: halton::sample(index, dimension) for n device-resident
    u32 indices into n device floats."""
    _check(lib().psy_halton_samples(dimension, d_indices_ptr, n, d_out_ptr, stream))


def halton_samples(dimension, indices):
    """halton::sample(index, dimension) for a host array of indices, computed on
    the GPU (device buffers through torch); returns float32 numpy."""
    import torch
    idx = torch.from_numpy(np.ascontiguousarray(indices, dtype=np.uint32).view(np.int32)).cuda()
    out = torch.empty(idx.numel(), dtype=torch.float32, device="cuda")
    halton_samples_device(dimension, idx.data_ptr(), idx.numel(), out.data_ptr())
    torch.cuda.synchronize()
    return out.cpu().numpy()


SAMPLER_OPS = {"hash_u32": 0, "hash_u32_to_f32": 1, "golden_ratio_sample": 2, "get_sample_4d": 3,
               "wavelengths": 4}


def device_samplers(op, args):
    """psy_debug_samplers: the render path's samplers evaluated on the GPU.
    args: (n, 5) uint32 rows (a, b, c, d, e); returns (n, 4) uint32 words
    (f32 results as their bits)."""
    import torch
    args = np.ascontiguousarray(args, dtype=np.uint32).reshape(-1, 5)
    n = args.shape[0]
    d_args = torch.from_numpy(args.view(np.int32).copy()).cuda()
    d_out = torch.zeros((n, 4), dtype=torch.int32, device="cuda")
    _check(lib().psy_debug_samplers(SAMPLER_OPS[op], d_args.data_ptr(), n, d_out.data_ptr(), None))
    return d_out.cpu().numpy().view(np.uint32)


def push_tables():
    """Host-side only (no GPU needed): the traversal table as the device holds
    it (8 octants x 48 codes) and the static-scene traversal's push tables
    (row per octant and code; 32 rows x 16 hit masks of 16-bit entries)."""
    table = np.zeros((8, 48), dtype=np.uint8)
    rows = np.zeros((8, 48), dtype=np.uint8)
    lut = np.zeros((32, 16), dtype=np.uint16)
    _check(lib().psy_debug_push_tables(table.ctypes.data, rows.ctypes.data, lut.ctypes.data))
    return table, rows, lut


class Scene:
    """A scene resident on the GPU (psy_scene_create)."""

    def __init__(self, scene_data, bounds="fp32", shading="f64", ray_order="as_given", bvh="sah"):
        self.data = scene_data
        self._desc = scene_data.desc()
        opts = abi.PsySceneOptions()
        opts.bounds_precision = abi.PSY_BOUNDS_FP16 if bounds == "fp16" else abi.PSY_BOUNDS_FP32
        opts.shading_precision = abi.PSY_SHADING_F32 if shading == "f32" else abi.PSY_SHADING_F64
        opts.ray_order = abi.PSY_RAY_ORDER_BINNED if ray_order == "binned" else abi.PSY_RAY_ORDER_AS_GIVEN
        opts.bvh_build = abi.PSY_BVH_GPU if bvh == "gpu" else abi.PSY_BVH_SAH
        h = C.c_void_p()
        _check(lib().psy_scene_create(C.byref(self._desc), C.byref(opts), C.byref(h)))
        self.h = h
        self.width, self.height, self.spp = scene_data.width, scene_data.height, scene_data.spp

    def close(self):
        if getattr(self, "h", None):
            lib().psy_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def device_bytes(self):
        v = C.c_uint64()
        _check(lib().psy_scene_device_bytes(self.h, C.byref(v)))
        return v.value

    def info(self):
        a, b, c = C.c_uint32(), C.c_uint32(), C.c_uint32()
        _check(lib().psy_debug_scene_info(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return {"max_stack": a.value, "nodes": b.value, "stack_variant": c.value}

    def mesh_bvh_info(self, obj):
        n = self.data.objects[obj]["indices"].shape[0]
        order = np.zeros(n, dtype=np.uint32)
        nc = C.c_uint32()
        _check(lib().psy_debug_mesh_bvh_info(self.h, obj, order.ctypes.data, C.byref(nc)))
        return order, nc.value

    def counters(self, enable):
        """Read (and zero) the render traversal counters, then enable or
        disable counting for later renders: (node visits, triangle tests,
        rays)."""
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(lib().psy_debug_counters(self.h, 1 if enable else 0, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def flags(self):
        """Scene facts the traversal kernel choice depends on: {'static_fast',
        'ordered_slabs', 'fp16'}."""
        f = C.c_uint32()
        _check(lib().psy_debug_scene_flags(self.h, C.byref(f)))
        return {"static_fast": bool(f.value & 1), "ordered_slabs": bool(f.value & 2), "fp16": bool(f.value & 4)}

    def set_trace(self, mode=1, minb=4):
        """Traversal kernel: mode 0 = one thread per ray, 1 = persistent with
        lane refill, 2 = warp packets, 3 = the static-scene traversal (scenes
        with motion, instance transforms or FP16 bounds use mode 0's kernels);
        minb = target resident blocks per SM (4-8; 6-12 for mode 3)."""
        _check(lib().psy_debug_set_trace(self.h, mode, minb))

    def set_shade(self, minb):
        """Shading kernel register budget: 4, 6 or 8 resident blocks per SM."""
        _check(lib().psy_debug_set_shade(self.h, minb))

    def set_sort(self, bits):
        """Path ordering between wavefront iterations: 0 = off; 4, 10, 13, 16
        = counting sort by occlusion, octant and origin cell; 19, 25, 31 =
        radix sort by occlusion and a two-point key."""
        _check(lib().psy_debug_set_sort(self.h, bits))

    def set_launch(self, grid=0, wave_paths=0):
        _check(lib().psy_debug_set_launch(self.h, grid, wave_paths))

    def color_spectra(self, heros):
        """Each tabulated colour's spectrum at the hero wavelengths `heros`,
        by the upsampling and from its table: two arrays (colours, n, 4)."""
        import torch
        nc = C.c_uint32()
        _check(lib().psy_debug_color_spectra(self.h, 0, None, None, None, C.byref(nc)))
        n = len(heros)
        d_h = torch.from_numpy(np.asarray(heros, dtype=np.float32)).cuda()
        ex = torch.zeros((max(1, nc.value), n, 4), dtype=torch.float32, device="cuda")
        tb = torch.zeros_like(ex)
        _check(lib().psy_debug_color_spectra(self.h, n, d_h.data_ptr(), ex.data_ptr(), tb.data_ptr(), C.byref(nc)))
        return ex.cpu().numpy()[: nc.value], tb.cpu().numpy()[: nc.value]

    def set_resident_tail(self, iterations):
        """The last `iterations` wavefront iterations of a wave launch each
        kernel on its resident blocks (0: none; images unchanged)."""
        _check(lib().psy_debug_set_resident_tail(self.h, iterations))

    def autotune(self, probe_paths=0, repeats=0, max_wave_mib=0):
        """psy_autotune: time a probe render under candidate launch
        configurations and keep the fastest on the scene (images unchanged).
        max_wave_mib caps the wave buffers of the larger-wave step (0: the
        library's bound)."""
        o = abi.PsyTuneOptions()
        o.probe_paths, o.repeats, o.max_wave_mib = probe_paths, repeats, max_wave_mib
        r = abi.PsyTuneResult()
        _check(lib().psy_autotune(self.h, C.byref(o), C.byref(r)))
        return r.as_dict()

    def set_ray_order(self, binned=True):
        """Trace calls of >= 65,536 rays: sort the rays by their two-point
        key (origin and a point along the ray) first."""
        _check(lib().psy_debug_set_ray_order(self.h, 1 if binned else 0))

    def ray_order(self, rays):
        """The order a binned trace call gives a host batch of PsyRay
        records: (sorted keys, ray index at each position) as numpy arrays."""
        import torch
        n = len(rays)
        d_rays = torch.from_numpy(np.ascontiguousarray(rays).view(np.uint8).reshape(-1)).cuda()
        d_keys = torch.empty(n, dtype=torch.int32, device="cuda")
        d_order = torch.empty(n, dtype=torch.int32, device="cuda")
        _check(lib().psy_debug_ray_order(self.h, d_rays.data_ptr(), n, d_keys.data_ptr(), d_order.data_ptr(), None))
        return d_keys.cpu().numpy().view(np.uint32), d_order.cpu().numpy().view(np.uint32)

    def set_graph(self, on=True):
        """Replay each render wave from a captured CUDA graph."""
        _check(lib().psy_debug_set_graph(self.h, 1 if on else 0))

    def render_sized(self, width, height, spp, seed, d_xyz_ptr, stream=None):
        """Whole image at another resolution through the scene's camera into a
        device buffer (blocking): one request on the plain render path."""
        _check(lib().psy_debug_render_sized(self.h, width, height, spp, seed, d_xyz_ptr, stream))


class Tracer:
    """Tracer::from_assembly / trace / rays_traced over the GPU scene."""

    def __init__(self, scene):
        self.scene = scene

    def trace(self, rays, full=False):
        rays = np.ascontiguousarray(rays, dtype=abi.ray_dtype())
        n = len(rays)
        hits = np.zeros(n, dtype=abi.hit_dtype())
        fh = np.zeros(n, dtype=abi.surface_hit_dtype()) if full else None
        _check(lib().psy_trace(self.scene.h, rays.ctypes.data, n, hits.ctypes.data,
                               fh.ctypes.data if full else None, None))
        return (hits, fh) if full else hits

    def trace_device(self, d_rays_ptr, n, d_hits_ptr, stream=None):
        _check(lib().psy_trace_device(self.scene.h, d_rays_ptr, n, d_hits_ptr, stream))

    def rays_traced(self):
        v = C.c_uint64()
        _check(lib().psy_rays_traced(self.scene.h, C.byref(v)))
        return v.value


class Renderer:
    """Renderer::render over the GPU scene: XYZ image (height, width, 3)."""

    def __init__(self, scene):
        self.scene = scene

    def render(self, crop=None, out=None):
        """psy_render_image: the scene's image (height x width x 3 XYZ) into
        a host array -- `out` when given (C-contiguous float32 of that shape,
        e.g. a view of pinned memory), else a new one -- and the render
        statistics."""
        shape = (self.scene.height, self.scene.width, 3)
        if out is None:
            img = np.zeros(shape, dtype=np.float32)
        else:
            if out.shape != shape or out.dtype != np.float32 or not out.flags["C_CONTIGUOUS"]:
                raise ValueError("out must be a C-contiguous float32 array of shape %s" % (shape,))
            img = out
        st = abi.PsyRenderStats()
        cr = (C.c_uint32 * 4)(*crop) if crop is not None else None
        _check(lib().psy_render_image(self.scene.h, cr, img.ctypes.data, C.byref(st)))
        return img, st.as_dict()

    def render_device(self, d_xyz_ptr, stream=None, crop=None, stats=False):
        st = abi.PsyRenderStats() if stats else None
        cr = (C.c_uint32 * 4)(*crop) if crop is not None else None
        _check(lib().psy_render_image_device(self.scene.h, cr, d_xyz_ptr, stream, C.byref(st) if stats else None))
        return st.as_dict() if stats else None

    def render_rows_device(self, first_row, row_step, d_xyz_ptr, stream=None, stats=False):
        """psy_render_rows_device: image rows first_row, first_row +
        row_step, ... into a compact device buffer (rows x width x 3)."""
        st = abi.PsyRenderStats() if stats else None
        _check(lib().psy_render_rows_device(self.scene.h, first_row, row_step, d_xyz_ptr, stream,
                                            C.byref(st) if stats else None))
        return st.as_dict() if stats else None

    def render_bucket_noalloc(self, x, y, w, h, d_xyz_ptr, spp=None, seed=None, stream=None):
        """psy_render_bucket_noalloc: render into a caller-owned DEVICE buffer
        of w*h*3 floats; the library allocates no device memory for it."""
        b = abi.PsyBucket(x, y, w, h)
        _check(lib().psy_render_bucket_noalloc(self.scene.h, C.byref(b),
                                               spp if spp is not None else self.scene.spp,
                                               seed if seed is not None else self.scene.data.seed, d_xyz_ptr, stream))

    def render_paths(self, x, y, w, h, spp=None, seed=None):
        """psy_debug_render_paths: every path's final colour (n, 4) and hero
        wavelength (n,) of a bucket, sample s of pixel (x', y') at index
        ((y' - y) * w + (x' - x)) * spp + s."""
        spp = spp if spp is not None else self.scene.spp
        n = w * h * spp
        col = np.zeros((n, 4), dtype=np.float32)
        wl = np.zeros(n, dtype=np.float32)
        b = abi.PsyBucket(x, y, w, h)
        _check(lib().psy_debug_render_paths(self.scene.h, C.byref(b), spp,
                                            seed if seed is not None else self.scene.data.seed,
                                            col.ctypes.data, wl.ctypes.data))
        return col, wl

    def render_bucket(self, x, y, w, h, spp=None, seed=None):
        out = np.zeros((h, w, 3), dtype=np.float32)
        b = abi.PsyBucket(x, y, w, h)
        st = abi.PsyRenderStats()
        _check(lib().psy_render_bucket(self.scene.h, C.byref(b), spp if spp is not None else self.scene.spp,
                                       seed if seed is not None else self.scene.data.seed, out.ctypes.data,
                                       C.byref(st)))
        return out, st.as_dict()


class Server:
    """Render server over resident scenes (psy_server_*, psy_submit,
    psy_poll, psy_wait, psy_cancel)."""

    def __init__(self, hbm_budget_bytes=0, wave_paths=0, max_active=0, use_graphs=False, waves_in_flight=0,
                 policy="fifo", aging_ms=0):
        o = abi.PsyServerOptions()
        o.hbm_budget_bytes = hbm_budget_bytes
        o.wave_paths = wave_paths
        o.max_active = max_active
        o.use_graphs = 1 if use_graphs else 0
        o.waves_in_flight = waves_in_flight
        o.policy = abi.PSY_SCHED_SHORTEST if policy == "shortest" else abi.PSY_SCHED_FIFO
        o.aging_ms = aging_ms
        h = C.c_void_p()
        _check(lib().psy_server_create(C.byref(o), C.byref(h)))
        self.h = h
        self._scenes = []
        self._bufs = {}

    def add_scene(self, scene):
        v = C.c_uint32()
        _check(lib().psy_server_add_scene(self.h, scene.h, C.byref(v)))
        self._scenes.append(scene)  # the server borrows it
        return v.value

    def submit(self, lane, width, height, spp, seed, out=None, d_out=None):
        """Queue a request.  out: a float32 host array of height*width*3
        (allocated when neither out nor d_out is given); d_out: a device
        pointer instead.  Returns the request id."""
        if out is None and d_out is None:
            out = np.zeros((height, width, 3), dtype=np.float32)
        r = abi.PsyRequest()
        r.scene, r.width, r.height, r.spp, r.seed = lane, width, height, spp, seed
        r.xyz_out = out.ctypes.data if out is not None else None
        r.d_xyz_out = d_out
        v = C.c_uint64()
        _check(lib().psy_submit(self.h, C.byref(r), C.byref(v)))
        self._bufs[v.value] = out
        return v.value

    def result(self, rid):
        return self._bufs.get(rid)

    def poll(self, rid):
        st = abi.PsyRequestStatus()
        _check(lib().psy_poll(self.h, rid, C.byref(st)))
        return st.as_dict()

    def wait(self, rid, timeout=120.0):
        st = abi.PsyRequestStatus()
        _check(lib().psy_wait(self.h, rid, timeout, C.byref(st)))
        return st.as_dict()

    def cancel(self, rid):
        _check(lib().psy_cancel(self.h, rid))

    def stats(self):
        st = abi.PsyServerStats()
        _check(lib().psy_server_stats(self.h, C.byref(st)))
        return st.as_dict()

    def close(self):
        if getattr(self, "h", None):
            lib().psy_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
