"""Oracle (test infrastructure only): numpy-level wrappers over the oracle
library -- build a scene from a SceneData, trace ray arrays, render images."""
import ctypes as C

import numpy as np

from . import lib as _lib32
from . import lib64 as _lib64


class OracleScene:
    """A scene in the oracle.  f64=True uses the FP64 oracle build (the same
    algorithm with f64 arithmetic) for trace and render calls."""

    def __init__(self, scene_data, f64=False):
        self._data = scene_data
        self._desc = scene_data.desc()
        self._L = _lib64() if f64 else _lib32()
        self.h = self._L.psyo_scene_create(C.byref(self._desc))
        if not self.h:
            raise RuntimeError("oracle scene build failed")
        self.width, self.height, self.spp = scene_data.width, scene_data.height, scene_data.spp

    def close(self):
        if self.h:
            self._L.psyo_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def trace(self, rays, threads=1, full=False):
        """rays: numpy array of abi.ray_dtype().  Returns (hits, full_or_None,
        node_tests, tri_tests)."""
        from psychopath_gb300 import abi
        rays = np.ascontiguousarray(rays)
        n = len(rays)
        hits = np.zeros(n, dtype=abi.hit_dtype())
        fh = np.zeros(n, dtype=abi.surface_hit_dtype()) if full else None
        nt, tt = C.c_uint64(0), C.c_uint64(0)
        rc = self._L.psyo_trace(self.h, rays.ctypes.data, n, hits.ctypes.data,
                               fh.ctypes.data if full else None, C.byref(nt), C.byref(tt), threads)
        if rc != 0:
            raise RuntimeError("psyo_trace failed: %d" % rc)
        return hits, fh, nt.value, tt.value

    def render(self, spb=4096, threads=1, crop=None, max_buckets=0):
        from psychopath_gb300 import abi
        img = np.zeros((self.height, self.width, 3), dtype=np.float32)
        st = abi.PsyRenderStats()
        cr = (C.c_uint32 * 4)(*crop) if crop is not None else None
        rc = self._L.psyo_render(self.h, spb, threads, cr, max_buckets, img.ctypes.data, C.byref(st))
        if rc != 0:
            raise RuntimeError("psyo_render failed: %d" % rc)
        return img, st.as_dict()

    def render_sampled(self, stride, max_buckets=0, spb=4096, threads=1):
        """Render every stride-th bucket of the Hilbert order (a bounded sample
        of the frame spread over the image)."""
        from psychopath_gb300 import abi
        img = np.zeros((self.height, self.width, 3), dtype=np.float32)
        st = abi.PsyRenderStats()
        rc = self._L.psyo_render_sampled(self.h, spb, threads, None, stride, max_buckets, img.ctypes.data, C.byref(st))
        if rc != 0:
            raise RuntimeError("psyo_render_sampled failed: %d" % rc)
        return img, st.as_dict()

    def render_paths(self, x, y, w, h):
        from psychopath_gb300 import abi
        n = w * h * self.spp
        col = np.zeros((n, 4), dtype=np.float32)
        wl = np.zeros(n, dtype=np.float32)
        nr = np.zeros(n, dtype=np.uint32)
        b = abi.PsyBucket(x, y, w, h)
        rc = self._L.psyo_render_paths(self.h, C.byref(b), col.ctypes.data, wl.ctypes.data, nr.ctypes.data)
        if rc != 0:
            raise RuntimeError("psyo_render_paths failed: %d" % rc)
        return col, wl, nr

    def light_tree_info(self):
        """(nodes, leaves, depth) of the scene's light tree."""
        n, l, d = C.c_uint32(), C.c_uint32(), C.c_uint32()
        rc = self._L.psyo_light_tree_info(self.h, C.byref(n), C.byref(l), C.byref(d))
        if rc != 0:
            raise RuntimeError("light tree info failed")
        return n.value, l.value, d.value

    def mesh_bvh_info(self, obj):
        o = self._data.objects[obj]
        n = o["indices"].shape[0]
        order = np.zeros(n, dtype=np.uint32)
        nc = C.c_uint32(0)
        rc = self._L.psyo_mesh_bvh_info(self.h, obj, order.ctypes.data, C.byref(nc))
        if rc != 0:
            raise RuntimeError("bvh info failed")
        return order, nc.value
