"""The GPU library's host-side BVH build produces the reference's trees: the
same triangle order after the SAH build and the same BVH4 node count as the
oracle's restatement of src/accel/bvh_base.rs + src/accel/bvh4.rs (runs on
CPU: only the host build)."""
import numpy as np
import pytest

from oracle.runner import OracleScene
from psychopath_gb300 import gpu

from . import scene_cases as sc


@pytest.mark.parametrize("case", ["cornell", "sphere", "motion", "grid"])
def test_bvh_identical_to_oracle(gpu_lib, case):
    if case == "cornell":
        s = sc.cornell()
    elif case == "sphere":
        s = sc.sphere_small(level=4)
    elif case == "motion":
        s = sc.motion_small()
    else:
        s, _, _ = sc.grid_small()
    o = OracleScene(s)
    for obj, od in enumerate(s.objects):
        if od["kind"] != 0:
            continue
        order_g, nodes_g, max_stack = gpu.host_build_info(s, obj)
        order_o, nodes_o = o.mesh_bvh_info(obj)
        assert np.array_equal(order_g, order_o), (case, obj)
        assert nodes_g == nodes_o, (case, obj, nodes_g, nodes_o)
        assert 0 < max_stack <= 192


def test_invalid_descriptions_rejected(gpu_lib):
    import ctypes as C
    from psychopath_gb300 import abi
    s = sc.cornell()
    s.objects[0]["indices"] = s.objects[0]["indices"].copy()
    s.objects[0]["indices"][0, 0] = 10 ** 6  # index out of range
    with pytest.raises(gpu.PsyError) as e:
        gpu.host_build_info(s, 0)
    assert e.value.code == abi.PSY_E_INVALID


def test_gpu_bvh_needs_a_device(gpu_lib):
    """The host-only build entry point rejects GPU-built BVHs cleanly."""
    import ctypes as C
    from psychopath_gb300 import abi
    from . import scene_cases as sc
    sd = sc.cornell()
    desc = sd.desc()
    opts = abi.PsySceneOptions()
    opts.bvh_build = abi.PSY_BVH_GPU
    order = np.zeros(64, dtype=np.uint32)
    nc, ms = C.c_uint32(), C.c_uint32()
    rc = gpu_lib.psy_debug_host_build(C.byref(desc), C.byref(opts), 0, order.ctypes.data, C.byref(nc), C.byref(ms))
    assert rc == abi.PSY_E_UNSUPPORTED


def test_deep_scene_needs_the_large_stack(gpu_lib):
    """The deep test scene's worst-case stack exceeds 64 entries, so its GPU
    traces run the 192-entry kernels."""
    _, _, max_stack = gpu.host_build_info(sc.deep_stack(), 0)
    assert 64 < max_stack <= 192


@pytest.mark.parametrize("case", ["grid", "sphere", "motion", "deep"])
def test_threaded_bvh_build_equals_serial(gpu_lib, case):
    """Large subtrees of the host SAH build run on worker threads into their
    own arrays and are spliced in; the scene's BVH4 nodes and motion bounds
    must be byte-identical to a build on one thread."""
    from psychopath_gb300 import scenes
    if case == "grid":
        s, _, _ = scenes.grid_mesh(512, 256)  # 262,144 triangles: several threaded levels
    elif case == "sphere":
        s = sc.sphere_small(level=7)
    elif case == "motion":
        s = sc.motion_small(n=100, level=6)  # the deforming mesh: 81,920 triangles, 3 keys
    else:
        s = sc.deep_stack()
    a_nodes, a_ext = gpu.host_nodes(s)
    b_nodes, b_ext = gpu.host_nodes(s, serial=True)
    assert a_nodes.size > 0
    assert np.array_equal(a_nodes, b_nodes) and np.array_equal(a_ext, b_ext)


def _decode_fp16_nodes(raw32, raw16):
    """The f32 child boxes of every node and the boxes its FP16 copy decodes
    to, with the device's arithmetic: bound = fl32(corner + f16 offset) (PTX
    add.rn.f32.f16: the f16 converts exactly, the f32 sum rounds to nearest).
    Returns (lo32, hi32, lo16, hi16) of shape (nodes, 3, 4), the child counts
    and the meta words of the FP16 copies."""
    n = raw32.size // 128
    f32 = raw32.view(np.float32).reshape(n, 32)
    u32 = raw32.view(np.uint32).reshape(n, 32)
    lo32 = np.stack([f32[:, 0:4], f32[:, 8:12], f32[:, 16:20]], axis=1)
    hi32 = np.stack([f32[:, 4:8], f32[:, 12:16], f32[:, 20:24]], axis=1)
    count = u32[:, 30] >> 8
    h = raw16.reshape(n, 96)
    anchor = h[:, 0:16].copy().view(np.float32).reshape(n, 4)
    meta = h[:, 12:16].copy().view(np.uint32).reshape(n)
    ext = h[:, 32:38].copy().view(np.float16).reshape(n, 3).astype(np.float32)
    planes = h[:, 40:88].copy().view(np.float16).reshape(n, 6, 4).astype(np.float32)
    a = anchor[:, :3]
    top = (a + ext).astype(np.float32)
    lo16 = (a[:, :, None] + planes[:, 0::2, :]).astype(np.float32)
    hi16 = (top[:, :, None] + planes[:, 1::2, :]).astype(np.float32)
    return lo32, hi32, lo16, hi16, count, meta


@pytest.mark.parametrize("case", ["cornell", "ground_sphere", "grid"])
def test_fp16_nodes_contain_the_f32_boxes_and_keep_flat_faces_flat(gpu_lib, case):
    """Every FP16 node that the traversal reads (no f32 flag) decodes, with
    the device's own rounding, to child boxes that contain the f32 boxes,
    and a child that is flat on an axis (a floor, a wall) decodes exactly
    flat on that axis: a box a few f16 ulps thick around a ground plane
    holds the origins of every ray leaving the plane.  The ground-plane node
    of the sphere-on-a-ground scene keeps its FP16 copy."""
    from psychopath_gb300 import scenes
    if case == "cornell":
        s = sc.cornell()
    elif case == "ground_sphere":
        s = scenes.mesh_stress(64, 36, 1, level=5)
    else:
        s, _, _ = sc.grid_small()
    raw32, _ = gpu.host_nodes(s, bounds="fp16")
    raw16 = gpu.host_nodes_h(s)
    lo32, hi32, lo16, hi16, count, meta = _decode_fp16_nodes(raw32, raw16)
    used = (meta & 0x30000) == 0
    assert used.mean() > 0.95, used.mean()
    flat_seen = 0
    for i in np.nonzero(used)[0]:
        c = int(count[i])
        assert np.all(lo16[i, :, :c] <= lo32[i, :, :c]) and np.all(hi16[i, :, :c] >= hi32[i, :, :c]), i
        flat = lo32[i, :, :c] == hi32[i, :, :c]
        flat_seen += int(flat.sum())
        assert np.array_equal(lo16[i, :, :c][flat], lo32[i, :, :c][flat]), i
        assert np.array_equal(hi16[i, :, :c][flat], hi32[i, :, :c][flat]), i
    if case != "grid":
        assert flat_seen > 0
    if case == "ground_sphere":
        # the node whose children include the ground (y extent [0, 0]) and
        # the sphere reaching below it reads its FP16 copy
        both = [i for i in range(count.size)
                if np.any((lo32[i, 1, :count[i]] == 0) & (hi32[i, 1, :count[i]] == 0))
                and np.any(lo32[i, 1, :count[i]] < 0)]
        assert both and all(used[i] for i in both)
