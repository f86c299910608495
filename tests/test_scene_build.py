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
