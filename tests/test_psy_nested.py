"""Nested assemblies in the .psy reader: instances of objects inside
instanced sub-assemblies become root instances whose transform keys combine
their enclosing instances' keys as the tracer's TransformStack does
(src/transform_stack.rs:33-62 with merge_slices_to, src/algorithm.rs:266-305).
The key arithmetic is checked bit for bit against the oracle's Transform
multiply and lerp (pinned by the reference's own unit tests), names are
scoped per assembly as AssemblyBuilder's maps are.  CPU only."""
import ctypes as C

import numpy as np
import pytest

from psychopath_gb300 import psy_file

F12 = C.c_float * 12


def _o_mul(L, a, b):
    out = F12()
    L.psyo_xf_mul(F12(*a), F12(*b), out)
    return np.array(list(out), dtype=np.float32)


def _o_lerp(L, a, b, t):
    out = F12()
    L.psyo_xf_lerp(F12(*a), F12(*b), C.c_float(t), out)
    return np.array(list(out), dtype=np.float32)


def _o_lerp_slice(L, keys, alpha):
    alpha = np.float32(alpha)
    if len(keys) == 1 or alpha == np.float32(1.0):
        return keys[-1]
    tmp = alpha * np.float32(len(keys) - 1)
    i1 = int(tmp)
    return _o_lerp(L, keys[i1], keys[i1 + 1], float(tmp - np.float32(i1)))


def _o_merge(L, parent, child):
    """merge_slices_to over 12-float keys with the oracle's primitives."""
    if not parent:
        return list(child)
    if not child:
        return list(parent)
    if len(parent) == len(child):
        return [_o_mul(L, p, c) for p, c in zip(parent, child)]
    if len(parent) > len(child):
        s = np.float32(len(parent) - 1)
        return [_o_mul(L, p, _o_lerp_slice(L, child, np.float32(i) / s)) for i, p in enumerate(parent)]
    s = np.float32(len(child) - 1)
    return [_o_mul(L, _o_lerp_slice(L, parent, np.float32(i) / s), c) for i, c in enumerate(child)]


def _m4(v12):
    m = np.zeros((4, 4))
    m[:3, :4] = np.asarray(v12, dtype=np.float32).reshape(3, 4)
    m[3, 3] = 1.0
    return m


def _v12(m4):
    return np.asarray(m4, dtype=np.float64)[:3, :4].astype(np.float32).reshape(-1)


def test_key_merge_matches_oracle_primitives(oracle_lib):
    rng = np.random.default_rng(21)
    for n_parent, n_child in [(1, 1), (2, 2), (3, 1), (1, 4), (2, 5), (4, 3), (0, 2), (3, 0)]:
        parent = [rng.normal(size=12).astype(np.float32) for _ in range(n_parent)]
        child = [rng.normal(size=12).astype(np.float32) for _ in range(n_child)]
        got = psy_file.merge_transform_keys([_m4(p) for p in parent], [_m4(c) for c in child])
        want = _o_merge(oracle_lib, parent, child)
        assert len(got) == len(want) == max(n_parent, n_child)
        for g, w in zip(got, want):
            assert _v12(g).tobytes() == np.asarray(w, dtype=np.float32).tobytes()


NESTED = r"""
Scene $nested {
    Output { Path ["out/nested.png"] }
    RenderSettings { Resolution [16 16] SamplesPerPixel [1] Seed [1] }
    Camera { Fov [40] Transform [1 0 0 0  0 1 0 0  0 0 1 0  0 0 -5 1] }
    World { BackgroundShader { Type [Color] Color [rec709, 0.1 0.1 0.1] } }
    Assembly {
        SurfaceShader $Red { Type [Lambert] Color [rec709, 0.8 0.1 0.1] }
        MeshSurface $tri { Vertices [0 0 0  1 0 0  0 1 0] FaceVertCounts [3] FaceVertIndices [0 1 2] }
        Assembly $cluster {
            SurfaceShader $Red { Type [Lambert] Color [rec709, 0.1 0.8 0.1] }
            MeshSurface $quad { Vertices [0 0 0  1 0 0  1 1 0  0 1 0] FaceVertCounts [4] FaceVertIndices [0 1 2 3] }
            SphereLight $bulb { Radius [0.1] Color [rec709, 5 5 5] }
            Assembly $pair {
                MeshSurface $tri { Vertices [0 0 0  2 0 0  0 2 0] FaceVertCounts [3] FaceVertIndices [0 1 2] }
                Instance { Data [$tri] Transform [1 0 0 0  0 1 0 0  0 0 1 0  0.5 0 0 1] }
                Instance { Data [$tri] }
            }
            Instance { Data [$quad] SurfaceShaderBind [$Red]
                       Transform [1 0 0 0  0 1 0 0  0 0 1 0  0 0 1 1]
                       Transform [1 0 0 0  0 1 0 0  0 0 1 0  0 0 2 1]
                       Transform [1 0 0 0  0 1 0 0  0 0 1 0  0 0 3 1] }
            Instance { Data [$bulb] Transform [1 0 0 0  0 1 0 0  0 0 1 0  0 3 0 1] }
            Instance { Data [$pair] Transform [0 1 0 0  -1 0 0 0  0 0 1 0  0 0 0 1] }
        }
        Instance { Data [$tri] SurfaceShaderBind [$Red] }
        Instance { Data [$cluster] SurfaceShaderBind [$Red]
                   Transform [1 0 0 0  0 1 0 0  0 0 1 0  2 0 0 1]
                   Transform [2 0 0 0  0 2 0 0  0 0 2 0  2 0 0 1] }
        Instance { Data [$cluster] }
    }
}
"""


def _key(vals16):
    return psy_file.parse_matrix(" ".join(str(v) for v in vals16), None, "")


def test_nested_assemblies_flatten():
    ps = psy_file.load_psy(NESTED)
    sd = ps.data
    # root: tri; cluster x2, each = quad, bulb, pair(tri, tri)
    assert len(sd.instances) == 1 + 2 * 4
    objs = [o["kind"] for o in sd.objects]
    assert len(objs) == 4  # root tri, cluster quad, cluster bulb, pair tri (each added once)
    # shader scopes: the root's $Red on the root tri, the cluster's own $Red on
    # the quad; the cluster instance's binding is ignored, pair's tris have none
    red_root, red_cluster = ps.shader_names["$Red"], 1
    assert sd.instances[0][1] == red_root
    quad_a = sd.instances[1]
    assert quad_a[1] == red_cluster != red_root
    assert sd.instances[3][1] == -1 and sd.instances[4][1] == -1
    # keys: cluster instance (2 keys) x quad (3 keys) -> 3 merged keys
    c1 = [_key([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 2, 0, 0, 1]), _key([2, 0, 0, 0, 0, 2, 0, 0, 0, 0, 2, 0, 2, 0, 0, 1])]
    q = [_key([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, z, 1]) for z in (1, 2, 3)]
    want = psy_file.merge_transform_keys(c1, q)
    assert len(quad_a[2]) == 3
    for g, w in zip(quad_a[2], want):
        assert np.array_equal(g, w)
    # the pair's second tri has no keys of its own: cluster x pair
    rot = [_key([0, 1, 0, 0, -1, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1])]
    want_pair = psy_file.merge_transform_keys(c1, rot)
    assert all(np.array_equal(g, w) for g, w in zip(sd.instances[4][2], want_pair))
    # the second cluster instance has no keys: its contents keep their own
    assert len(sd.instances[5][2]) == 3 and np.array_equal(sd.instances[5][2][1], q[1])
    assert len(sd.instances[8][2]) == 1 and np.array_equal(sd.instances[8][2][0], rot[0])
    # merged key counts: the longer of the enclosing and the own keys
    assert [len(k) for _, _, k in sd.instances] == [0, 3, 2, 2, 2, 3, 1, 1, 1]
    sd.desc()


_LATE = NESTED.replace(
    "        Instance { Data [$tri] SurfaceShaderBind [$Red] }\n",
    "").replace(
    "        SurfaceShader $Red { Type [Lambert] Color [rec709, 0.8 0.1 0.1] }\n        MeshSurface $tri",
    "        SurfaceShader $Red { Type [Lambert] Color [rec709, 0.8 0.1 0.1] }\n"
    "        Instance { Data [$tri] SurfaceShaderBind [$Red] }\n        MeshSurface $tri")


# a shader bound by an Instance above the shader's definition
_LATE_SHADER = NESTED.replace(
    "        SurfaceShader $Red { Type [Lambert] Color [rec709, 0.8 0.1 0.1] }\n        MeshSurface $tri",
    "        MeshSurface $tri").replace(
    "        Instance { Data [$tri] SurfaceShaderBind [$Red] }\n",
    "        Instance { Data [$tri] SurfaceShaderBind [$Red] }\n"
    "        SurfaceShader $Red { Type [Lambert] Color [rec709, 0.8 0.1 0.1] }\n")
# a second object of the same name after an Instance of the first
_REDEFINED = NESTED.replace(
    "        Instance { Data [$tri] SurfaceShaderBind [$Red] }\n",
    "        Instance { Data [$tri] SurfaceShaderBind [$Red] }\n"
    "        MeshSurface $tri { Vertices [0 0 0  3 0 0  0 3 0] FaceVertCounts [3] FaceVertIndices [0 1 2] }\n")
_REDEFINED_SHADER = NESTED.replace(
    "        MeshSurface $tri { Vertices [0 0 0  1 0 0",
    "        SurfaceShader $Red { Type [Lambert] Color [rec709, 0.2 0.2 0.2] }\n"
    "        MeshSurface $tri { Vertices [0 0 0  1 0 0")


def test_mutated_scenes_differ_from_nested():
    for t in (_LATE, _LATE_SHADER, _REDEFINED, _REDEFINED_SHADER):
        assert t != NESTED


@pytest.mark.parametrize("bad,msg", [
    (NESTED.replace("Data [$pair]", "Data [$nothere]"), "unknown data"),
    (_LATE, "unknown data"),  # instanced above its definition, which the reference rejects
    (_LATE_SHADER, "unknown shader"),  # bound above the shader's definition (src/scene/assembly.rs:250-255)
    (_REDEFINED, "already defined"),  # AssemblyBuilder::add_object rejects a used name
    (_REDEFINED_SHADER, "already defined"),  # add_surface_shader rejects a used name
    (NESTED.replace("Instance { Data [$tri] SurfaceShaderBind [$Red] }",
                    "Instance { Data [$quad] }"), "unknown data"),  # $quad is scoped to $cluster
])
def test_nested_scoping_errors(bad, msg):
    with pytest.raises(psy_file.PsyFileError) as e:
        psy_file.load_psy(bad)
    assert msg in str(e.value)


def test_flattened_nested_scene_builds_and_renders_on_cpu(oracle_lib, gpu_lib):
    """The flattened description is an ordinary scene: the library's host-side
    build accepts it and the oracle renders it to a finite image."""
    from oracle.runner import OracleScene
    from psychopath_gb300 import gpu
    sd = psy_file.load_psy(NESTED).data
    _, nodes, max_stack = gpu.host_build_info(sd, 1)
    assert nodes >= 1 and max_stack >= 1
    img, _ = OracleScene(sd).render(threads=2)
    assert img.shape == (16, 16, 3) and np.isfinite(img).all() and img.max() > 0
