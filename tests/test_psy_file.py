"""The .psy reader (psychopath_gb300/psy_file.py) against the reference
parser's rules: tokenizer (comments, escapes, idents with dots), leaf
formats (column-major Transform, colour spaces), polygon fan
triangulation, f32 parsing, errors with line numbers, and the older
example-scene layout.  CPU only; the scene it reads is written here in the
current layout."""
import math
import os

import numpy as np
import pytest

from psychopath_gb300 import abi, psy_file, scenes

# A small scene in the current layout: shaders and objects inside the root
# Assembly, shader bindings on instances, two camera keys, a 2-key instance
# transform, a pentagon, per-vertex normals, every light kind.
SCENE = r"""
# comment before the scene
Scene $Test.scene {
    Output { Path ["out/test.png"] }
    RenderSettings {
        Resolution [40 24]
        SamplesPerPixel [4]
        Seed [7]
    }
    Camera {
        Fov [39.449188]
        Fov [41.0]
        Transform [1 0 0 0  0 0 1 0  0 1 0 0  0.5 -8 2.5 1]
        Transform [1 0 0 0  0 0 1 0  0 1 0 0  0.6 -8 2.5 1]
    }
    World {
        BackgroundShader { Type [Color] Color [rec709, 0.05 0.06 0.07] }
        DistantDiskLight {
            Radius [0.0043633]
            Direction [0.3 0.2 -1.0]
            Color [blackbody, 5778 2.0]
        }
    }
    Assembly {
        SurfaceShader $White { Type [Lambert] Color [rec709, 0.7295 0.7355 0.729] }
        SurfaceShader $Gold {
            Type [GGX]
            Color [rec709, 0.9 0.6 0.2]
            Roughness [0.35]
            Fresnel [0.25]
        }
        SurfaceShader $Glow { Type [Emit] Color [color_temperature, 4000 3.0] }
        MeshSurface $floor.001 {
            Vertices [-3 -3 0  3 -3 0  3 3 0  -3 3 0]
            FaceVertCounts [4]
            FaceVertIndices [0 1 2 3]
        }
        MeshSurface $pent {   # a pentagon with normals: a fan of three triangles
            Vertices [0 0 1  1 0 1  1.3 1 1  0.5 1.6 1  -0.3 1 1]
            Normals [0 0 2  0 0.1 1  0 0 3  0.1 0 1  0 0 1]
            FaceVertCounts [5]
            FaceVertIndices [0 1 2 3 4]
        }
        SphereLight $bulb { Radius [0.25] Color [rec709, 20 20 20] }
        RectangleLight $panel { Dimensions [1.35 1.1] Color [rec709, 84.3 53.8 18.5] }
        Instance { Data [$floor.001] SurfaceShaderBind [$White] }
        Instance {
            Data [$pent]
            SurfaceShaderBind [$Gold]
            Transform [1 0 0 0  0 1 0 0  0 0 1 0  0 0 0 1]
            Transform [1 0 0 0  0 1 0 0  0 0 1 0  0.2 0 0 1]
        }
        Instance { Data [$pent] SurfaceShaderBind [$Glow] Transform [1 0 0 0  0 1 0 0  0 0 1 0  -2 0 -0.5 1] }
        Instance { Data [$bulb] Transform [1 0 0 0  0 1 0 0  0 0 1 0  0 0 -4 1] }
        Instance { Data [$panel] Transform [1 0 0 0  0 1 0 0  0 0 1 0  1 1 -5 1] }
    }
}
"""


def test_scene_structure():
    ps = psy_file.load_psy(SCENE, max_bounces=3)
    sd = ps.data
    assert ps.name == "$Test.scene" and ps.output_path == "out/test.png"
    assert (sd.width, sd.height, sd.spp, sd.seed, sd.max_bounces) == (40, 24, 4, 7, 3)
    assert [o["kind"] for o in sd.objects] == [abi.PSY_OBJ_MESH, abi.PSY_OBJ_MESH, abi.PSY_OBJ_SPHERE_LIGHT,
                                               abi.PSY_OBJ_RECT_LIGHT]
    assert [s.kind for s in sd.shaders] == [abi.PSY_SHADER_LAMBERT, abi.PSY_SHADER_GGX, abi.PSY_SHADER_EMIT]
    assert sd.shaders[1].roughness == np.float32(0.35) and sd.shaders[1].fresnel == np.float32(0.25)
    assert sd.shaders[2].color.kind == abi.PSY_COLOR_TEMPERATURE
    # quad and pentagon: fans from the first vertex (psy_mesh_surface.rs:95-110)
    assert sd.objects[0]["indices"].tolist() == [[0, 1, 2], [0, 2, 3]]
    assert sd.objects[1]["indices"].tolist() == [[0, 1, 2], [0, 2, 3], [0, 3, 4]]
    # normals normalised at parse time, in f32
    n = sd.objects[1]["normals"][0]
    assert n.dtype == np.float32 and np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-6)
    assert n[0].tolist() == [0.0, 0.0, 1.0]
    # instances: shader binding and transform keys; column-major 4x4 -> rows
    objs = [i[0] for i in sd.instances]
    shaders = [i[1] for i in sd.instances]
    assert objs == [0, 1, 1, 2, 3] and shaders == [0, 1, 2, -1, -1]
    assert len(sd.instances[0][2]) == 0 and len(sd.instances[1][2]) == 2
    assert sd.instances[1][2][1][0, 3] == np.float64(np.float32(0.2))
    assert sd.instances[2][2][0][:3, 3].tolist() == [-2.0, 0.0, -0.5]
    # camera: keys, f32 degrees -> radians as the reference computes it
    mats, fovs, ap, fd = sd.camera
    k = np.float32(np.float32(math.pi) / np.float32(180.0))
    assert fovs[0] == np.float32(np.float32(39.449188) * k)
    assert len(mats) == 2 and mats[0][:3].tolist() == [[1, 0, 0, 0.5], [0, 0, 1, -8], [0, 1, 0, 2.5]]
    # background and the distant light
    bg = scenes.rec709_e_to_xyz([0.05, 0.06, 0.07])
    assert [sd.background.v[i] for i in range(3)] == [float(x) for x in bg]
    assert sd.distant[0][0] == [np.float32(0.0043633)]
    assert sd.distant[0][2][0].kind == abi.PSY_COLOR_BLACKBODY
    sd.desc()  # builds the C description


def test_host_build_of_parsed_scene(gpu_lib):
    """The parsed scene goes through the library's host-side build (BVH,
    light tree) without a GPU."""
    from psychopath_gb300 import gpu
    sd = psy_file.load_psy(SCENE).data
    order, nodes, max_stack = gpu.host_build_info(sd, 1)
    assert sorted(order.tolist()) == [0, 1, 2] and nodes >= 1 and max_stack >= 1


def test_parse_f32_rounds_once():
    # 1 + 2^-24 is halfway between the f32 neighbours 1 and 1 + 2^-23; text
    # just above it must round up, text just below it down, text exactly on
    # it to even (1.0) -- rounding through f64 first gets the first two wrong
    assert psy_file.parse_f32("1.000000059604644775390625") == np.float32(1.0)
    assert psy_file.parse_f32("1.0000000596046447753906251") == np.nextafter(np.float32(1), np.float32(2))
    assert psy_file.parse_f32("1.0000000596046447753906249") == np.float32(1.0)
    assert psy_file.parse_f32("-0.5") == np.float32(-0.5)
    assert psy_file.parse_f32("3e-2") == np.float32(0.03)


def test_tokenizer_details():
    t = psy_file.parse_data_tree("A $a\\ b { B [x \\] y] # c\n C { } }  # end")
    a = t.children[0]
    assert a.type_name == "A" and a.ident == "$a\\ b"
    assert a.children[0].contents == "x \\] y" and a.children[1].type_name == "C"


@pytest.mark.parametrize("bad,msg", [
    ("Scene { Output { Path [\"x\"] }", "line 1"),                      # missing '}'
    ("Scene {\n Output { Path [x] }\n}", "quotes"),                      # unquoted path
    (SCENE.replace("[Lambert]", "[Velvet]"), "unknown SurfaceShader"),
    (SCENE.replace("Data [$bulb]", "Data [$nothing]"), "unknown data"),
    (SCENE.replace("FaceVertCounts [5]", "FaceVertCounts [2 3]"), "three vertices"),
    (SCENE.replace("Transform [1 0 0 0  0 1 0 0  0 0 1 0  0 0 -4 1]", "Transform [1 0 0]"), "16 numbers"),
])
def test_errors_name_the_line(bad, msg):
    with pytest.raises(psy_file.PsyFileError) as e:
        psy_file.load_psy(bad)
    assert msg in str(e.value)


# A checkout of the reference (its example_scenes/ directory), named by the
# PSY_REFERENCE_ROOT environment variable; the test is skipped without one.
REF = os.path.join(os.environ.get("PSY_REFERENCE_ROOT", ""), "example_scenes")


@pytest.mark.skipif(not os.environ.get("PSY_REFERENCE_ROOT") or not os.path.isdir(REF),
                    reason="PSY_REFERENCE_ROOT not set to a reference checkout")
@pytest.mark.parametrize("name,objects,instances,shaders,res", [
    ("cube.psy", 3, 3, 1, (960, 540)),
    ("cornell_box.psy", None, None, 3, (512, 512)),
])
def test_reference_example_scenes(name, objects, instances, shaders, res):
    """The reference's two example scenes (older layout: Scene-level Shaders
    and Objects sections, shader bound on the mesh) read with layout='auto';
    the current layout rejects them, as the reference's own parser does."""
    text = open(os.path.join(REF, name)).read()
    ps = psy_file.load_psy(text)
    sd = ps.data
    assert (sd.width, sd.height) == res and sd.spp == 16 and sd.seed == 1
    assert len(sd.shaders) == shaders
    if objects is not None:
        assert len(sd.objects) == objects and len(sd.instances) == instances
    assert all(i[1] >= 0 for i in sd.instances if sd.objects[i[0]]["kind"] == abi.PSY_OBJ_MESH)
    sd.desc()
    with pytest.raises(psy_file.PsyFileError):
        psy_file.load_psy(text, layout="current")
