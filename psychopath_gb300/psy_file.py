"""Reader for Psychopath's .psy scene files: parses a scene into a
`SceneData` (the flattened `PsySceneDesc` the C ABI consumes), following the
reference's parser:

  tokenizer / data tree     src/parse/data_tree.rs:22-44, 287-546
  Scene, RenderSettings,    src/parse/psy.rs:95-377 (parse_scene,
  Camera, World               parse_render_settings, parse_camera,
                              parse_world)
  Transform, Color leaves   src/parse/psy.rs:554-615 (parse_matrix,
                              parse_color)
  Assembly, Instance        src/parse/psy_assembly.rs:17-188
  MeshSurface               src/parse/psy_mesh_surface.rs:27-127
  Sphere / Rectangle /      src/parse/psy_light.rs
  DistantDisk lights
  SurfaceShader             src/parse/psy_surface_shader.rs

Numbers are read as f32 with correct rounding (the reference parses text
straight to f32), and everything the reference computes at parse time is
computed here in f32 with the same operation order: degrees to radians for
the field of view, normal normalisation, rec709 to XYZ.

Layout: the reference's parser reads shaders and objects inside the root
Assembly and binds shaders on instances.  Its two example scenes use an
older layout -- `Shaders {}` and `Objects {}` sections at Scene level and
`SurfaceShaderBind` on the mesh -- which that parser does not read;
`layout="auto"` accepts them by treating both sections as part of the root
assembly and applying a mesh's binding to its instances that have none.

Nested assemblies are flattened into the one-level description: every
instance of an object inside instanced assemblies becomes a root instance
whose transform keys combine those of its enclosing instances as the
tracer's TransformStack does at trace time, so geometry, transforms and
shaders are the reference's.  Two things differ from tracing the hierarchy:
instance ids are renumbered in depth-first order, and lights inside nested
assemblies join the root light tree, so light selection probabilities (not
the converged image) differ from the reference's per-assembly light trees.
"""
import math
import struct
from decimal import Decimal

import numpy as np

from . import abi, scenes


class PsyFileError(ValueError):
    """A .psy file the reader cannot turn into a scene (the reference's
    PsyParseError cases), with the line it refers to."""


# ---------------------------------------------------------------- data tree
class Node:
    """Internal node (children) or leaf (contents) of the data tree."""

    __slots__ = ("type_name", "ident", "children", "contents", "offset")

    def __init__(self, type_name, ident=None, children=None, contents=None, offset=0):
        self.type_name, self.ident, self.children, self.contents, self.offset = (
            type_name, ident, children, contents, offset)

    @property
    def is_leaf(self):
        return self.children is None

    def leaves(self, type_name):
        return [c for c in self.children or [] if c.is_leaf and c.type_name == type_name]

    def internals(self, type_name):
        return [c for c in self.children or [] if not c.is_leaf and c.type_name == type_name]

    def nodes(self, type_name):
        return [c for c in self.children or [] if c.type_name == type_name]


_WS = " \t\r\n"
_RESERVED = "{}[]$#\\"


def _is_ident_char(c):
    return c not in _WS and c not in _RESERVED


class _Tokens:
    def __init__(self, text):
        self.t = text
        self.i = 0

    def skip(self):
        t, n = self.t, len(self.t)
        while True:
            j = self.i
            while j < n and t[j] in _WS:
                j += 1
            if j < n and t[j] == "#":
                while j < n and t[j] not in "\r\n":
                    j += 1
            if j == self.i:
                return
            self.i = j

    def next(self):
        """(kind, value, offset) with kind in '{', '}', '[', ']', 'type',
        'ident', 'end', 'unknown'."""
        self.skip()
        t, i = self.t, self.i
        if i >= len(t):
            return ("end", None, i)
        c = t[i]
        if c in "{}[]":
            self.i = i + 1
            return (c, c, i)
        if c == "$":
            j = i + 1
            esc = False
            while j < len(t):
                ch = t[j]
                if esc:
                    esc = False
                elif ch == "\\":
                    esc = True
                elif not _is_ident_char(ch):
                    break
                j += 1
            self.i = j
            return ("ident", t[i:j], i)
        if _is_ident_char(c):
            j = i
            while j < len(t) and _is_ident_char(t[j]):
                j += 1
            self.i = j
            return ("type", t[i:j], i)
        return ("unknown", c, i)

    def leaf_contents(self):
        t, i = self.t, self.i
        j = i
        esc = False
        while j < len(t):
            ch = t[j]
            if esc:
                esc = False
            elif ch == "\\":
                esc = True
            elif ch == "]":
                break
            j += 1
        self.i = j
        return t[i:j]


def _line(text, offset):
    return text.count("\n", 0, offset) + 1


def parse_data_tree(text):
    """The whole file as a ROOT node (src/parse/data_tree.rs:22-44)."""
    tk = _Tokens(text)

    def err(msg, off):
        raise PsyFileError("line %d: %s" % (_line(text, off), msg))

    def node():
        save = tk.i
        kind, val, off = tk.next()
        if kind != "type":
            tk.i = save
            return None
        k2, v2, o2 = tk.next()
        ident = None
        if k2 == "ident":
            ident = v2
            k2, v2, o2 = tk.next()
            if k2 != "{":
                err("missing '{' after %s %s" % (val, ident), o2)
        if k2 == "{":
            children = []
            while True:
                c = node()
                if c is None:
                    break
                children.append(c)
            k3, _, o3 = tk.next()
            if k3 != "}":
                err("missing '}' closing %s" % val, o3)
            return Node(val, ident, children, None, off)
        if k2 == "[":
            contents = tk.leaf_contents()
            k3, _, o3 = tk.next()
            if k3 != "]":
                err("missing ']' closing %s" % val, o3)
            return Node(val, None, None, contents, off)
        err("expected '{' or '[' after %s" % val, o2)

    items = []
    while True:
        n = node()
        if n is None:
            break
        items.append(n)
    tk.skip()
    if tk.i != len(text):
        err("failed to parse the entire file", tk.i)
    return Node("ROOT", None, items, None, 0)


# ---------------------------------------------------------------- numbers
def parse_f32(s):
    """Decimal text -> nearest f32 (ties to even), as a direct text-to-f32
    conversion does.  Going through f64 first can round twice; that only
    happens when the f64 value sits exactly halfway between two f32s, and
    then the exact decimal value decides."""
    x = float(s)
    f = np.float32(x)
    if not np.isfinite(f) or float(f) == x:
        return f
    other = np.nextafter(f, np.float32(np.inf) if x > float(f) else np.float32(-np.inf), dtype=np.float32)
    mid = (float(f) + float(other)) / 2.0  # exact in f64
    if x != mid:
        return f
    d = Decimal(s.strip())
    lo, hi = (f, other) if float(f) < float(other) else (other, f)
    dm = Decimal(float(lo)) + (Decimal(float(hi)) - Decimal(float(lo))) / 2
    if d < dm:
        return lo
    if d > dm:
        return hi
    even = lo if (struct.unpack("<I", struct.pack("<f", float(lo)))[0] & 1) == 0 else hi
    return even


def _floats(contents, what, node, text, count=None):
    toks = contents.split()
    try:
        vals = [parse_f32(t) for t in toks]
    except ValueError:
        raise PsyFileError("line %d: %s must be decimal numbers" % (_line(text, node.offset), what))
    if count is not None and len(vals) != count:
        raise PsyFileError("line %d: %s needs %d numbers, found %d" % (_line(text, node.offset), what, count,
                                                                        len(vals)))
    return vals


def _uints(contents, what, node, text):
    try:
        vals = [int(t) for t in contents.split()]
    except ValueError:
        raise PsyFileError("line %d: %s must be integers" % (_line(text, node.offset), what))
    if any(v < 0 for v in vals):
        raise PsyFileError("line %d: %s must be non-negative" % (_line(text, node.offset), what))
    return vals


def parse_matrix(contents, node, text):
    """16 numbers, column-major 4x4; the last row is dropped
    (src/parse/psy.rs:554-568).  Returns the 4x4 (f64 holding f32 values)
    in the row layout `SceneData` takes."""
    n = _floats(contents, "Transform", node, text, 16)
    m = np.zeros((4, 4), dtype=np.float64)
    for r in range(3):
        for c in range(4):
            m[r, c] = float(n[4 * c + r])
    m[3, 3] = 1.0
    return m


def parse_color(contents, node, text):
    """'rec709, r g b' / 'blackbody, K factor' / 'color_temperature, K factor'
    (src/parse/psy.rs:578-615)."""
    items = [s.strip() for s in contents.split(",")]
    if len(items) != 2:
        raise PsyFileError("line %d: colour must be '<space>, <values>'" % _line(text, node.offset))
    kind, vals = items
    if kind == "rec709":
        v = _floats(vals, "rec709 colour", node, text, 3)
        return scenes.xyz_color(np.array(v, dtype=np.float32))
    if kind in ("blackbody", "color_temperature"):
        v = _floats(vals, kind + " colour", node, text, 2)
        c = abi.PsyColor()
        c.kind = abi.PSY_COLOR_BLACKBODY if kind == "blackbody" else abi.PSY_COLOR_TEMPERATURE
        c.v[0], c.v[1], c.v[2] = float(v[0]), float(v[1]), 0.0
        return c
    raise PsyFileError("line %d: unknown colour space '%s'" % (_line(text, node.offset), kind))


def _normalized_f32(v):
    """glam normalize in f32: v * (1 / sqrt((x*x + y*y) + z*z))."""
    v = np.asarray(v, dtype=np.float32)
    d = (v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1]) + v[..., 2] * v[..., 2]
    r = np.float32(1.0) / np.sqrt(d)
    return v * r[..., None]


# ---------------------------------------------------------------- scene
def _one(node, type_name, text):
    found = node.nodes(type_name)
    if len(found) != 1:
        raise PsyFileError("line %d: %s needs exactly one %s section, found %d" % (
            _line(text, node.offset), node.type_name, type_name, len(found)))
    return found[0]


def _leaf1(node, type_name, text, required=True):
    found = node.leaves(type_name)
    if not found:
        if required:
            raise PsyFileError("line %d: %s is missing %s" % (_line(text, node.offset), node.type_name, type_name))
        return None
    return found[0]


def _render_settings(node, text):
    res = _leaf1(node, "Resolution", text)
    spp = _leaf1(node, "SamplesPerPixel", text)
    r = _uints(res.contents, "Resolution", res, text)
    s = _uints(spp.contents, "SamplesPerPixel", spp, text)
    if len(r) != 2 or len(s) != 1:
        raise PsyFileError("line %d: Resolution is '[width height]', SamplesPerPixel '[n]'" % _line(text, node.offset))
    seed = 0
    sd = _leaf1(node, "Seed", text, required=False)
    if sd is not None:
        v = _uints(sd.contents, "Seed", sd, text)
        if len(v) != 1:
            raise PsyFileError("line %d: Seed is '[n]'" % _line(text, sd.offset))
        seed = v[0]
    return r[0], r[1], s[0], seed


def _camera(node, text):
    mats, fovs, fds, ars = [], [], [], []
    deg = np.float32(np.float32(math.pi) / np.float32(180.0))
    for c in node.children:
        if not c.is_leaf:
            continue
        if c.type_name == "Fov":
            fovs.append(np.float32(_floats(c.contents, "Fov", c, text, 1)[0] * deg))
        elif c.type_name == "FocalDistance":
            fds.append(_floats(c.contents, "FocalDistance", c, text, 1)[0])
        elif c.type_name == "ApertureRadius":
            ars.append(_floats(c.contents, "ApertureRadius", c, text, 1)[0])
        elif c.type_name == "Transform":
            mats.append(parse_matrix(c.contents, c, text))
    if not mats or not fovs:
        raise PsyFileError("line %d: Camera needs at least a Fov and a Transform" % _line(text, node.offset))
    return mats, fovs, ars, fds


def _shader(node, text):
    t = _leaf1(node, "Type", text).contents.strip()
    col = _leaf1(node, "Color", text)
    color = parse_color(col.contents, col, text)
    s = abi.PsyShaderDesc()
    s.color = color
    if t == "Lambert":
        s.kind = abi.PSY_SHADER_LAMBERT
    elif t == "Emit":
        s.kind = abi.PSY_SHADER_EMIT
    elif t == "GGX":
        s.kind = abi.PSY_SHADER_GGX
        r = _leaf1(node, "Roughness", text)
        f = _leaf1(node, "Fresnel", text)
        s.roughness = float(_floats(r.contents, "Roughness", r, text, 1)[0])
        s.fresnel = float(_floats(f.contents, "Fresnel", f, text, 1)[0])
    else:
        raise PsyFileError("line %d: unknown SurfaceShader type '%s'" % (_line(text, node.offset), t))
    return s


def _mesh(node, text):
    verts = []
    for lf in node.leaves("Vertices"):
        v = _floats(lf.contents, "Vertices", lf, text)
        verts.append(np.array(v[: len(v) // 3 * 3], dtype=np.float32).reshape(-1, 3))
    if not verts:
        raise PsyFileError("line %d: MeshSurface has no Vertices" % _line(text, node.offset))
    nv = verts[0].shape[0]
    if any(v.shape[0] != nv for v in verts):
        raise PsyFileError("line %d: every Vertices time sample needs the same count" % _line(text, node.offset))
    normals = []
    for lf in node.leaves("Normals"):
        n = _floats(lf.contents, "Normals", lf, text)
        normals.append(_normalized_f32(np.array(n[: len(n) // 3 * 3], dtype=np.float32).reshape(-1, 3)))
    if normals and (len(normals) != len(verts) or any(n.shape[0] != nv for n in normals)):
        raise PsyFileError("line %d: Normals must match Vertices in time samples and count" % _line(text, node.offset))
    fvc = node.leaves("FaceVertCounts")
    fvi = node.leaves("FaceVertIndices")
    counts = _uints(fvc[0].contents, "FaceVertCounts", fvc[0], text) if fvc else []
    idx = _uints(fvi[0].contents, "FaceVertIndices", fvi[0], text) if fvi else []
    tris = []
    ii = 0
    for fc in counts:
        if fc < 3:
            raise PsyFileError("line %d: polygons need at least three vertices" % _line(text, node.offset))
        if ii + fc > len(idx):
            raise PsyFileError("line %d: FaceVertIndices is shorter than FaceVertCounts says" % _line(text, node.offset))
        for vi in range(fc - 2):  # fan from the polygon's first vertex
            tris.append((idx[ii], idx[ii + vi + 1], idx[ii + vi + 2]))
        ii += fc
    tris = np.array(tris, dtype=np.uint32).reshape(-1, 3)
    if tris.size and int(tris.max()) >= nv:
        raise PsyFileError("line %d: face vertex index out of range" % _line(text, node.offset))
    return np.stack(verts), (np.stack(normals) if normals else None), tris


def _light_keys(node, text, leaf, count):
    out = []
    for lf in node.leaves(leaf):
        out.append(_floats(lf.contents, leaf, lf, text, count))
    return out


def _colors(node, text):
    return [parse_color(lf.contents, lf, text) for lf in node.leaves("Color")]


class PsyScene:
    """A parsed .psy scene: `data` (SceneData) plus the names the file used."""

    def __init__(self, data, name, output_path, object_names, shader_names):
        self.data, self.name, self.output_path = data, name, output_path
        self.object_names, self.shader_names = object_names, shader_names


# ---------------------------------------------------------------- assemblies
class _Assembly:
    """One Assembly section: its shaders, objects and sub-assemblies by name
    (names are scoped to the assembly, as AssemblyBuilder's maps are,
    src/scene/assembly.rs:150-300) and its Instance nodes."""

    def __init__(self):
        self.shaders, self.objects, self.binds, self.assemblies, self.instances = {}, {}, {}, {}, []
        self.defined_at = {}  # object / assembly name -> position of its definition
        self.shader_at = {}   # shader name -> position of its definition


def _parse_assembly(content, sd, text, layout):
    """Reads the children of an Assembly (parse_assembly,
    src/parse/psy_assembly.rs:17-188): shaders, meshes and lights are added
    to the scene once; sub-assemblies are read into their own scopes and
    instanced later."""
    a = _Assembly()
    for pos, c in enumerate(content):
        t = c.type_name
        # objects and assemblies share one name space, shaders have their
        # own; a name defined twice is rejected as AssemblyBuilder does
        # (add_object / add_assembly / add_surface_shader, src/scene/assembly.rs:184-221)
        if t in ("MeshSurface", "SphereLight", "RectangleLight", "Assembly") and c.ident is not None:
            if c.ident in a.defined_at:
                raise PsyFileError("line %d: '%s' is already defined in this assembly" % (_line(text, c.offset), c.ident))
            a.defined_at[c.ident] = pos
        if t == "SurfaceShader":
            if c.is_leaf or c.ident is None:
                raise PsyFileError("line %d: a SurfaceShader needs a $name and a body" % _line(text, c.offset))
            if c.ident in a.shaders:
                raise PsyFileError("line %d: shader '%s' is already defined in this assembly" % (_line(text, c.offset), c.ident))
            a.shader_at[c.ident] = pos
            a.shaders[c.ident] = sd.add_shader(0)
            sd.shaders[a.shaders[c.ident]] = _shader(c, text)
        elif t == "MeshSurface":
            if c.is_leaf or c.ident is None:
                raise PsyFileError("line %d: a MeshSurface needs a $name and a body" % _line(text, c.offset))
            v, n, tr = _mesh(c, text)
            a.objects[c.ident] = sd.add_mesh(v, tr, n)
            if layout == "auto" and c.leaves("SurfaceShaderBind"):
                # older layout: the shader is bound on the object
                a.binds[c.ident] = c.leaves("SurfaceShaderBind")[0]
        elif t == "SphereLight":
            radii = [k[0] for k in _light_keys(c, text, "Radius", 1)]
            a.objects[c.ident] = sd.add_sphere_light(radii, _colors(c, text))
        elif t == "RectangleLight":
            dims = _light_keys(c, text, "Dimensions", 2)
            a.objects[c.ident] = sd.add_rect_light(dims, _colors(c, text))
        elif t == "Assembly":
            if c.is_leaf or c.ident is None:
                raise PsyFileError("line %d: an Assembly needs a $name and a body" % _line(text, c.offset))
            a.assemblies[c.ident] = _parse_assembly(list(c.children), sd, text, layout)
        elif t == "Instance":
            a.instances.append((pos, c))
    return a


def _instantiate(a, parent_keys, sd, text):
    """Adds the instances of assembly `a` to the scene with the transform
    keys of its enclosing instances combined as the tracer's TransformStack
    does at trace time (src/tracer.rs:96-110, src/transform_stack.rs:33-62):
    an instance of an object gets the combined keys; an instance of a
    sub-assembly pushes its keys and instances that assembly's content."""
    for pos, c in a.instances:
        data = c.leaves("Data")
        if len(data) != 1:
            raise PsyFileError("line %d: an Instance needs exactly one Data" % _line(text, c.offset))
        name = data[0].contents.strip()
        # the reference adds an instance when it reads it, so its data must be
        # defined above it in the same assembly (src/parse/psy_assembly.rs:76-89)
        if (name not in a.objects and name not in a.assemblies) or a.defined_at.get(name, pos) > pos:
            raise PsyFileError("line %d: Instance of unknown data '%s'" % (_line(text, data[0].offset), name))
        bind = c.leaves("SurfaceShaderBind") or ([a.binds[name]] if name in a.binds else [])
        shader = -1
        if bind:
            sname = bind[0].contents.strip()
            # add_instance looks the shader up when it reads the Instance
            # (src/scene/assembly.rs:250-255): it must be defined above it
            if sname not in a.shaders or a.shader_at.get(sname, pos) > pos:
                raise PsyFileError("line %d: unknown shader '%s'" % (_line(text, bind[0].offset), sname))
            shader = a.shaders[sname]
        keys = merge_transform_keys(parent_keys, [parse_matrix(t.contents, t, text) for t in c.leaves("Transform")])
        if name in a.objects:
            sd.add_instance(a.objects[name], shader, keys)
        else:
            # the tracer ignores a shader bound on an assembly instance; the
            # objects inside use their own assembly's bindings
            _instantiate(a.assemblies[name], keys, sd, text)


# ---------------------------------------------------------------- transform keys
def _f32_3x4(m):
    return np.asarray(m, dtype=np.float64)[:3, :4].astype(np.float32)


def _to4(o):
    m = np.zeros((4, 4), dtype=np.float64)
    m[:3, :4] = o
    m[3, 3] = 1.0
    return m


def xf_mul(a, b):
    """`a * b` for the reference's Transform (sub_crates/math3d/src/transform.rs:89-96,
    glam's Affine3A product with b applied after a): rows of b times
    columns of a, each sum in f32 left to right; 4x4 row-layout matrices."""
    L, R = _f32_3x4(b), _f32_3x4(a)
    o = np.zeros((3, 4), dtype=np.float32)
    for r in range(3):
        for c in range(3):
            o[r, c] = (L[r, 0] * R[0, c] + L[r, 1] * R[1, c]) + L[r, 2] * R[2, c]
        o[r, 3] = ((L[r, 0] * R[0, 3] + L[r, 1] * R[1, 3]) + L[r, 2] * R[2, 3]) + L[r, 3]
    return _to4(o)


def xf_lerp(a, b, alpha):
    """Transform lerp (src/lerp.rs:109-113): a * (1 - alpha) + b * alpha per element, f32."""
    alpha = np.float32(alpha)
    ia = np.float32(1.0) - alpha
    return _to4(_f32_3x4(a) * ia + _f32_3x4(b) * alpha)


def lerp_slice_keys(keys, alpha):
    """lerp_slice (src/lerp.rs:20-35) over transform keys, f32."""
    alpha = np.float32(alpha)
    if len(keys) == 1 or alpha == np.float32(1.0):
        return keys[-1]
    tmp = alpha * np.float32(len(keys) - 1)
    i1 = int(tmp)
    return xf_lerp(keys[i1], keys[i1 + 1], tmp - np.float32(i1))


def merge_transform_keys(parent, child):
    """TransformStack::push (src/transform_stack.rs:33-62) with
    merge_slices_to (src/algorithm.rs:266-305): the enclosing keys times the
    instance's keys, the shorter list lerped at the longer one's key times
    i / (n - 1).  An empty side leaves the other unchanged."""
    if not parent:
        return list(child)
    if not child:
        return list(parent)
    if len(parent) == len(child):
        return [xf_mul(p, c) for p, c in zip(parent, child)]
    if len(parent) > len(child):
        s = np.float32(len(parent) - 1)
        return [xf_mul(p, lerp_slice_keys(child, np.float32(i) / s)) for i, p in enumerate(parent)]
    s = np.float32(len(child) - 1)
    return [xf_mul(lerp_slice_keys(parent, np.float32(i) / s), c) for i, c in enumerate(child)]


def load_psy(text, scene_index=0, layout="auto", max_bounces=2):
    """Parse .psy text and return the scene_index-th Scene as a PsyScene.
    max_bounces is the bounce limit of the light paths (the reference
    renderer hard-codes 2, src/renderer.rs:599)."""
    root = parse_data_tree(text)
    sc = root.internals("Scene")
    if scene_index >= len(sc):
        raise PsyFileError("file has %d Scene sections" % len(sc))
    scene = sc[scene_index]
    out = _one(scene, "Output", text)
    path_leaf = _leaf1(out, "Path", text)
    p = path_leaf.contents.strip()
    if len(p) < 2 or p[0] != '"' or not p.endswith('"'):
        raise PsyFileError("line %d: file paths must be surrounded by quotes" % _line(text, path_leaf.offset))
    w, h, spp, seed = _render_settings(_one(scene, "RenderSettings", text), text)
    mats, fovs, ars, fds = _camera(_one(scene, "Camera", text), text)
    world = _one(scene, "World", text)
    asm = _one(scene, "Assembly", text)

    sd = scenes.SceneData(w, h, spp, seed=seed, max_bounces=max_bounces)
    sd.set_camera(mats, [], ars, fds, fovs_rad=fovs)
    bgs = _one(world, "BackgroundShader", text)
    bt = _leaf1(bgs, "Type", text).contents.strip()
    if bt != "Color":
        raise PsyFileError("line %d: unknown BackgroundShader type '%s'" % (_line(text, bgs.offset), bt))
    bc = _leaf1(bgs, "Color", text)
    sd.background = parse_color(bc.contents, bc, text)
    for dl in world.internals("DistantDiskLight"):
        radii = [k[0] for k in _light_keys(dl, text, "Radius", 1)]
        dirs = _light_keys(dl, text, "Direction", 3)
        cols = _colors(dl, text)
        if not radii or not dirs or not cols:
            raise PsyFileError("line %d: DistantDiskLight needs Radius, Direction and Color" % _line(text, dl.offset))
        sd.add_distant_light(radii, np.array(dirs, dtype=np.float32), cols)

    # root assembly content, plus the Scene-level Shaders / Objects sections
    # of the older layout
    content = list(asm.children)
    if layout == "auto":
        for sec in ("Shaders", "Objects"):
            for s in scene.internals(sec):
                content = list(s.children) + content
    elif layout != "current":
        raise ValueError("layout is 'auto' or 'current'")
    root = _parse_assembly(content, sd, text, layout)
    _instantiate(root, [], sd, text)
    return PsyScene(sd, scene.ident, p[1:-1], root.objects, root.shaders)


def load_psy_file(path, **kw):
    with open(path, "r", encoding="utf-8") as f:
        return load_psy(f.read(), **kw)
