"""Scene descriptions for the tracing path.

`SceneData` owns numpy arrays for meshes, lights, instances, camera and
render settings and produces the `PsySceneDesc` the C ABI consumes -- the
flattened form of the reference's `Scene` (the Rust host fills the same
struct from its .psy parser).  The procedural builders below produce the
synthetic workloads the benchmarks run on (all seeded, nothing downloaded):

  cornell_box()        Cornell box, 5 wall quads + 2 rotated boxes, 0.25x0.25
                       rectangle light, Lambert albedos; 512x512x16, 4 bounces
  mesh_stress()        noise-displaced icosphere (level 8, 1,310,720 tris) on a
                       2-tri ground, sphere light r=0.1 + 0.5 deg sun, GGX;
                       1920x1080x64, 6 bounces
  motion_instances()   2,000 motion-blurred instances of a 20,480-tri displaced
                       sphere, one deforming mesh, 64 sphere lights;
                       1280x720x32
  grid_mesh()          2048x1024-quad (4,194,304 tri) displaced grid, for the
                       traversal microbenchmark, with coherent / incoherent
                       ray sets
"""
import ctypes as C
import math

import numpy as np

from . import abi


# ---------------------------------------------------------------- colour
def _rgb_to_xyz_matrix(r, g, b, w):
    """ACES CTL RGBtoXYZ (the reference's sub_crates/color/build.rs), in f64,
    rounded to 10 decimals as the generated Rust source is, then to f32."""
    Y = 1.0
    X = w[0] * Y / w[1]
    Z = (1.0 - w[0] - w[1]) * Y / w[1]
    d = r[0] * (b[1] - g[1]) + b[0] * (g[1] - r[1]) + g[0] * (r[1] - b[1])
    sr = (X * (b[1] - g[1]) - g[0] * (Y * (b[1] - 1.0) + b[1] * (X + Z)) + b[0] * (Y * (g[1] - 1.0) + g[1] * (X + Z))) / d
    sg = (X * (r[1] - b[1]) + r[0] * (Y * (b[1] - 1.0) + b[1] * (X + Z)) - b[0] * (Y * (r[1] - 1.0) + r[1] * (X + Z))) / d
    sb = (X * (g[1] - r[1]) - r[0] * (Y * (g[1] - 1.0) + g[1] * (X + Z)) + g[0] * (Y * (r[1] - 1.0) + r[1] * (X + Z))) / d
    m = [sr * r[0], sg * g[0], sb * b[0], sr * r[1], sg * g[1], sb * b[1],
         sr * (1.0 - r[0] - r[1]), sg * (1.0 - g[0] - g[1]), sb * (1.0 - b[0] - b[1])]
    return np.array([float("%.10f" % v) for v in m], dtype=np.float32).reshape(3, 3)


_REC709_E = _rgb_to_xyz_matrix((0.640, 0.330), (0.300, 0.600), (0.150, 0.060), (1.0 / 3.0, 1.0 / 3.0))


def rec709_e_to_xyz(rgb):
    """f32 evaluation in the reference's order: (r*m0 + g*m1) + b*m2."""
    rgb = np.asarray(rgb, dtype=np.float32)
    m = _REC709_E
    out = np.empty(3, dtype=np.float32)
    for i in range(3):
        out[i] = (rgb[0] * m[i, 0] + rgb[1] * m[i, 1]) + rgb[2] * m[i, 2]
    return out


def xyz_color(rgb):
    c = abi.PsyColor()
    c.kind = abi.PSY_COLOR_XYZ
    x = rec709_e_to_xyz(rgb)
    c.v[0], c.v[1], c.v[2] = float(x[0]), float(x[1]), float(x[2])
    return c


def blackbody_color(temperature, factor, normalized=False):
    c = abi.PsyColor()
    c.kind = abi.PSY_COLOR_TEMPERATURE if normalized else abi.PSY_COLOR_BLACKBODY
    c.v[0], c.v[1], c.v[2] = temperature, factor, 0.0
    return c


# ---------------------------------------------------------------- transforms
def translate(t):
    m = np.eye(4)
    m[:3, 3] = t
    return m


def rot_axis(axis, angle):
    axis = np.asarray(axis, dtype=np.float64)
    axis = axis / np.linalg.norm(axis)
    x, y, z = axis
    c, s = math.cos(angle), math.sin(angle)
    C1 = 1 - c
    m = np.eye(4)
    m[:3, :3] = [[c + x * x * C1, x * y * C1 - z * s, x * z * C1 + y * s],
                 [y * x * C1 + z * s, c + y * y * C1, y * z * C1 - x * s],
                 [z * x * C1 - y * s, z * y * C1 + x * s, c + z * z * C1]]
    return m


def to_psy_transform(m4):
    """4x4 (f64) -> PsyTransform (3x4 row-major f32)."""
    t = abi.PsyTransform()
    vals = np.asarray(m4, dtype=np.float64)[:3, :4].astype(np.float32).reshape(-1)
    for i in range(12):
        t.m[i] = float(vals[i])
    return t


def world_to_object(obj_to_world):
    return np.linalg.inv(obj_to_world)


# ---------------------------------------------------------------- scene container
class SceneData:
    """Numpy-backed scene description; `desc()` returns a PsySceneDesc whose
    pointers stay valid while this object lives."""

    def __init__(self, width, height, spp, seed=0, max_bounces=2):
        self.width, self.height, self.spp, self.seed, self.max_bounces = width, height, spp, seed, max_bounces
        self.objects = []      # dicts
        self.shaders = []      # PsyShaderDesc
        self.instances = []    # (object, shader, [4x4 world->object keys])
        self.camera = None
        self.background = xyz_color((0.0, 0.0, 0.0))
        self.distant = []      # (radii, directions, colors)
        self._keep = []

    # -- content
    def add_shader(self, kind, rgb=(0.8, 0.8, 0.8), roughness=0.0, fresnel=0.0, color=None):
        s = abi.PsyShaderDesc()
        s.kind = kind
        s.color = color if color is not None else xyz_color(rgb)
        s.roughness, s.fresnel = roughness, fresnel
        self.shaders.append(s)
        return len(self.shaders) - 1

    def add_mesh(self, verts, indices, normals=None):
        """verts: [time][n][3] or [n][3]; indices: [m][3]; normals like verts."""
        v = np.ascontiguousarray(np.asarray(verts, dtype=np.float32))
        if v.ndim == 2:
            v = v[None]
        n = None
        if normals is not None:
            n = np.ascontiguousarray(np.asarray(normals, dtype=np.float32))
            if n.ndim == 2:
                n = n[None]
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.uint32))
        self.objects.append(dict(kind=abi.PSY_OBJ_MESH, verts=v, normals=n, indices=idx))
        return len(self.objects) - 1

    def add_rect_light(self, dims, colors):
        d = np.ascontiguousarray(np.asarray(dims, dtype=np.float32).reshape(-1, 2))
        self.objects.append(dict(kind=abi.PSY_OBJ_RECT_LIGHT, dims=d, colors=list(colors)))
        return len(self.objects) - 1

    def add_sphere_light(self, radii, colors):
        d = np.ascontiguousarray(np.asarray(radii, dtype=np.float32).reshape(-1))
        self.objects.append(dict(kind=abi.PSY_OBJ_SPHERE_LIGHT, dims=d, colors=list(colors)))
        return len(self.objects) - 1

    def add_instance(self, obj, shader=-1, world_to_object_keys=()):
        self.instances.append((obj, shader, [np.asarray(k, dtype=np.float64) for k in world_to_object_keys]))
        return len(self.instances) - 1

    def set_camera(self, cam_to_world_keys, fovs_deg, aperture_radii=(), focus_distances=(), fovs_rad=None):
        """Camera keys; fields of view in degrees, or already in radians
        (fovs_rad, as f32 values computed by the caller)."""
        fovs = list(fovs_rad) if fovs_rad is not None else [math.radians(f) for f in fovs_deg]
        self.camera = ([np.asarray(k) for k in cam_to_world_keys], fovs, list(aperture_radii), list(focus_distances))

    def add_distant_light(self, radii, directions, colors):
        self.distant.append((list(radii), np.asarray(directions, dtype=np.float32).reshape(-1, 3), list(colors)))

    @property
    def num_tris(self):
        return sum(int(o["indices"].shape[0]) for o in self.objects if o["kind"] == abi.PSY_OBJ_MESH)

    # -- flatten
    def desc(self):
        keep = []
        d = abi.PsySceneDesc()
        objs = (abi.PsyObjectDesc * max(1, len(self.objects)))()
        for i, o in enumerate(self.objects):
            od = objs[i]
            od.kind = o["kind"]
            if o["kind"] == abi.PSY_OBJ_MESH:
                v = o["verts"]
                od.time_samples = v.shape[0]
                od.num_verts = v.shape[1]
                od.num_tris = o["indices"].shape[0]
                od.verts = v.ctypes.data_as(C.POINTER(C.c_float))
                od.normals = o["normals"].ctypes.data_as(C.POINTER(C.c_float)) if o["normals"] is not None else None
                od.indices = o["indices"].ctypes.data_as(C.POINTER(C.c_uint32))
            else:
                od.time_samples = len(o["colors"])
                od.dims = o["dims"].ctypes.data_as(C.POINTER(C.c_float))
                cols = (abi.PsyColor * len(o["colors"]))(*o["colors"])
                keep.append(cols)
                od.colors = cols
        keep.append(objs)
        d.num_objects, d.objects = len(self.objects), objs
        sh = (abi.PsyShaderDesc * max(1, len(self.shaders)))(*self.shaders)
        keep.append(sh)
        d.num_shaders, d.shaders = len(self.shaders), sh
        xforms = []
        insts = (abi.PsyInstanceDesc * max(1, len(self.instances)))()
        for i, (obj, shader, keys) in enumerate(self.instances):
            insts[i].object, insts[i].shader = obj, shader
            insts[i].xform_start, insts[i].xform_count = len(xforms), len(keys)
            xforms.extend(keys)
        keep.append(insts)
        d.num_instances, d.instances = len(self.instances), insts
        xf = (abi.PsyTransform * max(1, len(xforms)))(*[to_psy_transform(k) for k in xforms])
        keep.append(xf)
        d.num_xforms, d.xforms = len(xforms), xf
        if self.camera is None:
            raise ValueError("scene has no camera")
        ck, fovs, ap, fd = self.camera
        ct = (abi.PsyTransform * len(ck))(*[to_psy_transform(k) for k in ck])
        cf = (C.c_float * len(fovs))(*fovs)
        ca = (C.c_float * max(1, len(ap)))(*ap)
        cd = (C.c_float * max(1, len(fd)))(*fd)
        keep += [ct, cf, ca, cd]
        d.camera.num_transforms, d.camera.transforms = len(ck), ct
        d.camera.num_fovs, d.camera.fovs = len(fovs), cf
        d.camera.num_aperture_radii, d.camera.aperture_radii = len(ap), ca
        d.camera.num_focus_distances, d.camera.focus_distances = len(fd), cd
        d.background = self.background
        dl = (abi.PsyDistantLightDesc * max(1, len(self.distant)))()
        for i, (radii, dirs, cols) in enumerate(self.distant):
            r = (C.c_float * len(radii))(*radii)
            dd = np.ascontiguousarray(dirs)
            cc = (abi.PsyColor * len(cols))(*cols)
            keep += [r, dd, cc]
            dl[i].num_keys, dl[i].radii = len(radii), r
            dl[i].directions = dd.ctypes.data_as(C.POINTER(C.c_float))
            dl[i].colors = cc
        keep.append(dl)
        d.num_distant_lights, d.distant_lights = len(self.distant), dl
        d.width, d.height, d.spp, d.seed, d.max_bounces = self.width, self.height, self.spp, self.seed, self.max_bounces
        self._keep = keep
        return d


# ---------------------------------------------------------------- geometry helpers
def quad(p0, p1, p2, p3):
    """Two triangles (p0,p1,p2), (p0,p2,p3)."""
    return np.array([p0, p1, p2, p3], dtype=np.float64), np.array([[0, 1, 2], [0, 2, 3]], dtype=np.uint32)


def box(center, size, rot_y):
    """Axis-aligned box rotated about y; 12 tris."""
    sx, sy, sz = size
    c = np.array([[x, y, z] for x in (-sx / 2, sx / 2) for y in (0.0, sy) for z in (-sz / 2, sz / 2)], dtype=np.float64)
    R = rot_axis((0, 1, 0), rot_y)[:3, :3]
    v = c @ R.T + np.asarray(center, dtype=np.float64)
    # vertex index = ix*4 + iy*2 + iz
    faces = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    tris = []
    for a, b, cc, d in faces:
        tris += [[a, b, cc], [a, cc, d]]
    return v, np.array(tris, dtype=np.uint32)


def icosphere(level):
    """Unit icosphere with `level` 4-way subdivisions (20*4^level tris)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    for _ in range(level):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        e.sort(axis=1)
        key = e[:, 0] * (nv + 1) + e[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a = uniq // (nv + 1)
        b = uniq % (nv + 1)
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        v = np.concatenate([v, mid], axis=0)
        m = inv.reshape(3, -1) + nv
        m01, m12, m20 = m[0], m[1], m[2]
        f = np.concatenate([np.stack([f[:, 0], m01, m20], 1), np.stack([f[:, 1], m12, m01], 1),
                            np.stack([f[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)], axis=0)
    return v, f.astype(np.uint32)


def value_noise3(p, seed, octaves=3):
    """Seeded 3-octave value noise in [-1, 1] (lattice hash, smoothstep)."""
    p = np.asarray(p, dtype=np.float64)
    total = np.zeros(p.shape[0])
    amp, freq, norm = 1.0, 1.0, 0.0
    for o in range(octaves):
        q = p * freq * 2.0
        i0 = np.floor(q).astype(np.int64)
        fr = q - i0
        w = fr * fr * (3.0 - 2.0 * fr)
        acc = np.zeros(p.shape[0])
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    h = ((i0[:, 0] + dx) * 73856093) ^ ((i0[:, 1] + dy) * 19349663) ^ ((i0[:, 2] + dz) * 83492791)
                    h = (h ^ (seed * 2654435761 + o * 97531)) & 0xFFFFFFFF
                    h = (h ^ (h >> 16)) * 0x45d9f3b & 0xFFFFFFFF
                    h = (h ^ (h >> 16)) & 0xFFFFFFFF
                    val = (h / 4294967295.0) * 2.0 - 1.0
                    wx = w[:, 0] if dx else 1 - w[:, 0]
                    wy = w[:, 1] if dy else 1 - w[:, 1]
                    wz = w[:, 2] if dz else 1 - w[:, 2]
                    acc += val * wx * wy * wz
        total += acc * amp
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


def displaced_sphere(level, amplitude, seed):
    v, f = icosphere(level)
    n = value_noise3(v * 2.0, seed)
    v = v * (1.0 + amplitude * n)[:, None]
    return v, f


def look_at(eye, target, up=(0, 1, 0)):
    """Camera-to-world transform: camera looks down its local +z, image x to
    the right and y up."""
    eye = np.asarray(eye, dtype=np.float64)
    fwd = np.asarray(target, dtype=np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, np.asarray(up, dtype=np.float64))
    right /= np.linalg.norm(right)
    upv = np.cross(right, fwd)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = right, upv, fwd, eye
    return m


# ---------------------------------------------------------------- workloads
def cornell_box(width=512, height=512, spp=16, max_bounces=4, seed=0):
    """Procedural Cornell box: 5 axis-aligned wall quads (10 tris), 2 rotated
    boxes (24 tris), a 0.25x0.25 rectangle light under the ceiling."""
    s = SceneData(width, height, spp, seed, max_bounces)
    white = s.add_shader(abi.PSY_SHADER_LAMBERT, (0.73, 0.73, 0.73))
    red = s.add_shader(abi.PSY_SHADER_LAMBERT, (0.63, 0.065, 0.05))
    green = s.add_shader(abi.PSY_SHADER_LAMBERT, (0.14, 0.45, 0.091))
    # white walls: floor, ceiling, back
    vs, fs = [], []
    for q in ([(-1, 0, -1), (1, 0, -1), (1, 0, 1), (-1, 0, 1)],
              [(-1, 2, -1), (-1, 2, 1), (1, 2, 1), (1, 2, -1)],
              [(-1, 0, -1), (-1, 2, -1), (1, 2, -1), (1, 0, -1)]):
        v, f = quad(*q)
        fs.append(f + sum(len(x) for x in vs))
        vs.append(v)
    walls = s.add_mesh(np.concatenate(vs), np.concatenate(fs))
    v, f = quad((-1, 0, -1), (-1, 0, 1), (-1, 2, 1), (-1, 2, -1))
    left = s.add_mesh(v, f)
    v, f = quad((1, 0, -1), (1, 2, -1), (1, 2, 1), (1, 0, 1))
    right = s.add_mesh(v, f)
    v1, f1 = box((-0.35, 0.0, -0.3), (0.55, 1.2, 0.55), math.radians(17.0))
    v2, f2 = box((0.38, 0.0, 0.3), (0.55, 0.6, 0.55), math.radians(-18.0))
    boxes = s.add_mesh(np.concatenate([v1, v2]), np.concatenate([f1, f2 + len(v1)]))
    for obj, sh in ((walls, white), (left, red), (right, green), (boxes, white)):
        s.add_instance(obj, sh)
    light = s.add_rect_light([(0.25, 0.25)], [xyz_color((6.0, 6.0, 6.0))])
    # object z axis points down (-y world), light at the ceiling
    o2w = translate((0.0, 1.98, 0.0)) @ rot_axis((1, 0, 0), math.pi / 2)
    s.add_instance(light, -1, [world_to_object(o2w)])
    s.set_camera([look_at((0.0, 1.0, 3.9), (0.0, 1.0, 0.0))], [40.0])
    return s


def mesh_stress(width=1920, height=1080, spp=64, max_bounces=6, seed=0, level=8):
    """Noise-displaced icosphere (level 8 = 1,310,720 tris, amplitude 0.05) on
    a 2-tri ground plane; sphere light r=0.1 and a 0.5-degree sun disc; GGX
    with roughness drawn from U(0.1, 0.8) per object (fresnel 0.25)."""
    rng = np.random.default_rng(seed + 12345)
    s = SceneData(width, height, spp, seed, max_bounces)
    r1, r2 = rng.uniform(0.1, 0.8, size=2)
    sph_sh = s.add_shader(abi.PSY_SHADER_GGX, (0.8, 0.55, 0.35), roughness=float(r1), fresnel=0.25)
    gnd_sh = s.add_shader(abi.PSY_SHADER_GGX, (0.6, 0.6, 0.6), roughness=float(r2), fresnel=0.25)
    v, f = displaced_sphere(level, 0.05, seed)
    v = v + np.array([0.0, 1.0, 0.0])
    sph = s.add_mesh(v, f)
    gv, gf = quad((-20, 0, -20), (-20, 0, 20), (20, 0, 20), (20, 0, -20))
    gnd = s.add_mesh(gv, gf)
    s.add_instance(sph, sph_sh)
    s.add_instance(gnd, gnd_sh)
    lt = s.add_sphere_light([0.1], [xyz_color((40.0, 38.0, 34.0))])
    s.add_instance(lt, -1, [world_to_object(translate((1.4, 2.4, 1.2)))])
    sun_dir = np.array([-0.4, -1.0, -0.3])
    sun_dir /= np.linalg.norm(sun_dir)
    s.add_distant_light([math.radians(0.25)], sun_dir, [xyz_color((3000.0, 2900.0, 2700.0))])
    s.background = xyz_color((0.05, 0.07, 0.1))
    s.set_camera([look_at((0.0, 1.4, 4.2), (0.0, 0.9, 0.0))], [45.0])
    return s


def motion_instances(width=1280, height=720, spp=32, max_bounces=2, seed=0, n_instances=2000, level=5, n_lights=64):
    """2,000 instances of a 20,480-tri displaced sphere, uniform positions in
    a 100^3 box, 4-key transform motion (rotation <= 30 deg, translation <= 2);
    one extra mesh with 2-segment (3-key) deformation blur; 64 sphere lights
    sampled through the light tree."""
    rng = np.random.default_rng(seed + 777)
    s = SceneData(width, height, spp, seed, max_bounces)
    v, f = displaced_sphere(level, 0.05, seed + 1)
    mesh = s.add_mesh(v, f)
    shaders = [s.add_shader(abi.PSY_SHADER_LAMBERT, tuple(rng.uniform(0.2, 0.9, 3))) for _ in range(8)]
    for i in range(n_instances):
        pos = rng.uniform(-50.0, 50.0, 3)
        axis = rng.normal(size=3)
        total_angle = math.radians(rng.uniform(0.0, 30.0))
        trans = rng.uniform(-1.0, 1.0, 3)
        trans = trans / max(1e-9, np.linalg.norm(trans)) * rng.uniform(0.0, 2.0)
        scale = rng.uniform(0.6, 1.6)
        keys = []
        for k in range(4):
            a = k / 3.0
            o2w = translate(pos + trans * a) @ rot_axis(axis, total_angle * a) @ np.diag([scale, scale, scale, 1.0])
            keys.append(world_to_object(o2w))
        s.add_instance(mesh, shaders[i % len(shaders)], keys)
    # deforming mesh: 3 vertex keys
    dv, df = displaced_sphere(level, 0.05, seed + 2)
    keys = [dv * 4.0 + np.array([0.0, 0.0, -10.0]) + np.array([k * 1.5, 0.0, 0.0]) * (1.0 + 0.2 * dv[:, :1]) for k in range(3)]
    dmesh = s.add_mesh(np.stack(keys), df)
    s.add_instance(dmesh, shaders[0])
    for i in range(n_lights):
        lt = s.add_sphere_light([rng.uniform(0.5, 1.5)], [xyz_color(tuple(rng.uniform(20.0, 60.0, 3)))])
        s.add_instance(lt, -1, [world_to_object(translate(rng.uniform(-50.0, 50.0, 3)))])
    s.background = xyz_color((0.02, 0.02, 0.03))
    s.set_camera([look_at((0.0, 0.0, 95.0), (0.0, 0.0, 0.0))], [60.0])
    return s


def grid_mesh(nx=2048, ny=1024, seed=0, amplitude=0.05):
    """Noise-displaced grid of nx*ny quads (2*nx*ny tris) over [-1,1]x[-0.5,0.5]
    in the xz plane, displaced in y.  Returns a SceneData with the grid as its
    only object plus the vertex / index arrays (for ray generation)."""
    xs = np.linspace(-1.0, 1.0, nx + 1)
    zs = np.linspace(-0.5, 0.5, ny + 1)
    X, Z = np.meshgrid(xs, zs)
    P = np.stack([X.ravel(), np.zeros(X.size), Z.ravel()], 1)
    P[:, 1] = amplitude * value_noise3(P * 4.0, seed)
    ii = np.arange(ny)[:, None] * (nx + 1) + np.arange(nx)[None, :]
    a, b, c, d = ii, ii + 1, ii + nx + 2, ii + nx + 1
    f = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3), np.stack([a, c, d], -1).reshape(-1, 3)], 0)
    s = SceneData(64, 64, 1, seed, 2)
    sh = s.add_shader(abi.PSY_SHADER_LAMBERT, (0.7, 0.7, 0.7))
    obj = s.add_mesh(P, f.astype(np.uint32))
    s.add_instance(obj, sh)
    s.set_camera([look_at((0.0, 1.5, 1.5), (0.0, 0.0, 0.0))], [50.0])
    return s, P.astype(np.float32), f.astype(np.uint32)


def rays_array(orig, dirs, max_t=np.inf, time=0.0, wavelength=550.0, occlusion=False):
    r = np.zeros(len(orig), dtype=abi.ray_dtype())
    r["orig"] = orig
    r["dir"] = dirs
    r["max_t"] = max_t
    r["time"] = time
    r["wavelength"] = wavelength
    r["flags"] = abi.PSY_RAY_OCCLUSION if occlusion else 0
    return r


def coherent_rays(n_side, eye=(0.0, 1.5, 1.5), target=(0.0, 0.0, 0.0), fov_deg=50.0):
    """Pinhole camera rays, n_side x n_side, normalized directions."""
    m = look_at(eye, target)
    t = math.tan(math.radians(fov_deg) / 2)
    u = (np.arange(n_side) + 0.5) / n_side * 2 - 1
    U, V = np.meshgrid(u, -u)
    d = np.stack([U.ravel() * t, V.ravel() * t, np.ones(U.size)], 1)
    d = d @ m[:3, :3].T
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.broadcast_to(np.asarray(eye, dtype=np.float64), d.shape)
    return rays_array(o.astype(np.float32), d.astype(np.float32))


def incoherent_rays(P, F, n, seed=7):
    """Cosine-hemisphere directions from uniformly random surface points of the
    mesh (P, F), origins offset along the normal by the surface error bound."""
    rng = np.random.default_rng(seed)
    tri = rng.integers(0, F.shape[0], n)
    u, v = rng.random(n), rng.random(n)
    su = np.sqrt(u)
    b0, b1, b2 = 1 - su, su * (1 - v), v * su
    p0, p1, p2 = P[F[tri, 0]].astype(np.float64), P[F[tri, 1]].astype(np.float64), P[F[tri, 2]].astype(np.float64)
    pos = p0 * b0[:, None] + p1 * b1[:, None] + p2 * b2[:, None]
    nrm = np.cross(p1 - p0, p2 - p0)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm[nrm[:, 1] < 0] *= -1
    # cosine hemisphere around nrm
    r1, r2 = rng.random(n), rng.random(n)
    phi = 2 * math.pi * r1
    sr = np.sqrt(r2)
    local = np.stack([np.cos(phi) * sr, np.sin(phi) * sr, np.sqrt(np.maximum(0, 1 - r2))], 1)
    a = np.where(np.abs(nrm[:, :1]) > 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    tx = np.cross(a, nrm)
    tx /= np.linalg.norm(tx, axis=1, keepdims=True)
    ty = np.cross(nrm, tx)
    d = tx * local[:, :1] + ty * local[:, 1:2] + nrm * local[:, 2:3]
    err = np.abs(pos).max(axis=1) * 1e-6 + 1e-6
    o = pos + nrm * err[:, None] * 4
    return rays_array(o.astype(np.float32), d.astype(np.float32))
