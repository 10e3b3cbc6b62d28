"""The car mesh the reference draws into its G-buffer for the W17 scene: the GLB
reader (src/engine/glb.ts), MeshCar.load's vertex, index and tag buffers, its
draws and textures (src/engine/mesh-car.ts:46-213), and the MeshCam uniform the
engine fills each frame (src/engine/engine.ts:679-686), over libwt's mesh pass
(wt_mesh_*, wt_render_mesh).

    data = load_w17_mesh("path/to/public/models")   # the reference's asset files
    mesh = MeshCar(engine, data)
    renderer.frame(cam, look, view, mesh=mesh, shape=params)   # G-buffer, then the scene composite

`synthetic_mesh()` builds a stand-in in the same formats (analytic shapes
tessellated with numpy, a procedural texture, decals and a gurney tab); the
tests and the render workload use it where the reference's assets are absent.

Texture images are decoded here (zlib, then libwt's PNG unfilter) instead of by
the browser (main.ts:989-995); the browser's canvas round trip premultiplies
alpha, so partly transparent texels may differ from the reference's by the
rounding of that round trip.
"""
import ctypes
import json
import math
import os
import re
import struct
import zlib
from dataclasses import dataclass, field

import numpy as np

from . import _abi

FRONT_AXLE_X = 1.0            # CAR_LAYOUT.frontAxleX (car-model.ts:16)
REAR_AXLE_X = 4.4             # CAR_LAYOUT.wheels.rear.x
BASE_RIDE_H = 0.092           # CAR_LAYOUT.baseRideH
MESH_FRONT_AXLE_Z = 1.615     # car-model.ts:12-13
MESH_GROUND_Y = -0.04
WHEEL_MATERIALS = {"tread_medium.007", "sidewall.007", "mercedes_wheel_hub.007", "discs.007"}
EMISSIVE = re.compile(r"light|led|kers|lcd", re.I)  # mesh-car.ts:21-27
PAINT = re.compile(r"paint", re.I)
CARBON = re.compile(r"carbon", re.I)
PART_MASK, ASSEMBLY_SHIFT = 7, 3   # RIG (car-model.ts:44-50)
REAR_FLAP, REAR_WING = 3, 2
REAR_MAX_Z = 0.53
GURNEY_VISUAL_HEIGHT = 0.015       # mesh-car.ts:209
GURNEY_MAT = dict(color=(0.025, 0.026, 0.03, 1.0), metal=0.0, rough=0.35, coat=0.6, alpha_cut=0.0, emissive=0.0,
                  is_body=1.0)


# ---------------------------------------------------------------- GLB (glb.ts)
@dataclass
class GlbPrimitive:
    node: str
    material: int
    positions: np.ndarray   # [n, 3] float32, world space of the file
    normals: np.ndarray     # [n, 3] float32 or None
    uvs: np.ndarray         # [n, 2] float32 or None
    indices: np.ndarray     # uint32


@dataclass
class GlbMaterial:
    name: str
    base_color: tuple
    base_color_texture: int
    normal_texture: int
    metallic: float
    roughness: float
    blend: bool
    double_sided: bool


@dataclass
class GlbScene:
    primitives: list
    materials: list
    images: list            # [(mime, bytes)]
    texture_image: list
    asset: dict


_COMPONENTS = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT4": 16}


def _node_matrix(n):
    """nodeMatrix (glb.ts:36-49), float64 column-major."""
    if "matrix" in n:
        return [float(v) for v in n["matrix"]]
    tx, ty, tz = n.get("translation", [0, 0, 0])
    x, y, z, w = n.get("rotation", [0, 0, 0, 1])
    sx, sy, sz = n.get("scale", [1, 1, 1])
    m = [0.0] * 16
    m[0] = (1 - 2 * (y * y + z * z)) * sx; m[1] = 2 * (x * y + z * w) * sx; m[2] = 2 * (x * z - y * w) * sx
    m[4] = 2 * (x * y - z * w) * sy; m[5] = (1 - 2 * (x * x + z * z)) * sy; m[6] = 2 * (y * z + x * w) * sy
    m[8] = 2 * (x * z + y * w) * sz; m[9] = 2 * (y * z - x * w) * sz; m[10] = (1 - 2 * (x * x + y * y)) * sz
    m[12] = tx; m[13] = ty; m[14] = tz; m[15] = 1
    return [float(v) for v in m]


def _mul(a, b):
    """mul (glb.ts:51-59): sums in k order, in float64."""
    o = [0.0] * 16
    for c in range(4):
        for r in range(4):
            s = 0.0
            for k in range(4):
                s += a[k * 4 + r] * b[c * 4 + k]
            o[c * 4 + r] = s
    return o


def parse_glb(data):
    """parseGlb (glb.ts:61-150)."""
    buf = memoryview(data)
    if struct.unpack_from("<I", buf, 0)[0] != 0x46546C67:
        raise ValueError("Not a GLB file")
    json_len = struct.unpack_from("<I", buf, 12)[0]
    js = json.loads(bytes(buf[20:20 + json_len]).decode())
    bin_off = 20 + json_len + 8
    raw = np.frombuffer(data, np.uint8)

    def read_accessor(index):
        a = js["accessors"][index]
        bv = js["bufferViews"][a["bufferView"]]
        n = _COMPONENTS[a["type"]]
        ct = a["componentType"]
        size = 4 if ct in (5126, 5125) else (2 if ct == 5123 else 1)
        base = bin_off + bv.get("byteOffset", 0) + a.get("byteOffset", 0)
        stride = bv.get("byteStride", n * size)
        dt = {5126: "<f4", 5125: "<u4", 5123: "<u2"}.get(ct, "u1")
        view = np.lib.stride_tricks.as_strided(raw[base:], shape=(a["count"], n * size), strides=(stride, 1))
        vals = np.ascontiguousarray(view).view(dt).reshape(a["count"], n)
        return vals.astype(np.float32 if ct == 5126 else np.uint32)

    prims = []

    def walk(index, parent):
        node = js["nodes"][index]
        world = _mul(parent, _node_matrix(node))
        if "mesh" in node:
            W = world
            for p in js["meshes"][node["mesh"]]["primitives"]:
                pos = read_accessor(p["attributes"]["POSITION"]).astype(np.float64)
                x, y, z = pos[:, 0], pos[:, 1], pos[:, 2]
                wp = np.stack([W[0] * x + W[4] * y + W[8] * z + W[12], W[1] * x + W[5] * y + W[9] * z + W[13],
                               W[2] * x + W[6] * y + W[10] * z + W[14]], axis=1).astype(np.float32)
                wn = None
                if "NORMAL" in p["attributes"]:
                    nr = read_accessor(p["attributes"]["NORMAL"]).astype(np.float64)
                    a_, b_, c_ = nr[:, 0], nr[:, 1], nr[:, 2]
                    nx = W[0] * a_ + W[4] * b_ + W[8] * c_
                    ny = W[1] * a_ + W[5] * b_ + W[9] * c_
                    nz = W[2] * a_ + W[6] * b_ + W[10] * c_
                    ln = np.sqrt(nx * nx + ny * ny + nz * nz)
                    ln = np.where(ln == 0, 1.0, ln)
                    wn = np.stack([nx / ln, ny / ln, nz / ln], axis=1).astype(np.float32)
                uv = read_accessor(p["attributes"]["TEXCOORD_0"]) if "TEXCOORD_0" in p["attributes"] else None
                if "indices" in p:
                    idx = read_accessor(p["indices"]).reshape(-1).astype(np.uint32)
                else:
                    idx = np.arange(wp.shape[0], dtype=np.uint32)
                prims.append(GlbPrimitive(node.get("name", ""), p.get("material", 0), wp, wn, uv, idx))
        for ch in node.get("children", []):
            walk(ch, world)

    ident = [1.0, 0, 0, 0, 0, 1.0, 0, 0, 0, 0, 1.0, 0, 0, 0, 0, 1.0]
    for root in js["scenes"][js.get("scene", 0)]["nodes"]:
        walk(root, [float(v) for v in ident])
    mats = []
    for m in js.get("materials", []):
        pbr = m.get("pbrMetallicRoughness", {})
        mats.append(GlbMaterial(m.get("name", ""), tuple(pbr.get("baseColorFactor", [1, 1, 1, 1])),
                                pbr.get("baseColorTexture", {}).get("index"), m.get("normalTexture", {}).get("index"),
                                pbr.get("metallicFactor", 1), pbr.get("roughnessFactor", 1),
                                m.get("alphaMode") in ("BLEND", "MASK"), bool(m.get("doubleSided", False))))
    images = []
    for im in js.get("images", []):
        bv = js["bufferViews"][im["bufferView"]]
        o = bin_off + bv.get("byteOffset", 0)
        images.append((im.get("mimeType", ""), bytes(buf[o:o + bv["byteLength"]])))
    return GlbScene(prims, mats, images, [t["source"] for t in js.get("textures", [])], js.get("asset", {}))


# ---------------------------------------------------------------- PNG
def decode_png(data, lib=None):
    """A PNG (8-bit or lower depth; grey, RGB, palette, grey-alpha, RGBA; not
    interlaced) as (width, height, [h, w, 4] uint8 RGBA)."""
    lib = lib or _abi.load()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG")
    i, idat, plte, trns = 8, [], None, None
    while i < len(data):
        n, kind = struct.unpack(">I4s", data[i:i + 8])
        body = data[i + 8:i + 8 + n]
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = np.frombuffer(body, np.uint8)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
        i += 12 + n
    if interlace or depth not in (1, 2, 4, 8):
        raise ValueError(f"unsupported PNG (bit depth {depth}, interlace {interlace})")
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    row_bytes = (w * chans * depth + 7) // 8
    filtered = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8)
    if filtered.size < h * (row_bytes + 1):
        raise ValueError("truncated PNG data")
    out = np.empty((h, row_bytes), np.uint8)
    rc = lib.wt_png_unfilter(filtered.ctypes.data, h, row_bytes, max(1, chans * depth // 8), out.ctypes.data)
    if rc != 0:
        raise ValueError("bad PNG filter type")
    if depth < 8:  # unpack samples, most significant bits first
        bits = np.unpackbits(out, axis=1).reshape(h, -1, depth)
        vals = np.zeros(bits.shape[:2], np.uint16)
        for b in range(depth):
            vals = (vals << 1) | bits[:, :, b]
        samples = vals[:, :w * chans].astype(np.uint8)
        if ctype == 0:
            samples = (samples.astype(np.uint32) * 255 // ((1 << depth) - 1)).astype(np.uint8)
    else:
        samples = out[:, :w * chans]
    s = samples.reshape(h, w, chans)
    rgba = np.empty((h, w, 4), np.uint8)
    if ctype == 3:
        idx = s[:, :, 0]
        rgba[..., :3] = plte[idx]
        alpha = np.full(256, 255, np.uint8)
        if trns is not None:
            alpha[:len(trns)] = trns
        rgba[..., 3] = alpha[idx]
    elif ctype in (0, 4):
        rgba[..., :3] = s[:, :, :1]
        rgba[..., 3] = s[:, :, 1] if ctype == 4 else 255
    else:
        rgba[..., :3] = s[:, :, :3]
        rgba[..., 3] = s[:, :, 3] if ctype == 6 else 255
    return w, h, rgba


# ---------------------------------------------------------------- MeshCar.load
@dataclass
class DrawSpec:
    """One draw: its MeshMat values, index range, texture slot and state."""
    name: str
    color: tuple
    metal: float
    rough: float
    coat: float
    alpha_cut: float
    emissive: float
    is_body: float
    first: int
    count: int
    texture: int = -1
    blend: bool = False
    optional: bool = False


@dataclass
class MeshData:
    """MeshCar's buffers: verts [n, 8] float32 (x, y, z, u, nx, ny, nz, v), indices
    uint32, tags uint8 per vertex, draws in record order, textures as
    (width, height, [h, w, 4] uint8)."""
    verts: np.ndarray
    indices: np.ndarray
    tags: np.ndarray
    draws: list
    textures: list = field(default_factory=list)


def gurney_geometry(edge):
    """gurneyGeometry (mesh-car.ts:211-231): a thin tab normal to the chord along
    the trailing edge of the last rear-wing element, both sides."""
    verts, idx = [], []
    span = [dict(edge[0], z=0.0)] + list(edge) + [dict(edge[-1], z=REAR_MAX_Z)]
    for side in (1, -1):
        base = len(verts) // 8
        for s in span:
            dx, dy = s["te"][0] - s["le"][0], s["te"][1] - s["le"][1]
            ln = math.hypot(dx, dy) or 1.0
            up = (-dy / ln, dx / ln)
            top = (s["te"][0] + up[0] * GURNEY_VISUAL_HEIGHT, s["te"][1] + up[1] * GURNEY_VISUAL_HEIGHT)
            verts += [s["te"][0], s["te"][1], s["z"] * side, 0, dx / ln, dy / ln, 0, 0]
            verts += [top[0], top[1], s["z"] * side, 0, dx / ln, dy / ln, 0, 0]
        for i in range(len(span) - 1):
            a = base + i * 2
            idx += [a, a + 1, a + 2, a + 1, a + 3, a + 2]
    return np.array(verts, np.float32).reshape(-1, 8), np.array(idx, np.uint32)


def detach_seams(verts, indices, tags):
    """detachSeams (mesh-car.ts:236-264): a triangle that straddles assemblies goes
    to the assembly owning most of its corners (ties to the largest), borrowing
    duplicated vertices re-tagged for it.  Rewrites `indices` in place; returns
    (verts, tags)."""
    asm = tags >> ASSEMBLY_SHIFT
    f = indices.reshape(-1, 3)
    a = asm[f]
    mixed = np.nonzero(~((a[:, 0] == a[:, 1]) & (a[:, 1] == a[:, 2])))[0]
    extra, extra_tags, dup = [], [], {}
    base = tags.shape[0]
    for t in mixed.tolist():
        x, y, z = (int(v) for v in a[t])
        owner = x if (x == y or x == z) else (y if y == z else max(x, y, z))
        for k in range(3):
            v = int(f[t, k])
            if int(asm[v]) == owner:
                continue
            key = v * 4 + owner
            n = dup.get(key)
            if n is None:
                n = base + len(extra_tags)
                dup[key] = n
                extra.append(verts[v])
                extra_tags.append((int(tags[v]) & PART_MASK) | (owner << ASSEMBLY_SHIFT))
            f[t, k] = n
    if not extra_tags:
        return verts, tags
    return (np.concatenate([verts, np.array(extra, np.float32)]),
            np.concatenate([tags, np.array(extra_tags, np.uint8)]))


def to_car_frame(p):
    """toCarFrame (car-model.ts:27-29) of [n, 3] float32 -> float32."""
    p = p.astype(np.float64)
    return np.stack([FRONT_AXLE_X + (MESH_FRONT_AXLE_Z - p[:, 2]), p[:, 1] - MESH_GROUND_Y, p[:, 0]],
                    axis=1).astype(np.float32)


def normal_to_car_frame(n):
    """normalToCarFrame (car-model.ts:31-33)."""
    return np.stack([-n[:, 2], n[:, 1], n[:, 0]], axis=1).astype(np.float32)


def build_mesh(scene, vertex_parts, decode=None, gurney_edge=None):
    """MeshCar.load (mesh-car.ts:52-193) from a parsed GLB, the per-vertex part
    tags (w17.rig.bin) and the rear wing's trailing-edge stations."""
    verts, idx, ranges, vbase = [], [], [], 0
    ibase = 0
    for p in scene.primitives:
        n = p.positions.shape[0]
        v = np.zeros((n, 8), np.float32)
        v[:, 0:3] = to_car_frame(p.positions)
        v[:, 4:7] = normal_to_car_frame(p.normals) if p.normals is not None else np.array([0, 1, 0], np.float32)
        if p.uvs is not None:
            v[:, 3] = p.uvs[:, 0]
            v[:, 7] = p.uvs[:, 1]
        verts.append(v)
        idx.append(p.indices.astype(np.uint32) + np.uint32(vbase))
        ranges.append((ibase, p.indices.size, p.material))
        vbase += n
        ibase += p.indices.size
    mesh_vertices = vbase
    gurney = None
    if gurney_edge is not None:
        gv, gi = gurney_geometry(gurney_edge)
        verts.append(gv)
        idx.append(gi + np.uint32(vbase))
        gurney = (ibase, gi.size)
    verts = np.concatenate(verts)
    indices = np.concatenate(idx).astype(np.uint32)
    tags = np.zeros(verts.shape[0], np.uint8)
    tags[:mesh_vertices] = np.asarray(vertex_parts, np.uint8)[:mesh_vertices]
    tags[mesh_vertices:] = REAR_FLAP | (REAR_WING << ASSEMBLY_SHIFT)
    verts, tags = detach_seams(verts, indices, tags)
    decode = decode or (lambda b, mime: decode_png(b))
    textures, slot_of = [], {}

    def texture_for(ti):
        if ti is None:
            return -1
        img = scene.texture_image[ti]
        if img not in slot_of:
            mime, b = scene.images[img]
            w, h, rgba = decode(b, mime)
            slot_of[img] = len(textures)
            textures.append((w, h, rgba))
        return slot_of[img]

    draws = []
    order = sorted(range(len(ranges)), key=lambda i: int(scene.materials[ranges[i][2]].blend))  # stable
    for ri in order:
        first, count, mi = ranges[ri]
        m = scene.materials[mi]
        tex = texture_for(m.base_color_texture)
        draws.append(DrawSpec(m.name, tuple(m.base_color), min(m.metallic, 0.9), max(m.roughness, 0.05),
                              1.0 if PAINT.search(m.name) else (0.6 if CARBON.search(m.name) else 0.2),
                              0.02 if m.blend else 0.0, 1.5 if EMISSIVE.search(m.name) else 0.0,
                              0.0 if m.name in WHEEL_MATERIALS else 1.0, first, count, tex, m.blend))
    if gurney is not None:
        draws.append(DrawSpec("gurney", first=gurney[0], count=gurney[1], optional=True, **GURNEY_MAT))
    return MeshData(verts, indices, tags, draws, textures)


def load_w17_mesh(models_dir):
    """The reference's W17 assets (w17.glb, w17.rig.bin, w17.rig.json) as MeshCar's buffers."""
    with open(os.path.join(models_dir, "w17.glb"), "rb") as f:
        scene = parse_glb(f.read())
    parts = np.fromfile(os.path.join(models_dir, "w17.rig.bin"), np.uint8)
    with open(os.path.join(models_dir, "w17.rig.json")) as f:
        rig = json.load(f)
    return build_mesh(scene, parts, gurney_edge=rig["wings"]["rear"][-1])


# ---------------------------------------------------------------- the engine's side
def mesh_cam(cam, size, jitter, params):
    """MeshCar.setCamera as frame() calls it (engine.ts:679-686): cam a
    render.CameraState, jitter the frame's Halton offsets (jx, jy), params the
    ShapeParams (ride heights)."""
    c = _abi.MeshCam()
    c.view_proj[:] = [float(v) for v in cam.view_proj]
    c.cam_pos[:] = cam.pos
    c.ride_h = params.rideH
    c.jitter[:] = (-jitter[0] * 2 / size[0], jitter[1] * 2 / size[1])
    c.rake = math.atan((params.rearRideH - params.rideH) / (REAR_AXLE_X - FRONT_AXLE_X))
    c.base_ride = BASE_RIDE_H
    return c


class MeshCar:
    """A car mesh on an AeroEngine's device (wt_mesh_create and friends)."""

    def __init__(self, engine, data):
        self.engine = engine
        self.lib = engine.lib
        self.data = data
        v = np.ascontiguousarray(data.verts, np.float32)
        i = np.ascontiguousarray(data.indices, np.uint32)
        t = np.ascontiguousarray(data.tags, np.uint8)
        m = ctypes.c_void_p()
        engine._check(self.lib.wt_mesh_create(engine.ctx, v.ctypes.data, v.shape[0], i.ctypes.data, i.size,
                                              t.ctypes.data, ctypes.byref(m)), "wt_mesh_create")
        self.m = m
        for (w, h, rgba) in data.textures:
            px = np.ascontiguousarray(rgba, np.uint8)
            slot = ctypes.c_int32()
            engine._check(self.lib.wt_mesh_add_texture(self.m, w, h, px.ctypes.data, ctypes.byref(slot)),
                          "wt_mesh_add_texture")
        for d in data.draws:
            engine._check(self.lib.wt_mesh_add_draw(self.m, ctypes.byref(draw_struct(d))), "wt_mesh_add_draw")

    def record(self, renderer, cam, rig, gurney=False):
        """The G-buffer pass (engine.ts:716): cam a MeshCam, rig the [87, 4] Rig uniform."""
        r = np.ascontiguousarray(rig, np.float32)
        assert r.size == 87 * 4
        self.engine._check(self.lib.wt_render_mesh(renderer.r, self.m, ctypes.byref(cam), r.ctypes.data,
                                                   1 if gurney else 0), "wt_render_mesh")

    def close(self):
        if getattr(self, "m", None):
            self.lib.wt_mesh_destroy(self.m)
            self.m = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def draw_struct(d):
    s = _abi.MeshDraw()
    s.color[:] = d.color
    s.metal, s.rough, s.coat, s.alpha_cut = d.metal, d.rough, d.coat, d.alpha_cut
    s.emissive, s.has_tex, s.is_body = d.emissive, 1.0 if d.texture >= 0 else 0.0, d.is_body
    s.first_index, s.count, s.texture = d.first, d.count, d.texture
    s.blend, s.optional = 1 if d.blend else 0, 1 if d.optional else 0
    return s


def draw_words(data, gurney=False):
    """The draws as the oracle's 16-word records (MeshMat, count, texture, blend, unused), in draw order."""
    out = []
    for d in data.draws:
        if d.optional and not gurney:
            continue
        s = draw_struct(d)
        words = np.frombuffer(bytes(s), np.uint32)[:15].copy()
        out.append(np.concatenate([words, np.zeros(1, np.uint32)]))
    return np.array(out, np.uint32).reshape(-1, 16)


# ---------------------------------------------------------------- synthetic stand-in
def _patch(f, nu, nv, uv_scale=(1.0, 1.0)):
    """A parametric surface f(u, v) -> (position [.., 3], normal [.., 3]) on an
    nu x nv grid of cells: (verts [n, 8], local indices)."""
    u, v = np.meshgrid(np.linspace(0.0, 1.0, nu + 1), np.linspace(0.0, 1.0, nv + 1), indexing="ij")
    p, n = f(u, v)
    n = n / np.maximum(np.linalg.norm(n, axis=-1, keepdims=True), 1e-12)
    verts = np.concatenate([p[..., :3], (u * uv_scale[0])[..., None], n, (v * uv_scale[1])[..., None]], axis=-1)
    verts = verts[..., [0, 1, 2, 3, 4, 5, 6, 7]].reshape(-1, 8)
    i = np.arange((nu + 1) * (nv + 1)).reshape(nu + 1, nv + 1)
    a, b, c, d = i[:-1, :-1], i[1:, :-1], i[1:, 1:], i[:-1, 1:]
    tris = np.stack([a, b, c, a, c, d], axis=-1).reshape(-1)
    return verts, tris


def _box(lo, hi, n):
    """The six faces of an axis-aligned box, each n x n cells."""
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    out = []
    for axis in range(3):
        for side in (0, 1):
            a1, a2 = [k for k in range(3) if k != axis]

            def f(u, v, axis=axis, side=side, a1=a1, a2=a2):
                p = np.zeros(u.shape + (3,))
                p[..., axis] = hi[axis] if side else lo[axis]
                p[..., a1] = lo[a1] + u * (hi[a1] - lo[a1])
                p[..., a2] = lo[a2] + v * (hi[a2] - lo[a2])
                nrm = np.zeros(u.shape + (3,))
                nrm[..., axis] = 1.0 if side else -1.0
                return p, nrm
            out.append(_patch(f, n, n))
    return out


def _tub(nu, nt):
    """The body: an elliptic section swept along x, mirrored about z = 0."""
    def f(u, v):
        x = 0.05 + u * 4.85
        th = v * 2.0 * np.pi
        ry = 0.10 + 0.22 * np.sin(np.clip((x - 0.05) / 4.85, 0, 1) * np.pi) ** 0.7
        rz = 0.08 + 0.26 * np.sin(np.clip((x - 0.05) / 4.85, 0, 1) * np.pi) ** 0.5
        cy = 0.30 + 0.14 * np.clip((x - 0.6) / 2.0, 0, 1) - 0.10 * np.clip((x - 3.6) / 1.3, 0, 1)
        p = np.stack([x, cy + ry * np.sin(th), rz * np.cos(th)], axis=-1)
        n = np.stack([np.zeros_like(x), np.sin(th) / ry, np.cos(th) / rz], axis=-1)
        return p, n
    return _patch(f, nu, nt, (4.0, 2.0))


def _wheel(cx, cy, cz, r, hw, n):
    def f(u, v):
        th = u * 2.0 * np.pi
        z = cz - hw + v * 2.0 * hw
        p = np.stack([cx + r * np.cos(th), cy + r * np.sin(th), z], axis=-1)
        return p, np.stack([np.cos(th), np.sin(th), np.zeros_like(th)], axis=-1)
    return _patch(f, n, max(2, n // 6))


def _checker(w, h, cells, c0, c1, alpha=None):
    y, x = np.mgrid[0:h, 0:w]
    on = ((x * cells // w) + (y * cells // h)) % 2 == 1
    img = np.where(on[..., None], np.array(c1, np.uint8), np.array(c0, np.uint8)).astype(np.uint8)
    out = np.empty((h, w, 4), np.uint8)
    out[..., :3] = img
    out[..., 3] = 255 if alpha is None else alpha(x, y)
    return out


def synthetic_rear_stations():
    """Trailing-edge stations of the stand-in's rear flap (the rig's wings.rear[-1])."""
    return [dict(z=z, le=[4.70, 0.99], mid=[4.78, 1.00], te=[4.86, 1.02 + 0.02 * z]) for z in (0.05, 0.2, 0.35, 0.5)]


def synthetic_mesh(detail=1.0):
    """A stand-in car mesh in MeshCar's formats: a textured tub, sidepods (bodywork
    the rig squeezes), a floor of two large triangles, front and rear wings with
    rig-rotated flaps (parts 1-4) and static parts in their assemblies, a strip
    joining the front wing to the nose (so detach_seams has work), four wheels
    (is_body 0), an emissive light, two overlapping textured decals (blended) and
    the gurney tab.  `detail` scales the tessellation (1.0: about 20k triangles)."""
    k = max(0.25, float(detail))
    parts = []   # (verts, local indices, tag, group)

    def add(vi, tag, group):
        parts.append((vi[0].astype(np.float64), vi[1], tag, group))

    add(_tub(int(96 * k), int(48 * k)), 0, "body")
    for zs in (1.0, -1.0):
        lo, hi = (2.0, 0.15, 0.25), (3.9, 0.62, 0.62)
        for f in _box((lo[0], lo[1], min(zs * lo[2], zs * hi[2])), (hi[0], hi[1], max(zs * lo[2], zs * hi[2])),
                      max(2, int(10 * k))):
            add(f, 0, "pods")
    floor = (np.array([[1.2, 0.05, -0.7, 0, 0, 1, 0, 0], [4.6, 0.05, -0.7, 1, 0, 1, 0, 0],
                       [4.6, 0.05, 0.7, 1, 0, 1, 0, 1], [1.2, 0.05, 0.7, 0, 0, 1, 0, 1]], np.float64),
             np.array([0, 1, 2, 0, 2, 3]))
    add(floor, 0, "floor")
    nw = max(2, int(12 * k))
    for zs in (1.0, -1.0):
        z0, z1 = sorted((zs * 0.02, zs * 0.95))
        for f in _box((0.0, 0.10, z0), (0.45, 0.125, z1), nw):
            add(f, 8, "fwing")                 # front wing main plane: assembly 1, static
        z0, z1 = sorted((zs * 0.14, zs * 0.58))
        for f in _box((0.25, 0.16, z0), (0.42, 0.175, z1), nw):
            add(f, 9, "fwing")                 # flap A
        for f in _box((0.36, 0.22, z0), (0.50, 0.232, z1), nw):
            add(f, 10, "fwing")                # flap B
        z0, z1 = sorted((zs * 0.0, zs * 0.53))
        for f in _box((4.55, 0.84, z0), (4.75, 0.87, z1), nw):
            add(f, 20, "rwing")                # rear main plane: part 4
        for f in _box((4.70, 0.97, z0), (4.86, 0.99, z1), nw):
            add(f, 19, "rwing")                # rear flap: part 3
        z0, z1 = sorted((zs * 0.53, zs * 0.56))
        for f in _box((4.45, 0.45, z0), (4.95, 1.10, z1), nw):
            add(f, 16, "rwing")                # endplate: assembly 2, static
    # a strip from the nose tip (body) to the wing's main plane (front wing): mixed assemblies
    strip = (np.array([[0.10, 0.22, -0.05, 0, 0, 1, 0, 0], [0.10, 0.22, 0.05, 1, 0, 1, 0, 0],
                       [0.20, 0.125, -0.05, 0, 0, 1, 0, 1], [0.20, 0.125, 0.05, 1, 0, 1, 0, 1]], np.float64),
             np.array([0, 1, 2, 1, 3, 2]))
    strip_tags = np.array([0, 0, 8, 8], np.uint8)
    for (cx, cz) in ((1.0, 0.779), (1.0, -0.779), (4.4, 0.737), (4.4, -0.737)):
        add(_wheel(cx, 0.36, cz, 0.355, 0.18, max(8, int(32 * k))), 0, "wheels")
    light = (np.array([[4.96, 0.40, -0.04, 0, 1, 0, 0, 0], [4.96, 0.40, 0.04, 1, 1, 0, 0, 0],
                       [4.96, 0.46, 0.04, 1, 1, 0, 0, 1], [4.96, 0.46, -0.04, 0, 1, 0, 0, 1]], np.float64),
             np.array([0, 1, 2, 0, 2, 3]))
    add(light, 0, "light")

    def decal(x0, x1, lift, nu):
        def f(u, v):
            x = x0 + u * (x1 - x0)
            th = 0.25 * np.pi + v * 0.5 * np.pi
            ry = 0.10 + 0.22 * np.sin(np.clip((x - 0.05) / 4.85, 0, 1) * np.pi) ** 0.7 + lift
            rz = 0.08 + 0.26 * np.sin(np.clip((x - 0.05) / 4.85, 0, 1) * np.pi) ** 0.5 + lift
            cy = 0.30 + 0.14 * np.clip((x - 0.6) / 2.0, 0, 1) - 0.10 * np.clip((x - 3.6) / 1.3, 0, 1)
            return (np.stack([x, cy + ry * np.sin(th), rz * np.cos(th)], axis=-1),
                    np.stack([np.zeros_like(x), np.sin(th) / ry, np.cos(th) / rz], axis=-1))
        return _patch(f, nu, max(2, nu // 2))
    add(decal(1.2, 2.2, 0.0005, max(4, int(24 * k))), 0, "decal_a")
    add(decal(1.7, 2.9, 0.0010, max(4, int(24 * k))), 0, "decal_b")

    verts, idx, tags, ranges = [], [], [], {}
    vbase = 0
    groups = ["body", "pods", "floor", "fwing", "rwing", "wheels", "light", "decal_a", "decal_b"]
    for g in groups:
        first = sum(len(i) for i in idx)
        for (v, i, tag, grp) in parts:
            if grp != g:
                continue
            verts.append(v)
            idx.append(i + vbase)
            tags.append(np.full(v.shape[0], tag, np.uint8))
            vbase += v.shape[0]
        if g == "fwing":
            verts.append(strip[0])
            idx.append(strip[1] + vbase)
            tags.append(strip_tags)
            vbase += 4
        ranges[g] = (first, sum(len(i) for i in idx) - first)
    gv, gi = gurney_geometry(synthetic_rear_stations())
    first = sum(len(i) for i in idx)
    verts.append(gv.astype(np.float64))
    idx.append(gi.astype(np.int64) + vbase)
    tags.append(np.full(gv.shape[0], REAR_FLAP | (REAR_WING << ASSEMBLY_SHIFT), np.uint8))
    ranges["gurney"] = (first, gi.size)
    verts = np.concatenate(verts).astype(np.float32)
    indices = np.concatenate(idx).astype(np.uint32)
    tags = np.concatenate(tags)
    verts, tags = detach_seams(verts, indices, tags)
    textures = [
        (64, 64, _checker(64, 64, 8, (40, 200, 190), (20, 24, 30))),
        (48, 20, _checker(48, 20, 6, (230, 230, 235), (200, 30, 40),
                          alpha=lambda x, y: np.clip((x * 255) // 47, 0, 255).astype(np.uint8))),
        (32, 32, _checker(32, 32, 4, (250, 190, 20), (10, 10, 10),
                          alpha=lambda x, y: np.where((x // 8 + y // 8) % 2 == 0, 255, 0).astype(np.uint8))),
    ]
    mat = dict(alpha_cut=0.0, emissive=0.0, is_body=1.0)
    draws = [
        DrawSpec("mercedes_paint.007", (1.0, 1.0, 1.0, 1.0), 0.6, 0.25, 1.0, first=ranges["body"][0],
                 count=ranges["body"][1], texture=0, **mat),
        DrawSpec("mercedes_carbon1.007", (0.03, 0.03, 0.035, 1.0), 0.3, 0.4, 0.6, first=ranges["pods"][0],
                 count=ranges["pods"][1], **mat),
        DrawSpec("generics.007", (0.02, 0.02, 0.02, 1.0), 0.0, 0.7, 0.2, first=ranges["floor"][0],
                 count=ranges["floor"][1], **mat),
        DrawSpec("mercedes_carbon2.005", (0.04, 0.04, 0.045, 1.0), 0.3, 0.35, 0.6, first=ranges["fwing"][0],
                 count=ranges["fwing"][1], **mat),
        DrawSpec("sw_carbon.003", (0.05, 0.05, 0.05, 1.0), 0.3, 0.35, 0.6, first=ranges["rwing"][0],
                 count=ranges["rwing"][1], **mat),
        DrawSpec("tread_medium.007", (0.08, 0.08, 0.09, 1.0), 0.0, 0.8, 0.2, alpha_cut=0.0, emissive=0.0,
                 is_body=0.0, first=ranges["wheels"][0], count=ranges["wheels"][1]),
        DrawSpec("rear_light_2.007", (0.9, 0.05, 0.05, 1.0), 0.0, 0.3, 0.2, alpha_cut=0.0, emissive=1.5, is_body=1.0,
                 first=ranges["light"][0], count=ranges["light"][1]),
        DrawSpec("mercedes_decals.005", (1.0, 1.0, 1.0, 1.0), 0.0, 0.5, 0.2, alpha_cut=0.02, emissive=0.0,
                 is_body=1.0, first=ranges["decal_a"][0], count=ranges["decal_a"][1], texture=1, blend=True),
        DrawSpec("sw_decals.003", (1.0, 0.9, 0.8, 0.9), 0.0, 0.5, 0.2, alpha_cut=0.02, emissive=0.0, is_body=1.0,
                 first=ranges["decal_b"][0], count=ranges["decal_b"][1], texture=2, blend=True),
        DrawSpec("gurney", first=ranges["gurney"][0], count=ranges["gurney"][1], optional=True, **GURNEY_MAT),
    ]
    for d in draws:  # MeshCar's clamps (mesh-car.ts:150-158)
        d.metal = min(d.metal, 0.9)
        d.rough = max(d.rough, 0.05)
    return MeshData(verts, indices, tags, draws, textures)
