"""Seeded synthetic scenes for the rasteriser hot path.

Each scene holds a mesh in the reference's layouts (canmom/rasteriser ``face.h:6-13`` Triangle =
vertices[3], normals[3], uvs[3], material as 10 int32; vec3 positions / normals; vec2 uvs), the
reference's ``Light`` records (direction, intensity, colour; ``light.h:7-14``) and the ``Args``
fields the frame depends on (``arguments.h:7-21``).

The generators use only IEEE-exact numpy arithmetic (+, -, *, /, sqrt, floor) and integer random
streams, with sine, cosine and exp evaluated by fixed polynomials here rather than by the
platform's libm, so the same seed gives the same float32 meshes bit for bit on x86 and aarch64.
"""
from __future__ import annotations

import dataclasses
import hashlib
import math

import numpy as np

# ----------------------------------------------------------------------------------------------
# deterministic elementary functions (float64, fixed operation order, no libm)
# ----------------------------------------------------------------------------------------------
_TWO_PI = 6.283185307179586
_PI = 3.141592653589793
_HALF_PI = 1.5707963267948966


def _poly(x, coeffs):
    acc = np.full_like(x, coeffs[0])
    for c in coeffs[1:]:
        acc = acc * x
        acc = acc + c
    return acc


# Taylor coefficients of sin(x)/x and cos(x) in x^2, highest order first; |x| <= pi/4 after
# reduction keeps the truncation error below 1e-17.
_SIN_C = [(-1.0) ** k / math.factorial(2 * k + 1) for k in range(10, -1, -1)]
_COS_C = [(-1.0) ** k / math.factorial(2 * k) for k in range(10, -1, -1)]


def det_sincos(theta):
    """sin and cos of float64 ``theta`` by quadrant reduction plus a fixed Taylor polynomial."""
    t = np.asarray(theta, dtype=np.float64)
    q = np.floor(t / _HALF_PI + 0.5)
    r = t - q * _HALF_PI
    r2 = r * r
    s = _poly(r2, _SIN_C) * r
    c = _poly(r2, _COS_C)
    qi = np.mod(q, 4.0).astype(np.int64)
    sin_out = np.select([qi == 0, qi == 1, qi == 2, qi == 3], [s, c, -s, -c])
    cos_out = np.select([qi == 0, qi == 1, qi == 2, qi == 3], [c, -s, -c, s])
    return sin_out, cos_out


_LN2 = 0.6931471805599453
_EXP_C = [1.0 / math.factorial(k) for k in range(16, -1, -1)]


def det_exp(x):
    """exp of float64 ``x`` by 2^k scaling plus a fixed Taylor polynomial on |r| <= ln2/2."""
    t = np.asarray(x, dtype=np.float64)
    k = np.floor(t / _LN2 + 0.5)
    r = t - k * _LN2
    return np.ldexp(_poly(r, _EXP_C), k.astype(np.int64))


def _normalise_rows(v):
    n = np.sqrt(v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2])
    return v / n[:, None]


def _cross(a, b):
    return np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
                     a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                     a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], axis=1)


def _irwin_hall_normal(rng, n):
    """Approximately standard normal samples: the sum of 12 uniforms minus 6."""
    u = rng.random((n, 12))
    acc = u[:, 0].copy()
    for k in range(1, 12):
        acc = acc + u[:, k]
    return acc - 6.0


# ----------------------------------------------------------------------------------------------
# scene container
# ----------------------------------------------------------------------------------------------
@dataclasses.dataclass
class Scene:
    name: str
    pos: np.ndarray            # (nv, 3) float32
    tris: np.ndarray           # (ntri, 10) int32
    nrm: np.ndarray            # (nn, 3) float32
    uv: np.ndarray             # (nuv, 2) float32
    kd: np.ndarray             # (nmat, 3) float32
    lights: np.ndarray         # (nl, 7) float32: direction xyz, intensity, colour rgb
    width: int = 540
    height: int = 304
    wind_clockwise: bool = False
    scale: float = 1.0
    disp: tuple = (0.0, 0.0, 0.0)
    angles: tuple = (0.0, 0.0, 0.0)   # rx, ry, rz (YXZ Tait-Bryan)
    fovy_deg: float = 45.0
    z_near: float = 0.1
    z_far: float = 6.0
    vertex_albedo: object = None      # (nv, 3) float32 per-vertex albedo in place of Kd, or None

    def with_view(self, **kw):
        return dataclasses.replace(self, **kw)

    @property
    def ntri(self):
        return int(self.tris.shape[0])

    def mesh_digest(self):
        h = hashlib.sha256()
        for a in (self.pos, self.tris, self.nrm, self.uv, self.kd, self.lights):
            h.update(np.ascontiguousarray(a).tobytes())
        va = getattr(self, "vertex_albedo", None)
        if va is not None:
            h.update(b"vertex_albedo")
            h.update(np.ascontiguousarray(va).tobytes())
        return h.hexdigest()


def _tri_records(v, n=None, uv=None, mat=None):
    """Pack (ntri, 3) vertex / normal / uv index arrays and material ids into (ntri, 10) int32."""
    ntri = v.shape[0]
    out = np.empty((ntri, 10), dtype=np.int32)
    out[:, 0:3] = v
    out[:, 3:6] = v if n is None else n
    out[:, 6:9] = -1 if uv is None else uv
    out[:, 9] = 0 if mat is None else mat
    return out


def rig_three_point(light_scale=255.0):
    """Three directional lights: key (1,-1,-1) white 1.0, fill (-1,-0.5,-1) warm 0.5,
    back (0,0,1) cool 0.3; intensities multiplied by ``light_scale`` because the reference's
    shading output is on a 0-255 scale (shading.cpp:20-34)."""
    return np.array([[1, -1, -1, 1.0 * light_scale, 1, 1, 1],
                     [-1, -0.5, -1, 0.5 * light_scale, 1, 0.9, 0.7],
                     [0, 0, 1, 0.3 * light_scale, 0.7, 0.8, 1]], dtype=np.float32)


def rig_threepoint_csv():
    """The reference's sampledata/threepoint.csv light rig."""
    return np.array([[1, -0.5, -1, 512, 1, 1, 0.9],
                     [-1, 0, -1, 256, 1, 1, 0.5],
                     [1, 0, 1, 100, 0, 0, 1]], dtype=np.float32)


def rig_random(n, seed, light_scale=255.0):
    """``n`` lights: directions uniform on the sphere, intensity Exp(1)/n times ``light_scale``,
    colours uniform in [0, 1]^3."""
    rng = np.random.default_rng(seed)
    z = rng.random(n) * 2.0 - 1.0
    phi = rng.random(n) * _TWO_PI
    s, c = det_sincos(phi)
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    d = np.stack([r * c, r * s, z], axis=1)
    u = rng.random(n)
    inten = -np.log1p(-u) / n * light_scale  # only the light rig uses libm log; it is stored
    col = rng.random((n, 3))
    return np.concatenate([d, inten[:, None], col], axis=1).astype(np.float32)


# ----------------------------------------------------------------------------------------------
# meshes
# ----------------------------------------------------------------------------------------------
def square_scene():
    """renderer.cpp:32-50 add_square: two triangles, one normal, four uvs, white material."""
    pos = np.array([[-0.5, -0.5, 0], [0.5, -0.5, 0], [-0.5, 0.5, 0], [0.5, 0.5, 0]], np.float32)
    tris = np.array([[0, 1, 2, 0, 0, 0, 0, 1, 2, 0], [2, 1, 3, 0, 0, 0, 2, 1, 3, 0]], np.int32)
    return Scene("square", pos, tris, np.array([[0, 0, 1]], np.float32),
                 np.array([[0, 0], [1, 0], [0, 1], [1, 1]], np.float32),
                 np.array([[1, 1, 1]], np.float32), rig_threepoint_csv())


def plane_scene():
    """sampledata/plane.obj as tinyobjloader fan-triangulates it (face 1//1 2//1 4//1 3//1 ->
    (1,2,4), (1,4,3)), with plane.mtl's Kd 0.8."""
    pos = np.array([[-1, -1, 0], [1, -1, 0], [-1, 1, 0], [1, 1, 0]], np.float32)
    tris = np.array([[0, 1, 3, 0, 0, 0, -1, -1, -1, 0], [0, 3, 2, 0, 0, 0, -1, -1, -1, 0]], np.int32)
    return Scene("plane", pos, tris, np.array([[0, 0, 1]], np.float32), np.zeros((0, 2), np.float32),
                 np.array([[0.8, 0.8, 0.8]], np.float32), rig_threepoint_csv())


def icosphere(level, kd=(0.8, 0.8, 0.8)):
    """Subdivided icosahedron on the unit sphere; vertex normals are the normalised positions and
    share the vertex indices; faces wind anticlockwise seen from outside. Level 4: 2562 vertices,
    5120 triangles."""
    phi = (1.0 + math.sqrt(5.0)) / 2.0
    v = [(-1, phi, 0), (1, phi, 0), (-1, -phi, 0), (1, -phi, 0), (0, -1, phi), (0, 1, phi),
         (0, -1, -phi), (0, 1, -phi), (phi, 0, -1), (phi, 0, 1), (-phi, 0, -1), (-phi, 0, 1)]
    verts = [tuple(x) for x in _normalise_rows(np.array(v, np.float64))]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(level):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                pa, pb = verts[a], verts[b]
                m = np.array([[(pa[0] + pb[0]) / 2, (pa[1] + pb[1]) / 2, (pa[2] + pb[2]) / 2]])
                verts.append(tuple(_normalise_rows(m)[0]))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    p64 = np.array(verts, np.float64)
    f = np.array(faces, np.int64)
    f = _orient_outward(p64, f)
    pos = p64.astype(np.float32)
    return Scene(f"icosphere{level}", pos, _tri_records(f), pos.copy(), np.zeros((0, 2), np.float32),
                 np.array([kd], np.float32), rig_three_point())


def _orient_outward(p64, f):
    a, b, c = p64[f[:, 0]], p64[f[:, 1]], p64[f[:, 2]]
    nrm = _cross(b - a, c - a)
    cen = a + b + c
    d = nrm[:, 0] * cen[:, 0] + nrm[:, 1] * cen[:, 1] + nrm[:, 2] * cen[:, 2]
    flip = d < 0
    f = f.copy()
    f[flip, 1], f[flip, 2] = f[flip, 2].copy(), f[flip, 1].copy()
    return f


def uv_sphere(n_lon=1024, n_lat=512, seed=1, sigma=0.02, flat=True, kd=(0.8, 0.8, 0.8),
              vertex_albedo=False):
    """UV sphere with ``n_lon`` x ``n_lat`` segments: 2 poles + (n_lat-1) rings of n_lon vertices;
    each vertex radius is 1 + sigma*N(0,1) from ``seed``. With ``flat`` every face gets its own
    normal (one `vn` per face, as an OBJ with per-face normals); otherwise vertex normals are the
    normalised positions. 1024 x 512: 523,266 vertices and 1,046,528 triangles."""
    rng = np.random.default_rng(seed)
    ring = np.arange(1, n_lat, dtype=np.float64)
    st, ct = det_sincos(ring * (_PI / n_lat))
    sp, cp = det_sincos(np.arange(n_lon, dtype=np.float64) * (_TWO_PI / n_lon))
    body = np.stack([st[:, None] * cp[None, :], np.broadcast_to(ct[:, None], (n_lat - 1, n_lon)),
                     st[:, None] * sp[None, :]], axis=2).reshape(-1, 3)
    unit = np.concatenate([[[0.0, 1.0, 0.0]], body, [[0.0, -1.0, 0.0]]], axis=0)
    nv = unit.shape[0]
    radius = 1.0 + sigma * _irwin_hall_normal(rng, nv)
    p64 = unit * radius[:, None]
    south = nv - 1

    def rid(j, i):  # ring j in [0, n_lat-2], column i (wraps)
        return 1 + j * n_lon + (i % n_lon)

    i = np.arange(n_lon)
    faces = [np.stack([np.zeros(n_lon, np.int64), rid(0, i + 1), rid(0, i)], axis=1)]
    for j in range(n_lat - 2):
        a, b, c, d = rid(j, i), rid(j, i + 1), rid(j + 1, i), rid(j + 1, i + 1)
        faces.append(np.stack([a, b, c], axis=1))
        faces.append(np.stack([b, d, c], axis=1))
    faces.append(np.stack([np.full(n_lon, south, np.int64), rid(n_lat - 2, i), rid(n_lat - 2, i + 1)], axis=1))
    # Winding comes from the undisplaced sphere, so it is a property of the grid; the radius noise
    # then tilts facets and some face away from the camera, as on a real displaced surface.
    f = _orient_outward(unit, np.concatenate(faces, axis=0))
    pos = p64.astype(np.float32)
    if flat:
        a, b, c = p64[f[:, 0]], p64[f[:, 1]], p64[f[:, 2]]
        nrm = _normalise_rows(_cross(b - a, c - a)).astype(np.float32)
        nidx = np.repeat(np.arange(f.shape[0], dtype=np.int64)[:, None], 3, axis=1)
    else:
        nrm = _normalise_rows(unit).astype(np.float32)
        nidx = f
    kdarr = np.array([kd], np.float32)
    tris = _tri_records(f, nidx)
    sc = Scene(f"uvsphere{n_lon}x{n_lat}", pos, tris, nrm, np.zeros((0, 2), np.float32), kdarr,
               rig_three_point())
    if vertex_albedo:
        sc.vertex_albedo = rng.random((nv, 3)).astype(np.float32)
    return sc


def soup(n_tris, width, height, seed=2, fovy_deg=60.0, depth_range=(2.0, 50.0),
         area_range=(0.5, 500.0), back_fraction=0.5, kd=(0.8, 0.8, 0.8)):
    """Independent triangles: camera-space depth uniform in ``depth_range``, centroid uniform over
    the screen, screen area log-uniform in ``area_range`` px^2, random shape and rotation built in
    raster space and unprojected (model = identity, camera at z=+3 looking down -z), a
    ``back_fraction`` of them wound back-facing, and one flat normal per face."""
    rng = np.random.default_rng(seed)
    n = int(n_tris)
    W, H = float(width), float(height)
    aspect = W / H
    sh, ch = det_sincos(np.array(fovy_deg * _PI / 360.0))
    tan_half = float(sh / ch)
    d = depth_range[0] + (depth_range[1] - depth_range[0]) * rng.random(n)
    cx = rng.random(n) * W
    cy = rng.random(n) * H
    la, lb = math.log(area_range[0]), math.log(area_range[1])
    area = det_exp(la + (lb - la) * rng.random(n))
    a0 = rng.random(n) * _TWO_PI
    ang = a0[:, None] + np.array([0.0, _TWO_PI / 3, 2 * _TWO_PI / 3])[None, :] + (rng.random((n, 3)) - 0.5)
    rad = 0.5 + rng.random((n, 3))
    s, c = det_sincos(ang)
    ox, oy = rad * c, rad * s
    shape_area = 0.5 * np.abs((ox[:, 1] - ox[:, 0]) * (oy[:, 2] - oy[:, 0]) -
                              (ox[:, 2] - ox[:, 0]) * (oy[:, 1] - oy[:, 0]))
    k = np.sqrt(area / shape_area)
    X = cx[:, None] + ox * k[:, None]
    Y = cy[:, None] + oy * k[:, None]
    # Increasing angle in raster space (y down) gives a negative signed_area_2d: back-facing.
    front = rng.random(n) >= back_fraction
    order = np.where(front[:, None], np.array([[0, 2, 1]]), np.array([[0, 1, 2]]))
    X = np.take_along_axis(X, order, axis=1)
    Y = np.take_along_axis(Y, order, axis=1)
    dk = d[:, None] * (1.0 + 0.1 * (rng.random((n, 3)) - 0.5))
    ndx = 2.0 * X / W - 1.0
    ndy = 1.0 - 2.0 * Y / H
    px = ndx * dk * tan_half * aspect
    py = ndy * dk * tan_half
    pz = 3.0 - dk
    p64 = np.stack([px, py, pz], axis=2).reshape(-1, 3)
    a, b, cc = p64[0::3], p64[1::3], p64[2::3]
    nrm = _normalise_rows(_cross(b - a, cc - a)).astype(np.float32)
    v = np.arange(3 * n, dtype=np.int64).reshape(n, 3)
    nidx = np.repeat(np.arange(n, dtype=np.int64)[:, None], 3, axis=1)
    sc = Scene(f"soup{n}", p64.astype(np.float32), _tri_records(v, nidx), nrm,
               np.zeros((0, 2), np.float32), np.array([kd], np.float32), rig_three_point(),
               width=int(width), height=int(height), fovy_deg=fovy_deg, z_near=0.1, z_far=100.0)
    return sc


# ----------------------------------------------------------------------------------------------
# the named workloads
# ----------------------------------------------------------------------------------------------
CAMERA = dict(fovy_deg=60.0, z_near=0.1, z_far=100.0)


def config_icosphere_small():
    """Icosphere level 4 (5,120 triangles), 640x480, smooth, anticlockwise, ry = 0.5 rad."""
    return icosphere(4).with_view(width=640, height=480, angles=(0.0, 0.5, 0.0), **CAMERA)


def config_displaced_sphere(n_lon=1024, n_lat=512, width=1920, height=1080, seed=1):
    """Displaced UV sphere (1,046,528 triangles at 1024x512), flat normals, 1920x1080."""
    return uv_sphere(n_lon, n_lat, seed=seed).with_view(width=width, height=height, **CAMERA)


def spin_angles(frame, step=1.0 / 60.0):
    """Model rotation of spin frame ``frame``: ry advances by ``step`` rad per frame (1 rad/s at
    60 frames/s, the reference's spin loop with a fixed step; renderer.cpp:94-125)."""
    return (0.0, float(np.float32(frame * step)), 0.0)


def config_soup(n_tris=4_000_000, width=3840, height=2160, seed=2):
    """Overdraw-heavy triangle soup (4M triangles at 3840x2160)."""
    return soup(n_tris, width, height, seed=seed)


def with_spherical_uvs(sc, scale=1.0, offset=0.0):
    """The scene with one uv per vertex from its direction (u = atan2(z, x) / 2pi + 1/2,
    v = asin(y / |p|) / pi + 1/2, times `scale` plus `offset`, so uvs outside 0..1 can be asked for)
    and every triangle's uv indices equal to its vertex indices."""
    p = sc.pos.astype(np.float64)
    r = np.sqrt((p * p).sum(axis=1))
    r[r == 0] = 1.0
    u = np.arctan2(p[:, 2], p[:, 0]) / _TWO_PI + 0.5
    v = np.arcsin(np.clip(p[:, 1] / r, -1.0, 1.0)) / _PI + 0.5
    uv = (np.stack([u, v], axis=1) * scale + offset).astype(np.float32)
    tris = sc.tris.copy()
    tris[:, 6:9] = tris[:, 0:3]
    return dataclasses.replace(sc, uv=uv, tris=tris)


def config_many_lights(n_lon=1024, n_lat=512, width=1920, height=1080, n_lights=256, seed=4, light_seed=5):
    """Many-light shading workload: the displaced sphere with smooth normals (the normalised unit
    positions), per-vertex albedo uniform in [0,1]^3 and ``n_lights`` directional lights from
    rig_random (directions uniform on the sphere, intensity Exp(1)/n * 255, colours uniform)."""
    sc = uv_sphere(n_lon, n_lat, seed=seed, flat=False, vertex_albedo=True)
    return sc.with_view(width=width, height=height, lights=rig_random(n_lights, light_seed), **CAMERA)


def batch_workload(seed=3, n_frames=256, n_soups=16):
    """The uneven batch: icospheres L2-L7 and seeded soups of 1k-500k triangles (log-uniform sizes);
    each frame picks a mesh uniformly, a resolution from {256x256, 640x480, 1280x720, 1920x1080},
    random rx/ry and a 1-8 light rig. Returns (meshes, frames); a frame is (mesh index, width,
    height, angles, lights)."""
    rng = np.random.default_rng(seed)
    meshes = [icosphere(l) for l in range(2, 8)]
    for k in range(n_soups):
        n = int(round(float(det_exp(np.log(1000.0) + (np.log(500000.0) - np.log(1000.0)) * rng.random()))))
        meshes.append(soup(n, 1280, 720, seed=1000 + k))
    sizes = [(256, 256), (640, 480), (1280, 720), (1920, 1080)]
    frames = []
    for i in range(n_frames):
        mi = int(rng.integers(len(meshes)))
        W, H = sizes[int(rng.integers(4))]
        nl = int(rng.integers(1, 9))
        angles = (float(rng.uniform(-np.pi, np.pi)), float(rng.uniform(-np.pi, np.pi)), 0.0)
        frames.append((mi, W, H, angles, rig_random(nl, seed=10_000 + i)))
    return meshes, frames


def batch_frame_scene(meshes, frame):
    """The Scene one batch frame draws (60 deg / 0.1 / 100 projection)."""
    mi, W, H, angles, lights = frame
    return meshes[mi].with_view(width=W, height=H, angles=angles, lights=lights, fovy_deg=60.0, z_near=0.1,
                                z_far=100.0)

