"""Oracle test infrastructure: ctypes bindings for the two CPU checkers.

- ``Port``: the C restatement of the reference's draw_frame (oracle/rast_oracle.c), built into
  oracle/_build/liboracle.so. It runs anywhere this repository is built.
- ``Reference``: canmom/rasteriser's own drawing.cpp / geometry.cpp / shading.cpp compiled from the
  reference tree (oracle/Makefile ``ref``) into oracle/_ref/libref.so, with ref_harness.cpp. It
  exists only where the reference sources were present at build time.

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")
# The canmom/rasteriser source tree the reference oracle compiles from: RAST_REFERENCE, else the
# place this build's container mounts it. Absent on hosts without the reference sources.
REFERENCE_TREE = os.environ.get("RAST_REFERENCE") or "/root/reference"


def reference_tree():
    """The reference source tree, or None where it is not present."""
    return REFERENCE_TREE if os.path.isdir(os.path.join(REFERENCE_TREE, "headers")) else None


def build(with_reference=None, quiet=True):
    """Compile the port, and the reference when its sources are present."""
    if with_reference is None:
        with_reference = reference_tree() is not None
    targets = ["port"] + (["ref"] if with_reference else [])
    out = None if not quiet else subprocess.DEVNULL
    subprocess.run(["make", "-C", HERE, "-j8", f"REF={REFERENCE_TREE}"] + targets, check=True, stdout=out)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _p(a, t=C.c_float):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


class _OracleFrame(C.Structure):
    _fields_ = [("pos", C.POINTER(C.c_float)), ("nv", C.c_int64),
                ("tris", C.POINTER(C.c_int32)), ("ntri", C.c_int64),
                ("nrm", C.POINTER(C.c_float)), ("nn", C.c_int64),
                ("uv", C.POINTER(C.c_float)), ("nuv", C.c_int64),
                ("kd", C.POINTER(C.c_float)), ("nmat", C.c_int32),
                ("camera", C.POINTER(C.c_float)), ("normal_matrix", C.POINTER(C.c_float)),
                ("lights", C.POINTER(C.c_float)), ("nl", C.c_int32),
                ("width", C.c_uint32), ("height", C.c_uint32), ("wind_clockwise", C.c_int32),
                ("vcol", C.POINTER(C.c_float)), ("tex", C.POINTER(C.c_float)), ("tex_off", C.POINTER(C.c_int64)),
                ("tex_wh", C.POINTER(C.c_int32)), ("flat", C.c_int32)]


def cimg_normalize01(texels):
    """material.h:21 `diffuse_texture.normalize(0.f, 1.f)` (CImg, float): m, M over every value;
    (v - m) / (M - m) * (1 - 0) + 0, or 0 everywhere when m == M."""
    t = np.ascontiguousarray(texels, np.float32)
    m, M = np.float32(t.min()), np.float32(t.max())
    if m == M:
        return np.zeros_like(t)
    if m == 0 and M == 1:
        return t.copy()
    return (((t - m) / (M - m)) * np.float32(1.0) + np.float32(0.0)).astype(np.float32)


class Port:
    """The C restatement. ``draw`` takes the frame's matrices and already-transformed lights."""

    def __init__(self, path=PORT_SO):
        if not os.path.exists(path):
            build(with_reference=False)
        self.lib = C.CDLL(path)
        self.lib.oracle_draw_frame.restype = C.c_int
        self.lib.oracle_draw_frame.argtypes = [C.POINTER(_OracleFrame), C.POINTER(C.c_uint8),
                                               C.POINTER(C.c_float), C.POINTER(C.c_uint32),
                                               C.POINTER(C.c_uint64)]
        self.lib.oracle_raster_vertices.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int64,
                                                    C.c_uint32, C.c_uint32, C.POINTER(C.c_float)]
        self.lib.oracle_shade.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                          C.c_int32, C.POINTER(C.c_uint32)]
        self.lib.oracle_frame_matrices.restype = C.c_int
        self.lib.oracle_frame_matrices.argtypes = [C.c_uint32, C.c_uint32, C.c_float, C.POINTER(C.c_float),
                                                   C.POINTER(C.c_float), C.c_float, C.c_float, C.c_float] + \
            [C.POINTER(C.c_float)] * 5
        self.lib.oracle_transform_lights.restype = C.c_int
        self.lib.oracle_transform_lights.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int32,
                                                     C.POINTER(C.c_float)]

    def draw(self, scene, camera, normal_matrix, lights7, frame=None, depth=None, want_ids=True, textures=None,
             flat=False):
        """Returns (frame (3,H,W) uint8, depth (H,W) float32, ids (H,W) uint32 or None, stats).
        textures: per material a normalised (c>=3, h, w) float32 texture or None. flat: face
        normals in place of the vertex normals (Args::flat)."""
        W, H = scene.width, scene.height
        frame = np.zeros((3, H, W), np.uint8) if frame is None else np.ascontiguousarray(frame, np.uint8).copy()
        depth = np.ones((H, W), np.float32) if depth is None else _f32(depth).copy()
        ids = np.full((H, W), 0xFFFFFFFF, np.uint32) if want_ids else None
        keep = [_f32(scene.pos), _i32(scene.tris), _f32(scene.nrm), _f32(scene.uv), _f32(scene.kd),
                _f32(camera), _f32(normal_matrix), _f32(lights7)]
        vcol = getattr(scene, "vertex_albedo", None)
        vcol = _f32(vcol) if vcol is not None else None
        tex = off = wh = None
        if textures is not None:
            parts, off, wh, at = [], np.full(len(textures), -1, np.int64), np.zeros(2 * len(textures), np.int32), 0
            for i, t in enumerate(textures):
                if t is None:
                    continue
                t = _f32(t)
                off[i], wh[2 * i], wh[2 * i + 1] = at, t.shape[2], t.shape[1]
                parts.append(t[:3].ravel())
                at += parts[-1].size
            tex = np.concatenate(parts) if parts else np.zeros(1, np.float32)
        f = _OracleFrame(_p(keep[0]), scene.pos.shape[0], _p(keep[1], C.c_int32), scene.tris.shape[0],
                         _p(keep[2]), scene.nrm.shape[0], _p(keep[3]), scene.uv.shape[0],
                         _p(keep[4]), scene.kd.shape[0], _p(keep[5]), _p(keep[6]), _p(keep[7]),
                         keep[7].shape[0], W, H, int(scene.wind_clockwise), _p(vcol), _p(tex),
                         _p(off, C.c_int64), _p(wh, C.c_int32), int(bool(flat)))
        stats = np.zeros(4, np.uint64)
        rc = self.lib.oracle_draw_frame(C.byref(f), _p(frame, C.c_uint8), _p(depth),
                                        _p(ids, C.c_uint32), _p(stats, C.c_uint64))
        if rc != 0:
            raise RuntimeError("oracle_draw_frame failed")
        return frame, depth, ids, stats

    def matrices(self, width, height, scale, disp, angles, fovy_deg, z_near, z_far):
        """dict of model, view, modelview, camera, normal (each (16,) float32, column major):
        drawing.cpp:221-229 with the given projection (the C restatement)."""
        out = {k: np.zeros(16, np.float32) for k in ("model", "view", "modelview", "camera", "normal")}
        rc = self.lib.oracle_frame_matrices(width, height, scale, _p(_f32(disp)), _p(_f32(angles)), fovy_deg,
                                            z_near, z_far, *[_p(out[k]) for k in out])
        if rc != 0:
            raise RuntimeError("oracle_frame_matrices: bad argument")
        return out

    def transform_lights(self, view, lights7):
        """Light::transform of every (direction, intensity, rgb) record (geometry.cpp:124-133)."""
        li = _f32(lights7).reshape(-1, 7)
        out = np.empty_like(li)
        if self.lib.oracle_transform_lights(_p(_f32(view)), _p(li), li.shape[0], _p(out)) != 0:
            raise RuntimeError("oracle_transform_lights: bad argument")
        return out

    def frame_inputs(self, scene):
        """(camera, normal matrix, transformed lights, matrices) of a scene's frame, all from the
        C restatement."""
        m = self.matrices(scene.width, scene.height, scene.scale, scene.disp, scene.angles, scene.fovy_deg,
                          scene.z_near, scene.z_far)
        return m["camera"], m["normal"], self.transform_lights(m["view"], scene.lights), m

    def raster_vertices(self, camera, pos, width, height):
        pos = _f32(pos)
        out = np.empty((pos.shape[0], 4), np.float32)
        self.lib.oracle_raster_vertices(_p(_f32(camera)), _p(pos), pos.shape[0], width, height, _p(out))
        return out

    def shade(self, normal, albedo, lights7):
        out = np.zeros(3, np.uint32)
        l7 = _f32(lights7)
        self.lib.oracle_shade(_p(_f32(normal)), _p(_f32(albedo)), _p(l7), l7.shape[0], _p(out, C.c_uint32))
        return out


class Reference:
    """The reference's own draw_frame, compiled from its sources."""

    def __init__(self, path=REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} missing: build it with `make -C oracle ref` where the "
                                    "reference sources are present")
        self.lib = C.CDLL(path)
        self.lib.ref_set_projection.argtypes = [C.c_float, C.c_float, C.c_float]
        self.lib.ref_matrices.argtypes = [C.c_uint32, C.c_uint32, C.c_float, C.POINTER(C.c_float),
                                          C.POINTER(C.c_float), C.POINTER(C.c_float)]
        self.lib.ref_draw_frame.restype = C.c_int
        self.lib.ref_draw_frame.argtypes = [
            C.POINTER(C.c_float), C.c_int64, C.POINTER(C.c_int32), C.c_int64, C.POINTER(C.c_float), C.c_int64,
            C.POINTER(C.c_float), C.c_int64, C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float), C.c_int,
            C.c_uint32, C.c_uint32, C.c_int, C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float),
            C.POINTER(C.c_uint8), C.POINTER(C.c_float), C.POINTER(C.c_float)]
        self.lib.ref_raster_vertices.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int64,
                                                 C.c_uint32, C.c_uint32, C.POINTER(C.c_float)]
        self.lib.ref_signed_area_2d.restype = C.c_float
        self.lib.ref_signed_area_2d.argtypes = [C.POINTER(C.c_float)]
        self.lib.ref_shade.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                       C.c_int, C.POINTER(C.c_uint32)]
        self.lib.ref_draw_frame_tex.restype = C.c_int
        self.lib.ref_draw_frame_tex.argtypes = self.lib.ref_draw_frame.argtypes[:12] + [C.POINTER(C.c_char_p)] + \
            self.lib.ref_draw_frame.argtypes[12:]
        self.lib.ref_load_obj.restype = C.c_int
        self.lib.ref_load_obj.argtypes = [C.c_char_p, C.c_char_p]
        self.lib.ref_obj_counts.argtypes = [C.POINTER(C.c_int64)]
        self.lib.ref_obj_copy.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                          C.POINTER(C.c_int32), C.POINTER(C.c_float)]
        self.lib.ref_load_lights.restype = C.c_int
        self.lib.ref_load_lights.argtypes = [C.c_char_p, C.POINTER(C.c_float), C.c_int]

    def matrices(self, scene):
        """dict of model, view, modelview, camera, normal, camera45 (each (16,) float32, column major)."""
        self.lib.ref_set_projection(scene.fovy_deg, scene.z_near, scene.z_far)
        out = np.zeros(96, np.float32)
        disp, ang = _f32(scene.disp), _f32(scene.angles)
        self.lib.ref_matrices(scene.width, scene.height, scene.scale, _p(disp), _p(ang), _p(out))
        names = ["model", "view", "modelview", "camera", "normal", "camera45"]
        return {k: out[16 * i:16 * (i + 1)].copy() for i, k in enumerate(names)}

    def load_obj(self, path, mats_dir=""):
        """The reference's load_obj: dict of pos, nrm, uv, tris, kd (Material::sample at uv 0)."""
        if self.lib.ref_load_obj(os.fsencode(path), os.fsencode(mats_dir)) != 0:
            raise RuntimeError("reference load_obj raised")
        n = np.zeros(5, np.int64)
        self.lib.ref_obj_counts(_p(n, C.c_int64))
        pos, nrm, uv = np.zeros((n[0], 3), np.float32), np.zeros((n[1], 3), np.float32), np.zeros((n[2], 2), np.float32)
        tris, kd = np.zeros((n[3], 10), np.int32), np.zeros((n[4], 3), np.float32)
        self.lib.ref_obj_copy(_p(pos), _p(nrm), _p(uv), _p(tris, C.c_int32), _p(kd))
        return {"pos": pos, "nrm": nrm, "uv": uv, "tris": tris, "kd": kd}

    def load_lights(self, path, cap=4096):
        out = np.zeros((cap, 7), np.float32)
        n = self.lib.ref_load_lights(os.fsencode(path), _p(out), cap)
        return out[:min(n, cap)].copy()

    def draw(self, scene, frame=None, depth=None, textures=None):
        """Returns (frame (3,H,W) uint8, depth (H,W) float32, trans_dirs (nl,3)). textures: per
        material an image path the reference's Material loads, or None."""
        W, H = scene.width, scene.height
        self.lib.ref_set_projection(scene.fovy_deg, scene.z_near, scene.z_far)
        frame = np.zeros((3, H, W), np.uint8) if frame is None else np.ascontiguousarray(frame, np.uint8).copy()
        depth = np.ones((H, W), np.float32) if depth is None else _f32(depth).copy()
        pos, tris, nrm, uv, kd, li = (_f32(scene.pos), _i32(scene.tris), _f32(scene.nrm), _f32(scene.uv),
                                      _f32(scene.kd), _f32(scene.lights))
        td = np.zeros((li.shape[0], 3), np.float32)
        disp, ang = _f32(scene.disp), _f32(scene.angles)
        tex = None
        if textures is not None:
            tex = (C.c_char_p * len(textures))(*[os.fsencode(t) if t else None for t in textures])
        rc = self.lib.ref_draw_frame_tex(_p(pos), pos.shape[0], _p(tris, C.c_int32), tris.shape[0], _p(nrm),
                                         nrm.shape[0], _p(uv), uv.shape[0], _p(li), li.shape[0], _p(kd),
                                         kd.shape[0], tex, W, H, int(scene.wind_clockwise), scene.scale,
                                         _p(disp), _p(ang), _p(frame, C.c_uint8), _p(depth), _p(td))
        if rc != 0:
            raise RuntimeError("reference draw_frame raised")
        return frame, depth, td

    def raster_vertices(self, camera, pos, width, height):
        pos = _f32(pos)
        out = np.empty((pos.shape[0], 4), np.float32)
        self.lib.ref_raster_vertices(_p(_f32(camera)), _p(pos), pos.shape[0], width, height, _p(out))
        return out

    def signed_area_2d(self, v12):
        return self.lib.ref_signed_area_2d(_p(_f32(v12)))

    def shade(self, normal, albedo, lights7):
        out = np.zeros(3, np.uint32)
        l7 = _f32(lights7)
        self.lib.ref_shade(_p(_f32(normal)), _p(_f32(albedo)), _p(l7), l7.shape[0], _p(out, C.c_uint32))
        return out


def lights_with_dirs(scene, trans_dirs):
    """(nl, 7) records with the transformed directions in place of the world directions."""
    li = _f32(scene.lights).copy()
    li[:, 0:3] = trans_dirs
    return li
