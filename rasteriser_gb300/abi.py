"""ctypes binding of librast's C ABI (include/rast.h).

``Renderer`` mirrors the reference's per-frame entry point: ``draw_frame`` takes the mesh, the
lights, the ``Args`` fields that matter (size, winding, model transform) and caller-owned frame and
depth buffers, and renders into them exactly as canmom/rasteriser's draw_frame (drawing.cpp:205-258)
does, through the CUDA kernels. There is no CPU fallback: without the built library or a GPU the
calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _build

RAST_OK = 0
STATUS_NAMES = {0: "RAST_OK", 1: "RAST_ERR_INVALID_ARG", 2: "RAST_ERR_BAD_INDEX", 3: "RAST_ERR_NO_MESH",
                4: "RAST_ERR_CUDA", 5: "RAST_ERR_OUT_OF_MEMORY", 6: "RAST_ERR_BIN_OVERFLOW",
                7: "RAST_ERR_TIMEOUT", 8: "RAST_ERR_NO_DEVICE", 9: "RAST_ERR_INTERNAL"}
WIND_CLOCKWISE, CLEAR, FLAT = 1, 2, 4
OPT_SMALL_MAX_PIXELS, OPT_TILE_SIZE, OPT_BIN_CAPACITY, OPT_STAGE_TIMING, OPT_ROW_CHUNK = 1, 2, 3, 4, 5
OPT_SHADER, OPT_MLP_SAMPLES, OPT_MLP_BOUND_MILLI, OPT_TEST_SHADE_STALL, OPT_TILE_THREADS = 6, 7, 8, 9, 10
OPT_HOST_IN_PLACE = 11
OPT_MLP_NETWORK = 12
MLP_COMPACT, MLP_WIDE = 0, 1
SHADER_EXACT, SHADER_EXACT_DEFERRED, SHADER_LEARNED = 0, 1, 2
STAGES = ["arm", "vertex", "setup_raster", "bin_scan", "bin_scatter", "tile_raster", "resolve", "shade", "total"]
NO_TRIANGLE = 0xFFFFFFFF

class FrameDesc(C.Structure):
    """rast_frame_desc of include/rast.h."""
    _fields_ = [("mesh", C.c_int32), ("width", C.c_uint32), ("height", C.c_uint32), ("flags", C.c_uint32),
                ("camera", C.c_float * 16), ("normal", C.c_float * 16), ("d_lights7", C.c_void_p),
                ("nl", C.c_int32), ("reserved", C.c_int32), ("d_rgb_planar", C.c_void_p),
                ("d_depth", C.c_void_p), ("d_tri_id", C.c_void_p)]


BATCH_GRAPH = 1


class MlpTrainDesc(C.Structure):
    """rast_mlp_train_desc of include/rast.h (zero fields take their defaults)."""
    _fields_ = [("samples", C.c_int64), ("holdout", C.c_int64), ("epochs", C.c_int32), ("ctas", C.c_int32),
                ("lr", C.c_float), ("seed", C.c_uint64)]

class ObjData(C.Structure):
    """rast_obj_data of include/rast.h."""
    _fields_ = [("pos", C.POINTER(C.c_float)), ("nv", C.c_int64), ("nrm", C.POINTER(C.c_float)), ("nn", C.c_int64),
                ("uv", C.POINTER(C.c_float)), ("nuv", C.c_int64), ("tris", C.POINTER(C.c_int32)),
                ("ntri", C.c_int64), ("kd", C.POINTER(C.c_float)), ("nmat", C.c_int32),
                ("textures", C.POINTER(C.c_char_p))]


class SpinDesc(C.Structure):
    """rast_spin_desc of include/rast.h."""
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("flags", C.c_uint32), ("frames", C.c_int32),
                ("scale", C.c_float), ("disp", C.c_float * 3), ("angles", C.c_float * 3), ("step", C.c_float),
                ("fovy_deg", C.c_float), ("z_near", C.c_float), ("z_far", C.c_float),
                ("lights7", C.POINTER(C.c_float)), ("nl", C.c_int32)]


# Every function include/rast.h declares, with its ctypes signature.
_F, _I32, _I64, _U32, _P = C.POINTER(C.c_float), C.c_int32, C.c_int64, C.c_uint32, C.c_void_p
SIGNATURES = {
    "rast_frame_matrices": (C.c_int, [_U32, _U32, C.c_float, _F, _F, C.c_float, C.c_float, C.c_float,
                                      _F, _F, _F, _F, _F]),
    "rast_transform_lights": (C.c_int, [_F, _F, _I32, _F]),
    "rast_create": (C.c_int, [C.POINTER(_P), C.c_int]),
    "rast_destroy": (None, [_P]),
    "rast_last_error": (C.c_char_p, [_P]),
    "rast_status_string": (C.c_char_p, [C.c_int]),
    "rast_abi_version": (C.c_int, []),
    "rast_set_stream": (C.c_int, [_P, _P]),
    "rast_get_stream": (_P, [_P]),
    "rast_upload_mesh": (C.c_int, [_P, _F, _I64, _F, _I64, _F, _I64, C.POINTER(C.c_int32), _I64, _F, _I32]),
    "rast_set_lights": (C.c_int, [_P, _F, _I32]),
    # the per-frame calls take plain addresses (cheaper to pass than typed pointers)
    "rast_draw": (C.c_int, [_P, _P, _P, _U32, _U32, _U32, _P, _P, _P]),
    "rast_draw_device": (C.c_int, [_P, _P, _P, _U32, _U32, _U32, _P, _P, _P]),
    "rast_sync": (C.c_int, [_P]),
    "rast_get_stats": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "rast_set_option": (C.c_int, [_P, C.c_int, _I64]),
    "rast_get_option": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int64)]),
    "rast_get_stage_times": (C.c_int, [_P, _F]),
    "rast_get_device_status": (C.c_int, [_P, C.POINTER(C.c_uint32)]),
    "rast_add_mesh": (C.c_int, [_P, _F, _I64, _F, _I64, _F, _I64, C.POINTER(C.c_int32), _I64, _F, _I32,
                                C.POINTER(C.c_int32)]),
    "rast_draw_batch": (C.c_int, [_P, C.POINTER(FrameDesc), _I32, _I32, _U32]),
    "rast_get_batch_stats": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "rast_autotune": (C.c_int, [_P, C.POINTER(FrameDesc), _I32, _I32, _I32, C.POINTER(C.c_int64)]),
    "rast_draw_noalloc": (C.c_int, [_P, _I64, _P, _I64, _P, _I64, _P, _I32, _P, _I32, _F, _F, _U32, _U32, _U32,
                                    _P, _P, _P, _P]),
    "rast_upload_vertex_albedo": (C.c_int, [_P, _F, _I64]),
    "rast_upload_texture": (C.c_int, [_P, _I32, _F, _U32, _U32, _U32]),
    "rast_mlp_train": (C.c_int, [_P, C.POINTER(MlpTrainDesc), _F]),
    "rast_mlp_save": (C.c_int, [_P, _P, C.c_size_t, C.POINTER(C.c_size_t)]),
    "rast_mlp_load": (C.c_int, [_P, _P, C.c_size_t]),
    "rast_mlp_eval": (C.c_int, [_P, _F, _F, _I64, _I32, _F]),
    "rast_time_shading": (C.c_int, [_P, _I32, _F]),
    "rast_get_shade_stats": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "rast_obj_load": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(_P)]),
    "rast_obj_free": (None, [_P]),
    "rast_obj_view": (C.c_int, [_P, C.POINTER(ObjData)]),
    "rast_lights_load": (C.c_int, [C.c_char_p, _F, _I32, C.POINTER(C.c_int32)]),
    "rast_image_load": (C.c_int, [C.c_char_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                  _F, C.c_size_t]),
    "rast_depth_to_u8": (C.c_int, [_P, _P, _U32, _U32, _P]),
    "rast_depth_to_u8_host": (C.c_int, [_P, _F, _U32, _U32, C.POINTER(C.c_uint8)]),
    "rast_spin": (C.c_int, [_P, C.POINTER(SpinDesc), C.POINTER(C.c_uint8), _F, C.POINTER(C.c_double)]),
}

_lib = None


def library_path():
    """librast.so, or its self-checking build librast_checked.so when RAST_CHECKED=1."""
    return _build.lib_path(checked=os.environ.get("RAST_CHECKED") == "1")


def load(build_if_missing=True):
    """Load librast.so (building it first when it is missing). Raises if it cannot be loaded."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"librast is not built ({path}); run __graft_entry__.build()")
        _build.build(checked=os.environ.get("RAST_CHECKED") == "1")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class RastError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _fp(a):
    return a.ctypes.data_as(_F) if a is not None else None


def _addr(a):
    """Address of an array's data: a ctypes view of a writable buffer costs a fraction of
    `a.ctypes.data`, which the per-frame calls would otherwise pay for every buffer."""
    try:
        return C.addressof(C.c_char.from_buffer(a))
    except (TypeError, ValueError, BufferError):  # read-only or empty
        return a.ctypes.data


def frame_matrices(width, height, scale=1.0, disp=(0, 0, 0), angles=(0, 0, 0), fovy_deg=45.0, z_near=0.1,
                   z_far=6.0):
    """The draw_frame matrices (model, view, modelview, camera, normal) as (16,) float32 arrays."""
    lib = load()
    outs = [np.zeros(16, np.float32) for _ in range(5)]
    d, a = _f32(disp), _f32(angles)
    st = lib.rast_frame_matrices(width, height, scale, _fp(d), _fp(a), fovy_deg, z_near, z_far,
                                 *[_fp(o) for o in outs])
    if st != RAST_OK:
        raise RastError(st, "rast_frame_matrices")
    return dict(zip(["model", "view", "modelview", "camera", "normal"], outs))


def transform_lights(view, lights7):
    lib = load()
    li = _f32(lights7).copy()
    out = np.empty_like(li)
    st = lib.rast_transform_lights(_fp(_f32(view)), _fp(li), li.shape[0], _fp(out))
    if st != RAST_OK:
        raise RastError(st, "rast_transform_lights")
    return out


def _io_error(st, what):
    lib = load()
    return RastError(st, f"{what}: {lib.rast_last_error(None).decode()}")


def obj_load(path, mats_dir=""):
    """A Wavefront OBJ as the reference's load_obj reads it: dict of pos (nv,3), nrm (nn,3),
    uv (nuv,2), tris (ntri,10) int32, kd (nmat,3) and textures (list of str)."""
    lib = load()
    h = _P()
    st = lib.rast_obj_load(os.fsencode(path), os.fsencode(mats_dir), C.byref(h))
    if st != RAST_OK:
        raise _io_error(st, "rast_obj_load")
    try:
        d = ObjData()
        lib.rast_obj_view(h, C.byref(d))

        def arr(ptr, n, cols, dtype):
            if n == 0:
                return np.zeros((0, cols), dtype)
            return np.ctypeslib.as_array(ptr, shape=(n * cols,)).reshape(n, cols).astype(dtype, copy=True)

        return {"pos": arr(d.pos, d.nv, 3, np.float32), "nrm": arr(d.nrm, d.nn, 3, np.float32),
                "uv": arr(d.uv, d.nuv, 2, np.float32), "tris": arr(d.tris, d.ntri, 10, np.int32),
                "kd": arr(d.kd, d.nmat, 3, np.float32),
                "textures": [d.textures[i].decode() for i in range(d.nmat)]}
    finally:
        lib.rast_obj_free(h)


def lights_load(path):
    """The lights CSV as (n, 7) float32 records."""
    lib = load()
    n = C.c_int32()
    st = lib.rast_lights_load(os.fsencode(path), None, 0, C.byref(n))
    if st != RAST_OK:
        raise _io_error(st, "rast_lights_load")
    out = np.zeros((n.value, 7), np.float32)
    if n.value:
        st = lib.rast_lights_load(os.fsencode(path), _fp(out), n.value, C.byref(n))
        if st != RAST_OK:
            raise _io_error(st, "rast_lights_load")
    return out


def image_load(path):
    """A PGM / PPM / PFM image as float32 (channels, height, width), values as stored."""
    lib = load()
    w, h, c = C.c_uint32(), C.c_uint32(), C.c_uint32()
    st = lib.rast_image_load(os.fsencode(path), C.byref(w), C.byref(h), C.byref(c), None, 0)
    if st != RAST_OK:
        raise _io_error(st, "rast_image_load")
    out = np.zeros((c.value, h.value, w.value), np.float32)
    st = lib.rast_image_load(os.fsencode(path), C.byref(w), C.byref(h), C.byref(c), _fp(out), out.size)
    if st != RAST_OK:
        raise _io_error(st, "rast_image_load")
    return out


def scene_frame_inputs(scene):
    """Camera matrix, normal matrix and transformed lights of a scene's frame."""
    m = frame_matrices(scene.width, scene.height, scene.scale, scene.disp, scene.angles, scene.fovy_deg,
                       scene.z_near, scene.z_far)
    return m["camera"], m["normal"], transform_lights(m["view"], scene.lights), m


class Renderer:
    """One librast context on one device."""

    def __init__(self, device=0):
        self.lib = load()
        h = _P()
        st = self.lib.rast_create(C.byref(h), device)
        if st != RAST_OK:
            raise RastError(st, self.lib.rast_last_error(None).decode())
        self.h = h
        self._mesh_digest = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.rast_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what):
        if st != RAST_OK:
            raise RastError(st, f"{what}: {self.lib.rast_last_error(self.h).decode()}")

    # scene data -----------------------------------------------------------------------------
    def upload_mesh(self, pos, nrm, uv, tris, kd):
        pos, nrm, uv, kd = _f32(pos), _f32(nrm), _f32(uv), _f32(kd)
        tris = np.ascontiguousarray(tris, np.int32)
        st = self.lib.rast_upload_mesh(self.h, _fp(pos), pos.shape[0], _fp(nrm), nrm.shape[0],
                                       _fp(uv) if uv.size else None, uv.shape[0],
                                       tris.ctypes.data_as(C.POINTER(C.c_int32)), tris.shape[0], _fp(kd), kd.shape[0])
        self._check(st, "rast_upload_mesh")

    def upload_scene_mesh(self, scene):
        dg = scene.mesh_digest()
        if dg != self._mesh_digest:
            self.upload_mesh(scene.pos, scene.nrm, scene.uv, scene.tris, scene.kd)
            va = getattr(scene, "vertex_albedo", None)
            if va is not None:
                self.upload_vertex_albedo(va)
            self._mesh_digest = dg

    def upload_vertex_albedo(self, rgb):
        """Per-vertex albedo (nv, 3) in place of the materials' Kd; None returns to Kd."""
        if rgb is None:
            self._check(self.lib.rast_upload_vertex_albedo(self.h, None, 0), "rast_upload_vertex_albedo")
        else:
            a = _f32(rgb).reshape(-1, 3)
            self._check(self.lib.rast_upload_vertex_albedo(self.h, _fp(a), a.shape[0]), "rast_upload_vertex_albedo")
        self._mesh_digest = None

    def upload_texture(self, material, texels):
        """Texture of a material: texels (c, h, w) as loaded (e.g. image_load), or None to remove."""
        if texels is None:
            self._check(self.lib.rast_upload_texture(self.h, material, None, 0, 0, 0), "rast_upload_texture")
            return
        t = _f32(texels)
        self._check(self.lib.rast_upload_texture(self.h, material, _fp(t), t.shape[2], t.shape[1], t.shape[0]),
                    "rast_upload_texture")

    def set_lights(self, lights7):
        li = _f32(lights7).reshape(-1, 7)
        self._check(self.lib.rast_set_lights(self.h, _fp(li), li.shape[0]), "rast_set_lights")

    def set_option(self, opt, value):
        self._check(self.lib.rast_set_option(self.h, opt, int(value)), "rast_set_option")

    def get_option(self, opt):
        v = C.c_int64()
        self._check(self.lib.rast_get_option(self.h, opt, C.byref(v)), "rast_get_option")
        return v.value

    def set_stream(self, stream_handle):
        """Launch on a created CUDA stream (an integer cudaStream_t), or None for the context's own.
        Handle 0 is refused: in the C ABI it means the context's own stream, not the legacy default
        stream, and work timed on the default stream would not see the draws."""
        if stream_handle == 0:
            raise ValueError("stream handle 0 is ambiguous; pass a created stream or None")
        self._check(self.lib.rast_set_stream(self.h, _P(stream_handle) if stream_handle else None), "rast_set_stream")

    # drawing --------------------------------------------------------------------------------
    def draw(self, camera, normal, width, height, flags=0, frame=None, depth=None, want_ids=False, ids=None):
        """Host-buffer draw. frame: (3, H, W) uint8, depth: (H, W) float32, both read and written;
        ids: an optional (H, W) uint32 output (made here when want_ids and none is given)."""
        frame = np.zeros((3, height, width), np.uint8) if frame is None else frame
        depth = np.ones((height, width), np.float32) if depth is None else depth
        assert frame.dtype == np.uint8 and frame.flags.c_contiguous and frame.size == 3 * width * height
        assert depth.dtype == np.float32 and depth.flags.c_contiguous and depth.size == width * height
        if ids is None and want_ids:
            ids = np.empty((height, width), np.uint32)
        if ids is not None:
            assert ids.dtype == np.uint32 and ids.flags.c_contiguous and ids.size == width * height
        cam, nrm = _f32(camera), _f32(normal)  # kept alive across the call
        st = self.lib.rast_draw(self.h, _addr(cam), _addr(nrm), width, height, flags, _addr(frame), _addr(depth),
                                _addr(ids) if ids is not None else None)
        self._check(st, "rast_draw")
        return frame, depth, ids

    def draw_device(self, camera, normal, width, height, flags, d_rgb, d_depth, d_ids=0):
        """Device-buffer draw on the context's stream; pointers are integers (e.g. tensor.data_ptr())."""
        cam, nrm = _f32(camera), _f32(normal)  # kept alive across the call
        st = self.lib.rast_draw_device(self.h, _addr(cam), _addr(nrm), width, height, flags, d_rgb, d_depth,
                                       d_ids or None)
        self._check(st, "rast_draw_device")

    def sync(self):
        self._check(self.lib.rast_sync(self.h), "rast_sync")

    # batches ---------------------------------------------------------------------------------
    def add_mesh(self, pos, nrm, uv, tris, kd):
        pos, nrm, uv, kd = _f32(pos), _f32(nrm), _f32(uv), _f32(kd)
        tris = np.ascontiguousarray(tris, np.int32)
        mid = C.c_int32()
        st = self.lib.rast_add_mesh(self.h, _fp(pos), pos.shape[0], _fp(nrm), nrm.shape[0],
                                    _fp(uv) if uv.size else None, uv.shape[0],
                                    tris.ctypes.data_as(C.POINTER(C.c_int32)), tris.shape[0], _fp(kd), kd.shape[0],
                                    C.byref(mid))
        self._check(st, "rast_add_mesh")
        return mid.value

    @staticmethod
    def frame_desc(mesh, width, height, flags, camera, normal, d_lights, nl, d_rgb, d_depth, d_ids=0):
        f = FrameDesc()
        f.mesh, f.width, f.height, f.flags = mesh, width, height, flags
        f.camera[:] = [float(v) for v in np.asarray(camera, np.float32)]
        f.normal[:] = [float(v) for v in np.asarray(normal, np.float32)]
        f.d_lights7, f.nl = d_lights or None, nl
        f.d_rgb_planar, f.d_depth, f.d_tri_id = d_rgb, d_depth, d_ids or None
        return f

    def draw_batch(self, frames, lanes=8, graph=True):
        arr = (FrameDesc * len(frames))(*frames)
        self._check(self.lib.rast_draw_batch(self.h, arr, len(frames), lanes, BATCH_GRAPH if graph else 0),
                    "rast_draw_batch")
        self._batch_keepalive = arr

    def batch_stats(self, n):
        out = (C.c_uint64 * (8 * n))()
        self._check(self.lib.rast_get_batch_stats(self.h, out), "rast_get_batch_stats")
        return np.frombuffer(out, np.uint64).reshape(n, 8).copy()

    def autotune(self, frames, lanes=8, repeats=3):
        arr = (FrameDesc * len(frames))(*frames)
        out = (C.c_int64 * 5)()
        self._check(self.lib.rast_autotune(self.h, arr, len(frames), lanes, repeats, out), "rast_autotune")
        return dict(zip(["tile", "small_max", "row_chunk", "bin_capacity", "tile_threads"], list(out)))

    def stats(self):
        out = (C.c_uint64 * 8)()
        self._check(self.lib.rast_get_stats(self.h, out), "rast_get_stats")
        keys = ["front", "tested", "inside", "written", "binned_tris", "bin_entries", "launches", "host_in_place"]
        return dict(zip(keys, list(out)))

    def device_status(self):
        out = (C.c_uint32 * 4)()
        self._check(self.lib.rast_get_device_status(self.h, out), "rast_get_device_status")
        return list(out)

    def stage_times(self):
        """Per-stage device milliseconds of the last draw (RAST_OPT_STAGE_TIMING must be on)."""
        out = np.zeros(len(STAGES), np.float32)
        self._check(self.lib.rast_get_stage_times(self.h, _fp(out)), "rast_get_stage_times")
        return dict(zip(STAGES, [float(v) for v in out]))

    # learned shading ------------------------------------------------------------------------
    def mlp_train(self, samples=0, holdout=0, epochs=0, ctas=0, lr=0.0, seed=0):
        """Train the context's MLP for its current lights. Returns dict(mse, mean_err, max_err, seconds)."""
        d = MlpTrainDesc(samples, holdout, epochs, ctas, lr, seed)
        out = np.zeros(4, np.float32)
        self._check(self.lib.rast_mlp_train(self.h, C.byref(d), _fp(out)), "rast_mlp_train")
        return dict(zip(["mse", "mean_err", "max_err", "seconds"], [float(v) for v in out]))

    def mlp_save(self):
        size = C.c_size_t()
        self._check(self.lib.rast_mlp_save(self.h, None, 0, C.byref(size)), "rast_mlp_save")
        buf = (C.c_uint8 * size.value)()
        self._check(self.lib.rast_mlp_save(self.h, buf, size.value, C.byref(size)), "rast_mlp_save")
        return bytes(buf)

    def mlp_load(self, blob):
        buf = (C.c_uint8 * len(blob)).from_buffer_copy(blob)
        self._check(self.lib.rast_mlp_load(self.h, buf, len(blob)), "rast_mlp_load")

    def mlp_eval(self, normals, albedo, exact=False):
        """Radiance (n, 3) float32 of (normal, albedo) pairs through the tensor-core kernel or the
        exact shader, before clamping."""
        nv, al = _f32(normals).reshape(-1, 3), _f32(albedo).reshape(-1, 3)
        assert nv.shape == al.shape
        out = np.zeros_like(nv)
        self._check(self.lib.rast_mlp_eval(self.h, _fp(nv), _fp(al), nv.shape[0], 1 if exact else 0, _fp(out)),
                    "rast_mlp_eval")
        return out

    def depth_to_u8(self, d_depth, width, height, d_out):
        """renderer.cpp's depth view of a device depth buffer into device bytes (asynchronous)."""
        self._check(self.lib.rast_depth_to_u8(self.h, _P(d_depth), width, height, _P(d_out)), "rast_depth_to_u8")

    def depth_view(self, depth):
        """The depth view of a host depth buffer (H, W) float32 -> (H, W) uint8."""
        d = _f32(depth)
        out = np.zeros(d.shape, np.uint8)
        self._check(self.lib.rast_depth_to_u8_host(self.h, _fp(d), d.shape[1], d.shape[0],
                                                   out.ctypes.data_as(C.POINTER(C.c_uint8))), "rast_depth_to_u8_host")
        return out

    def spin(self, scene, frames, step=1.0 / 60.0):
        """The headless spin loop over the scene's mesh (uploaded if it changed): frames frames with
        ry advancing by step. Returns (last frame (3,H,W), last depth (H,W), seconds)."""
        self.upload_scene_mesh(scene)
        li = _f32(scene.lights).reshape(-1, 7)
        d = SpinDesc()
        d.width, d.height = scene.width, scene.height
        d.flags = WIND_CLOCKWISE if scene.wind_clockwise else 0
        d.frames = frames
        d.scale = scene.scale
        d.disp[:] = [float(v) for v in scene.disp]
        d.angles[:] = [float(v) for v in scene.angles]
        d.step = step
        d.fovy_deg, d.z_near, d.z_far = scene.fovy_deg, scene.z_near, scene.z_far
        d.lights7 = _fp(li)
        d.nl = li.shape[0]
        frame = np.zeros((3, scene.height, scene.width), np.uint8)
        depth = np.zeros((scene.height, scene.width), np.float32)
        sec = C.c_double()
        self._check(self.lib.rast_spin(self.h, C.byref(d), frame.ctypes.data_as(C.POINTER(C.c_uint8)), _fp(depth),
                                       C.byref(sec)), "rast_spin")
        return frame, depth, sec.value

    def time_shading(self, repeats=200):
        """Mean microseconds of one more run of the last draw's deferred shading pass (back to back)."""
        v = C.c_float()
        self._check(self.lib.rast_time_shading(self.h, repeats, C.byref(v)), "rast_time_shading")
        return float(v.value)

    def shade_stats(self):
        out = (C.c_uint64 * 4)()
        self._check(self.lib.rast_get_shade_stats(self.h, out), "rast_get_shade_stats")
        return {"tiles": int(out[0]), "fallback_tiles": int(out[1]), "checked": int(out[2]),
                "max_checked_err": out[3] / 1e6}

    def draw_scene(self, scene, frame=None, depth=None, want_ids=True, clear=False):
        """draw_frame for a Scene: uploads its mesh if it changed, sets its lights, renders."""
        self.upload_scene_mesh(scene)
        cam, nm, lights, _ = scene_frame_inputs(scene)
        self.set_lights(lights)
        flags = (WIND_CLOCKWISE if scene.wind_clockwise else 0) | (CLEAR if clear else 0)
        return self.draw(cam, nm, scene.width, scene.height, flags, frame, depth, want_ids)
