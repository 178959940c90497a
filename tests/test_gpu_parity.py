"""Parity of the CUDA path (through the C ABI) with the reference's draw_frame.

Bar: depth buffer and winning-triangle index bit for bit; coverage therefore exact; RGB8 within
1/255 per channel (RGB_TOL below). The checkers are the golden fixtures made by the reference's own
code and the C restatement (oracle port) run here on the same inputs.
"""
import numpy as np
import pytest

import edge_scenes as E
import golden_io
from rasteriser_gb300 import abi
from rasteriser_gb300 import scenes as S

pytestmark = pytest.mark.gpu

RGB_TOL = 1  # per channel, in 1/255 units


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def flags_of(sc, clear=False):
    return (abi.WIND_CLOCKWISE if sc.wind_clockwise else 0) | (abi.CLEAR if clear else 0)


def gpu_draw(r, sc, cam, nm, lights7, frame=None, depth=None, clear=False):
    r.upload_scene_mesh(sc)
    r.set_lights(lights7)
    f = None if frame is None else frame.copy()
    d = None if depth is None else depth.copy()
    return r.draw(cam, nm, sc.width, sc.height, flags_of(sc, clear), f, d, want_ids=True)


def assert_parity(gpu, want_frame, want_depth, want_ids=None):
    fg, dg, ig = gpu
    assert np.array_equal(bits(dg), bits(want_depth)), f"depth differs at {np.argwhere(bits(dg) != bits(want_depth))[:5]}"
    if want_ids is not None:
        assert np.array_equal(ig, want_ids), f"winning triangle differs at {np.argwhere(ig != want_ids)[:5]}"
    diff = np.abs(fg.astype(np.int16) - want_frame.astype(np.int16))
    assert diff.max() <= RGB_TOL, f"RGB differs by {diff.max()}"


@pytest.mark.parametrize("name", golden_io.names())
def test_golden(renderer, port, name):
    sc, g = golden_io.load(name)
    out = gpu_draw(renderer, sc, g["camera"], g["normal"], g["lights7"])
    _, _, ids, _ = port.draw(sc, g["camera"], g["normal"], g["lights7"])
    assert_parity(out, g["frame"], g["depth"], ids)
    assert np.array_equal(out[0], g["frame"]), "RGB not bit-exact (within tolerance, but expected exact)"


def random_scenes():
    out = []
    for seed in range(6):
        out.append(S.soup(3000 + 1231 * seed, 200 + 83 * seed, 150 + 41 * seed, seed=200 + seed,
                          area_range=(0.2, 3000.0 * (seed + 1))).with_view(wind_clockwise=bool(seed % 3 == 1)))
    out.append(S.config_displaced_sphere(200, 100, 640, 360).with_view(angles=(0.4, 2.1, -0.7)))
    out.append(S.config_displaced_sphere(64, 32, 97, 61).with_view(scale=3.0))  # fills and overflows the frame
    out.append(S.icosphere(2).with_view(width=1280, height=720, fovy_deg=60.0, z_near=0.1, z_far=100.0, scale=1.6))
    out += E.all_edge_scenes()
    return out


@pytest.mark.parametrize("idx", range(len(random_scenes())))
@pytest.mark.parametrize("tile,small_max,row_chunk,threads", [
    (16, 4096, 4, 0), (8, 1, 4, 0), (32, 65536, 8, 0), (16, 16, 8, 0), (16, 4096, 32, 0), (8, 65536, 32, 0),
    (16, 1, 32, 64), (16, 16, 32, 128), (32, 1, 32, 128), (32, 16, 32, 512)])
def test_against_port(renderer, port, idx, tile, small_max, row_chunk, threads):
    """Every tile size, path split, row chunk and number of threads per tile (the tile raster's
    pixels per thread) gives the port's depth, ids and fragment counts."""
    sc = random_scenes()[idx]
    renderer.set_option(abi.OPT_TILE_SIZE, tile)
    renderer.set_option(abi.OPT_SMALL_MAX_PIXELS, small_max)
    renderer.set_option(abi.OPT_ROW_CHUNK, row_chunk)
    renderer.set_option(abi.OPT_TILE_THREADS, threads)
    try:
        cam, nm, lights, _ = abi.scene_frame_inputs(sc)
        out = gpu_draw(renderer, sc, cam, nm, lights)
        fp, dp, ip, st = port.draw(sc, cam, nm, lights)
        assert_parity(out, fp, dp, ip)
        s = renderer.stats()
        assert (s["front"], s["tested"], s["inside"]) == (int(st[0]), int(st[1]), int(st[2]))
        assert s["written"] == int((ip != abi.NO_TRIANGLE).sum())
    finally:
        renderer.set_option(abi.OPT_TILE_SIZE, 16)
        renderer.set_option(abi.OPT_SMALL_MAX_PIXELS, 4096)
        renderer.set_option(abi.OPT_ROW_CHUNK, 32)
        renderer.set_option(abi.OPT_TILE_THREADS, 0)


def test_read_modify_write_buffers(renderer, port):
    """Existing depth is the value to beat (drawing.cpp:119); untouched pixels keep their colour."""
    sc = S.soup(8000, 300, 200, seed=17, area_range=(0.5, 4000.0))
    rng = np.random.default_rng(5)
    depth = rng.uniform(-1.5, 1.5, (sc.height, sc.width)).astype(np.float32)
    depth[::7, ::5] = -0.0
    depth[1::7, ::5] = 0.0
    depth[3::11, ::3] = np.nan
    depth[5::13, 1::4] = -np.inf
    depth[6::13, 2::4] = np.inf
    frame = rng.integers(0, 256, (3, sc.height, sc.width), dtype=np.uint8)
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    out = gpu_draw(renderer, sc, cam, nm, lights, frame, depth)
    fp, dp, ip, _ = port.draw(sc, cam, nm, lights, frame, depth)
    assert_parity(out, fp, dp, ip)


def test_clear_flag_equals_fresh_buffers(renderer):
    sc = S.config_icosphere_small()
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    fresh = gpu_draw(renderer, sc, cam, nm, lights)
    junk_f = np.full((3, sc.height, sc.width), 77, np.uint8)
    junk_d = np.full((sc.height, sc.width), -5.0, np.float32)
    for _ in range(3):  # the clear path re-arms its keys for the next frame
        cl = gpu_draw(renderer, sc, cam, nm, lights, junk_f, junk_d, clear=True)
        assert np.array_equal(cl[0], fresh[0]) and np.array_equal(bits(cl[1]), bits(fresh[1]))
        assert np.array_equal(cl[2], fresh[2])


def test_idempotent_redraw(renderer):
    """Drawing the same frame again into its own output changes nothing: every fragment now meets
    an equal or nearer depth, and the test is strict."""
    sc = S.soup(20000, 640, 360, seed=23)
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    f1, d1, _ = gpu_draw(renderer, sc, cam, nm, lights)
    f2, d2, i2 = gpu_draw(renderer, sc, cam, nm, lights, f1, d1)
    assert np.array_equal(f2, f1) and np.array_equal(bits(d2), bits(d1))
    assert np.all(i2 == abi.NO_TRIANGLE)


def test_deterministic_over_reruns(renderer):
    sc = S.soup(60000, 800, 600, seed=29, area_range=(1.0, 2000.0))
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    first = gpu_draw(renderer, sc, cam, nm, lights)
    for _ in range(10):
        again = gpu_draw(renderer, sc, cam, nm, lights)
        assert np.array_equal(again[2], first[2]) and np.array_equal(bits(again[1]), bits(first[1]))
        assert np.array_equal(again[0], first[0])


def test_bin_pool_overflow_recovers(renderer, port):
    """A pool far too small for the frame: the host draw grows it and redraws; the result is exact."""
    sc = S.soup(5000, 400, 300, seed=31, area_range=(200.0, 5000.0))
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    renderer.set_option(abi.OPT_BIN_CAPACITY, 16)
    try:
        out = gpu_draw(renderer, sc, cam, nm, lights)
        fp, dp, ip, _ = port.draw(sc, cam, nm, lights)
        assert_parity(out, fp, dp, ip)
        assert renderer.get_option(abi.OPT_BIN_CAPACITY) > 16
    finally:
        renderer.set_option(abi.OPT_BIN_CAPACITY, 0)


def test_device_draw_reports_bin_overflow(renderer, port):
    torch = pytest.importorskip("torch")
    sc = S.soup(5000, 400, 300, seed=37, area_range=(200.0, 5000.0))
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    renderer.upload_scene_mesh(sc)
    renderer.set_lights(lights)
    rgb = torch.zeros((3, sc.height, sc.width), dtype=torch.uint8, device="cuda")
    dep = torch.ones((sc.height, sc.width), dtype=torch.float32, device="cuda")
    renderer.set_option(abi.OPT_BIN_CAPACITY, 8)
    try:
        renderer.draw_device(cam, nm, sc.width, sc.height, abi.CLEAR, rgb.data_ptr(), dep.data_ptr())
        with pytest.raises(abi.RastError) as ei:
            renderer.sync()
        assert ei.value.status == 6
        renderer.draw_device(cam, nm, sc.width, sc.height, abi.CLEAR, rgb.data_ptr(), dep.data_ptr())
        renderer.sync()
        fp, dp, _, _ = port.draw(sc, cam, nm, lights)
        assert np.array_equal(bits(dep.cpu().numpy()), bits(dp))
        assert np.abs(rgb.cpu().numpy().astype(int) - fp).max() <= RGB_TOL
    finally:
        renderer.set_option(abi.OPT_BIN_CAPACITY, 0)


def test_bad_index_is_refused(renderer):
    sc = S.square_scene()
    tris = sc.tris.copy()
    for col, val in [(0, 4), (1, -1), (3, 1), (5, -2), (6, 4), (9, 1), (9, -1)]:
        t = tris.copy()
        t[1, col] = val
        with pytest.raises(abi.RastError) as ei:
            renderer.upload_mesh(sc.pos, sc.nrm, sc.uv, t, sc.kd)
        assert ei.value.status == 2
    renderer._mesh_digest = None


def test_invalid_arguments(renderer):
    sc = S.square_scene()
    renderer.upload_scene_mesh(sc)
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    import ctypes
    buf_f = np.zeros(3 * 40000 * 10, np.uint8)
    buf_d = np.ones(40000 * 10, np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    c, n = np.ascontiguousarray(cam), np.ascontiguousarray(nm)
    for w, h in [(0, 10), (10, 0), (40000, 10)]:
        st = renderer.lib.rast_draw(renderer.h, c.ctypes.data_as(fp), n.ctypes.data_as(fp), w, h, 0,
                                    buf_f.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), buf_d.ctypes.data_as(fp),
                                    None)
        assert st == 1
    st = renderer.lib.rast_draw(renderer.h, None, n.ctypes.data_as(fp), 10, 10, 0,
                                buf_f.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), buf_d.ctypes.data_as(fp), None)
    assert st == 1
    with pytest.raises(abi.RastError):
        renderer.set_option(abi.OPT_TILE_SIZE, 12)
    with pytest.raises(abi.RastError):
        renderer.set_lights(np.zeros((5000, 7), np.float32))


@pytest.mark.parametrize("row_chunk", [8, 32])
@pytest.mark.parametrize("key", sorted(golden_io.full_size()))
def test_full_size_against_reference_digest(renderer, port, key, row_chunk):
    """Full-size frames (1,046,528 triangles at 1920x1080; 4M at 3840x2160) against the digests of
    the reference's own output, and against the port run here; per-triangle rows in chunks of 8
    pixels and as whole rows (the passing interval's ends found from the edges' crossings)."""
    import hashlib
    e = golden_io.full_size()[key]
    sc = golden_io.full_size_scene(e)
    if sc.mesh_digest() != e["mesh"]:
        pytest.skip("generated mesh differs from the one the digest was made for")
    cam = np.array(e["camera"], np.float32)
    nm = np.array(e["normal"], np.float32)
    lights = np.array(e["lights7"], np.float32)
    renderer.set_option(abi.OPT_ROW_CHUNK, row_chunk)
    try:
        fg, dg, ig = gpu_draw(renderer, sc, cam, nm, lights)
    finally:
        renderer.set_option(abi.OPT_ROW_CHUNK, 32)
    assert hashlib.sha256(np.ascontiguousarray(dg).tobytes()).hexdigest() == e["depth"]
    assert hashlib.sha256(np.ascontiguousarray(fg).tobytes()).hexdigest() == e["frame_rgb"]
    fp, dp, ip, st = port.draw(sc, cam, nm, lights)
    assert np.array_equal(ig, ip)
    s = renderer.stats()
    assert (s["front"], s["tested"], s["inside"]) == (int(st[0]), int(st[1]), int(st[2]))


def _translates_host_addresses(device=0):
    """cudaDevAttrPageableMemoryAccessUsesHostPageTables (100) of the device through the CUDA
    runtime, or None when no runtime library can be loaded."""
    import ctypes
    import ctypes.util
    for name in (ctypes.util.find_library("cudart"), "libcudart.so", "/usr/local/cuda/lib64/libcudart.so"):
        if not name:
            continue
        try:
            rt = ctypes.CDLL(name)
        except OSError:
            continue
        v = ctypes.c_int(0)
        if rt.cudaDeviceGetAttribute(ctypes.byref(v), 100, device) == 0:
            return bool(v.value)
    return None


def _pinned(torch, shape, dtype):
    """A numpy view of page-locked host memory (the device maps it)."""
    tdt = {np.uint8: torch.uint8, np.float32: torch.float32, np.uint32: torch.int32}[dtype]
    a = torch.zeros(shape, dtype=tdt).pin_memory().numpy()
    return a.view(np.uint32) if dtype is np.uint32 else a


@pytest.mark.parametrize("clear", [False, True])
def test_pinned_host_buffers_used_in_place(renderer, port, clear):
    """Page-locked buffers are read and written by the kernels in place: read-modify-write keeps
    the pixels nothing wins, clear mode writes them all; both equal the port and the copy path."""
    torch = pytest.importorskip("torch")
    sc = S.soup(8000, 300, 200, seed=23, area_range=(0.5, 4000.0))
    rng = np.random.default_rng(9)
    depth0 = rng.uniform(-1.5, 1.5, (sc.height, sc.width)).astype(np.float32)
    depth0[::7, ::5] = -0.0
    depth0[3::11, ::3] = np.nan
    frame0 = rng.integers(0, 256, (3, sc.height, sc.width), dtype=np.uint8)
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    renderer.upload_scene_mesh(sc)
    renderer.set_lights(lights)
    f = _pinned(torch, (3, sc.height, sc.width), np.uint8)
    d = _pinned(torch, (sc.height, sc.width), np.float32)
    i = _pinned(torch, (sc.height, sc.width), np.uint32)
    f[...] = frame0
    d[...] = depth0
    renderer.draw(cam, nm, sc.width, sc.height, flags_of(sc, clear), f, d, ids=i)
    assert renderer.stats()["host_in_place"] == 1
    fp, dp, ip, _ = port.draw(sc, cam, nm, lights, None if clear else frame0, None if clear else depth0)
    assert_parity((f, d, i), fp, dp, ip)
    pageable = gpu_draw(renderer, sc, cam, nm, lights, frame0, depth0, clear=clear)
    assert np.array_equal(pageable[0], f) and np.array_equal(bits(pageable[1]), bits(d))
    assert np.array_equal(pageable[2], i)


def test_pinned_host_buffers_overflow_recovers(renderer, port):
    """After a bin-pool overflow the in-place draw has written nothing; the redraw is exact."""
    torch = pytest.importorskip("torch")
    sc = S.soup(5000, 400, 300, seed=41, area_range=(200.0, 5000.0))
    rng = np.random.default_rng(3)
    depth0 = rng.uniform(-1.0, 1.5, (sc.height, sc.width)).astype(np.float32)
    frame0 = rng.integers(0, 256, (3, sc.height, sc.width), dtype=np.uint8)
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    renderer.upload_scene_mesh(sc)
    renderer.set_lights(lights)
    f = _pinned(torch, (3, sc.height, sc.width), np.uint8)
    d = _pinned(torch, (sc.height, sc.width), np.float32)
    f[...] = frame0
    d[...] = depth0
    renderer.set_option(abi.OPT_BIN_CAPACITY, 16)
    try:
        renderer.draw(cam, nm, sc.width, sc.height, flags_of(sc), f, d)
        assert renderer.get_option(abi.OPT_BIN_CAPACITY) > 16
    finally:
        renderer.set_option(abi.OPT_BIN_CAPACITY, 0)
    fp, dp, _, _ = port.draw(sc, cam, nm, lights, frame0, depth0)
    assert np.array_equal(bits(d), bits(dp))
    assert np.abs(f.astype(int) - fp).max() <= RGB_TOL


@pytest.mark.parametrize("clear", [False, True])
def test_pageable_host_buffers_in_place_and_copied(renderer, port, clear):
    """Ordinary (pageable) host buffers: used in place where the device translates host addresses
    (RAST_OPT_HOST_IN_PLACE 1, the default), copied through device memory with 0. Both equal the
    port: read-modify-write keeps the pixels nothing wins, clear mode writes them all. The draw's
    statistics say which path ran."""
    sc = S.soup(8000, 300, 200, seed=29, area_range=(0.5, 4000.0))
    rng = np.random.default_rng(11)
    depth0 = rng.uniform(-1.5, 1.5, (sc.height, sc.width)).astype(np.float32)
    depth0[::7, ::5] = -0.0
    depth0[3::11, ::3] = np.nan
    frame0 = rng.integers(0, 256, (3, sc.height, sc.width), dtype=np.uint8)
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    fp, dp, ip, _ = port.draw(sc, cam, nm, lights, None if clear else frame0, None if clear else depth0)
    reach = _translates_host_addresses()
    try:
        for in_place in (1, 0):
            renderer.set_option(abi.OPT_HOST_IN_PLACE, in_place)
            assert renderer.get_option(abi.OPT_HOST_IN_PLACE) == in_place
            assert_parity(gpu_draw(renderer, sc, cam, nm, lights, frame0, depth0, clear=clear), fp, dp, ip)
            used = renderer.stats()["host_in_place"]
            if in_place == 0 or reach is not None:
                assert used == (1 if in_place and reach else 0)
    finally:
        renderer.set_option(abi.OPT_HOST_IN_PLACE, 1)


def test_pageable_host_buffers_overflow_recovers(renderer, port):
    """Pageable buffers used in place: after a bin-pool overflow the draw has written nothing, and
    the redraw is exact."""
    sc = S.soup(5000, 400, 300, seed=43, area_range=(200.0, 5000.0))
    rng = np.random.default_rng(5)
    depth0 = rng.uniform(-1.0, 1.5, (sc.height, sc.width)).astype(np.float32)
    frame0 = rng.integers(0, 256, (3, sc.height, sc.width), dtype=np.uint8)
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    renderer.set_option(abi.OPT_BIN_CAPACITY, 16)
    try:
        f, d, _ = gpu_draw(renderer, sc, cam, nm, lights, frame0, depth0)
        assert renderer.get_option(abi.OPT_BIN_CAPACITY) > 16
    finally:
        renderer.set_option(abi.OPT_BIN_CAPACITY, 0)
    fp, dp, _, _ = port.draw(sc, cam, nm, lights, frame0, depth0)
    assert np.array_equal(bits(d), bits(dp))
    assert np.abs(f.astype(int) - fp).max() <= RGB_TOL


def test_pinned_slice_of_larger_allocation(renderer, port):
    """A frame that is a slice of a bigger page-locked buffer is used in place too."""
    torch = pytest.importorskip("torch")
    sc = S.config_icosphere_small()
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    renderer.upload_scene_mesh(sc)
    renderer.set_lights(lights)
    n = sc.width * sc.height
    big = torch.zeros(3 * n + 4096, dtype=torch.uint8).pin_memory().numpy()
    f = big[1000:1000 + 3 * n].reshape(3, sc.height, sc.width)
    dbig = torch.ones(n + 64, dtype=torch.float32).pin_memory().numpy()
    d = dbig[16:16 + n].reshape(sc.height, sc.width)
    renderer.draw(cam, nm, sc.width, sc.height, flags_of(sc, True), f, d)
    fp, dp, _, _ = port.draw(sc, cam, nm, lights)
    assert np.array_equal(bits(d), bits(dp))
    assert np.abs(f.astype(int) - fp).max() <= RGB_TOL
    assert np.all(big[:1000] == 0) and np.all(big[1000 + 3 * n:] == 0)
    assert np.all(dbig[:16] == 1.0) and np.all(dbig[16 + n:] == 1.0)


def test_registered_host_buffers_used_in_place(renderer, port):
    """Ordinary arrays registered with cudaHostRegister are page-locked and mapped too: drawn in
    place, equal to the port."""
    torch = pytest.importorskip("torch")
    sc = S.soup(6000, 300, 200, seed=29, area_range=(0.5, 3000.0))
    rng = np.random.default_rng(13)
    depth0 = rng.uniform(-1.0, 1.5, (sc.height, sc.width)).astype(np.float32)
    frame0 = rng.integers(0, 256, (3, sc.height, sc.width), dtype=np.uint8)
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    renderer.upload_scene_mesh(sc)
    renderer.set_lights(lights)
    f, d = frame0.copy(), depth0.copy()
    rt = torch.cuda.cudart()
    assert int(rt.cudaHostRegister(f.ctypes.data, f.nbytes, 0)) == 0
    try:
        assert int(rt.cudaHostRegister(d.ctypes.data, d.nbytes, 0)) == 0
        try:
            renderer.draw(cam, nm, sc.width, sc.height, flags_of(sc), f, d)
        finally:
            rt.cudaHostUnregister(d.ctypes.data)
    finally:
        rt.cudaHostUnregister(f.ctypes.data)
    fp, dp, _, _ = port.draw(sc, cam, nm, lights, frame0, depth0)
    assert np.array_equal(bits(d), bits(dp))
    assert np.abs(f.astype(int) - fp).max() <= RGB_TOL


def face_normal_scene(sc):
    """The scene with per-face normals cross(p1 - p0, p2 - p0) (float32, no fused operations) as
    its vertex normals: what --flat shades with."""
    p, t = np.asarray(sc.pos, np.float32), np.asarray(sc.tris)
    a, b = p[t[:, 1]] - p[t[:, 0]], p[t[:, 2]] - p[t[:, 0]]
    fn = np.stack([a[:, 1] * b[:, 2] - b[:, 1] * a[:, 2], a[:, 2] * b[:, 0] - b[:, 2] * a[:, 0],
                   a[:, 0] * b[:, 1] - b[:, 0] * a[:, 1]], axis=1).astype(np.float32)
    tris = t.copy()
    tris[:, 3:6] = np.arange(t.shape[0], dtype=np.int32)[:, None]
    return sc.with_view(nrm=fn, tris=tris)


FLAT_SCENES = {
    "icosphere4": lambda: S.config_icosphere_small(),
    "smooth_sphere": lambda: S.uv_sphere(160, 80, seed=7, flat=False).with_view(
        width=400, height=300, fovy_deg=60.0, z_near=0.1, z_far=100.0, angles=(0.3, 1.1, 0.0)),
    "soup_cw": lambda: S.soup(8000, 320, 240, seed=77, area_range=(0.5, 3000.0)).with_view(wind_clockwise=True),
}


@pytest.mark.parametrize("name", sorted(FLAT_SCENES))
@pytest.mark.parametrize("clear", [True, False])
def test_flat_shading_matches_port(renderer, port, name, clear):
    """RAST_FLAT (--flat): face normals computed in the path, against the port's flat mode and
    against the port drawing the same mesh with per-face normals given as its vertex normals."""
    sc = FLAT_SCENES[name]()
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    rng = np.random.default_rng(12)
    frame0 = rng.integers(0, 256, (3, sc.height, sc.width), dtype=np.uint8)
    depth0 = rng.uniform(-1.0, 1.5, (sc.height, sc.width)).astype(np.float32)
    renderer.upload_scene_mesh(sc)
    renderer.set_lights(lights)
    flags = flags_of(sc, clear) | abi.FLAT
    out = renderer.draw(cam, nm, sc.width, sc.height, flags, None if clear else frame0.copy(),
                        None if clear else depth0.copy(), want_ids=True)
    f0, d0 = (None, None) if clear else (frame0, depth0)
    fp, dp, ip, _ = port.draw(sc, cam, nm, lights, f0, d0, flat=True)
    assert_parity(out, fp, dp, ip)
    assert np.array_equal(out[0], fp)
    ff, df, _, _ = port.draw(face_normal_scene(sc), cam, nm, lights, f0, d0)
    assert np.array_equal(bits(df), bits(dp)) and np.array_equal(ff, fp)
