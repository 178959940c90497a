"""rast_draw_noalloc: the draw for callers that must not allocate device memory (a host
application whose own pool owns all device memory, or a frame loop that cannot take the
device-wide synchronisation of cudaMalloc / cudaFree). It uses only the caller's device buffers and
a fixed array inside the library. Its output must equal the oracle port's and the context entry
point's (rast_draw_device) on the same inputs, call after call.

This file is collected last, so that a run stopping at the first failure has run every other test;
it builds and loads the library itself and also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from rasteriser_gb300 import abi
from rasteriser_gb300 import scenes as S

pytestmark = pytest.mark.gpu

RGB_TOL = 1  # per channel, 1/255 units, as in the other parity tests


def _call(lib, torch, dev, cam, nm, W, H, flags, rgb, depth, ids):
    fp = C.POINTER(C.c_float)
    c, n = np.ascontiguousarray(cam, np.float32), np.ascontiguousarray(nm, np.float32)
    return lib.rast_draw_noalloc(dev["pos"].data_ptr(), dev["pos"].shape[0], dev["nrm"].data_ptr(),
                                 dev["nrm"].shape[0], dev["tris"].data_ptr(), dev["tris"].shape[0],
                                 dev["kd"].data_ptr(), dev["kd"].shape[0], dev["lights"].data_ptr(),
                                 dev["lights"].shape[0], c.ctypes.data_as(fp), n.ctypes.data_as(fp), W, H, flags,
                                 rgb.data_ptr(), depth.data_ptr(), ids.data_ptr() if ids is not None else None,
                                 torch.cuda.current_stream().cuda_stream or None)


def _screen_covering(n, seed, W=1920, H=1080):
    """n triangles that each cover the whole 1920x1080 frame (one tile-bin entry per 16x16 tile
    each), at seeded depths, all facing the camera."""
    rng = np.random.default_rng(seed)
    z = rng.uniform(-1.0, 1.0, n).astype(np.float32)
    pos = np.zeros((3 * n, 3), np.float32)
    pos[0::3] = np.stack([np.full(n, -20.0), np.full(n, -20.0), z], 1)
    pos[1::3] = np.stack([np.full(n, 20.0), np.full(n, -20.0), z], 1)
    pos[2::3] = np.stack([np.zeros(n), np.full(n, 20.0), z], 1)
    tris = np.zeros((n, 10), np.int32)
    tris[:, 0:3] = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    tris[:, 3:6] = 0
    tris[:, 6:9] = -1
    nrm = np.array([[0.0, 0.0, 1.0]], np.float32)
    lights = np.array([[1, -1, -1, 255, 1, 1, 1]], np.float32)
    return S.Scene("screen_covering", pos, tris, nrm, np.zeros((0, 2), np.float32),
                   np.array([[0.8, 0.6, 0.4]], np.float32), lights, width=W, height=H, fovy_deg=60.0,
                   z_near=0.1, z_far=100.0)


def _device_mesh(torch, sc, lights):
    def d(a, dt):
        return torch.from_numpy(np.ascontiguousarray(a, dt)).to("cuda")
    return {"pos": d(sc.pos, np.float32), "nrm": d(sc.nrm, np.float32), "tris": d(sc.tris, np.int32),
            "kd": d(sc.kd, np.float32), "lights": d(lights, np.float32)}


@pytest.mark.parametrize("which", ["icosphere", "soup", "screen_covering"])
def test_noalloc_equals_port_and_context_draw_on_consecutive_calls(which, port):
    torch = pytest.importorskip("torch")
    lib = abi.load()
    sc = {"icosphere": S.config_icosphere_small,
          "soup": lambda: S.soup(20000, 640, 360, seed=41, area_range=(0.5, 3000.0)),
          "screen_covering": lambda: _screen_covering(40, seed=5)}[which]()
    W, H = sc.width, sc.height
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    rng = np.random.default_rng(7)
    init_rgb = torch.from_numpy(rng.integers(0, 256, 3 * W * H, dtype=np.uint8)).to("cuda")
    init_depth = torch.from_numpy(rng.uniform(-1.0, 2.0, W * H).astype(np.float32)).to("cuda")

    # the existing entry point: a context, its allocations, device buffers
    r = abi.Renderer(0)
    try:
        r.upload_scene_mesh(sc)
        r.set_lights(lights)
        want = {}
        for flags in (abi.CLEAR, 0):
            rgb, dep = init_rgb.clone(), init_depth.clone()
            ids = torch.empty(W * H, dtype=torch.int32, device="cuda")
            r.draw_device(cam, nm, W, H, flags, rgb.data_ptr(), dep.data_ptr(), ids.data_ptr())
            r.sync()
            want[flags] = (rgb.cpu().numpy(), dep.cpu().numpy(), ids.cpu().numpy())
    finally:
        r.close()

    dev = _device_mesh(torch, sc, lights)
    for flags in (abi.CLEAR, 0):
        for _ in range(2):  # two calls in a row share the fixed array
            rgb, dep = init_rgb.clone(), init_depth.clone()
            ids = torch.empty(W * H, dtype=torch.int32, device="cuda")
            st = _call(lib, torch, dev, cam, nm, W, H, flags, rgb, dep, ids)
            assert st == 0, lib.rast_last_error(None).decode()
            torch.cuda.synchronize()
            w_rgb, w_dep, w_ids = want[flags]
            assert np.array_equal(dep.cpu().numpy().view(np.uint32), w_dep.view(np.uint32))
            assert np.array_equal(ids.cpu().numpy(), w_ids)
            assert np.abs(rgb.cpu().numpy().astype(int) - w_rgb.astype(int)).max() <= RGB_TOL
            # and directly against the oracle port, fed the same incoming frame and depth
            frame0 = None if flags == abi.CLEAR else init_rgb.cpu().numpy().reshape(3, H, W)
            depth0 = None if flags == abi.CLEAR else init_depth.cpu().numpy().reshape(H, W)
            fp, dp, ip, _ = port.draw(sc, cam, nm, lights, frame0, depth0)
            assert np.array_equal(dep.cpu().numpy().reshape(H, W).view(np.uint32), dp.view(np.uint32))
            assert np.array_equal(ids.cpu().numpy().reshape(H, W).view(np.uint32), np.asarray(ip).view(np.uint32))
            assert np.abs(rgb.cpu().numpy().reshape(3, H, W).astype(int) - fp.astype(int)).max() <= RGB_TOL


def test_noalloc_refuses_what_does_not_fit_and_bad_indices():
    torch = pytest.importorskip("torch")
    lib = abi.load()
    sc = S.config_icosphere_small()
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    dev = _device_mesh(torch, sc, lights)
    W, H = 8192, 8192  # 512 MiB of depth keys alone
    rgb = torch.zeros(1, dtype=torch.uint8, device="cuda")
    dep = torch.zeros(1, dtype=torch.float32, device="cuda")
    st = _call(lib, torch, dev, cam, nm, W, H, abi.CLEAR, rgb, dep, None)
    assert st == 1 and b"fixed array" in lib.rast_last_error(None)

    bad = sc.tris.copy()
    bad[5, 1] = sc.pos.shape[0]  # vertex index one past the end
    dev["tris"] = torch.from_numpy(bad).to("cuda")
    rgb = torch.zeros(3 * sc.width * sc.height, dtype=torch.uint8, device="cuda")
    dep = torch.ones(sc.width * sc.height, dtype=torch.float32, device="cuda")
    st = _call(lib, torch, dev, cam, nm, sc.width, sc.height, abi.CLEAR, rgb, dep, None)
    assert st == 2


def test_noalloc_bin_overflow_leaves_the_buffers_unchanged():
    """Thousands of screen-sized triangles need more tile-bin entries than the fixed array holds:
    the call reports RAST_ERR_BIN_OVERFLOW and the caller's frame, depth and ids are untouched, in
    both modes; the next call that fits draws normally."""
    torch = pytest.importorskip("torch")
    lib = abi.load()
    sc = _screen_covering(4000, seed=6)
    W, H = sc.width, sc.height
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    dev = _device_mesh(torch, sc, lights)
    rng = np.random.default_rng(8)
    init_rgb = torch.from_numpy(rng.integers(0, 256, 3 * W * H, dtype=np.uint8)).to("cuda")
    init_depth = torch.from_numpy(rng.uniform(-1.0, 2.0, W * H).astype(np.float32)).to("cuda")
    init_ids = torch.from_numpy(rng.integers(0, 1 << 30, W * H, dtype=np.int32)).to("cuda")
    for flags in (abi.CLEAR, 0):
        rgb, dep, ids = init_rgb.clone(), init_depth.clone(), init_ids.clone()
        st = _call(lib, torch, dev, cam, nm, W, H, flags, rgb, dep, ids)
        assert st == 6, (st, lib.rast_last_error(None).decode())
        torch.cuda.synchronize()
        assert torch.equal(rgb, init_rgb) and torch.equal(dep, init_depth) and torch.equal(ids, init_ids)
    small = _screen_covering(8, seed=6)
    dev = _device_mesh(torch, small, lights)
    rgb, dep = init_rgb.clone(), init_depth.clone()
    assert _call(lib, torch, dev, cam, nm, W, H, abi.CLEAR, rgb, dep, None) == 0
    torch.cuda.synchronize()
    assert not torch.equal(dep, init_depth)
