"""The headless renderer (renderer.cpp's modes) and the depth view, through the C ABI and the
rast_render program, against the oracle port and a numpy restatement of CImg's normalize."""
import os
import subprocess

import numpy as np
import pytest

from rasteriser_gb300 import _build, abi
from rasteriser_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def cimg_normalize_u8(depth):
    """renderer.cpp:93: (v - m) / (M - m) * 255 + 0 in float32 (m, M by < and >), then the C
    conversion to unsigned char; 0 everywhere when m == M."""
    d = np.asarray(depth, np.float32)
    m, M = np.float32(d.min()), np.float32(d.max())
    if m == M:
        return np.zeros(d.shape, np.uint8)
    v = ((d - m) / (M - m)) * np.float32(255.0) + np.float32(0.0)
    return v.astype(np.float32).astype(np.uint8)


def read_pnm(path):
    with open(path, "rb") as fh:
        data = fh.read()
    parts = data.split(maxsplit=4)
    kind, w, h = parts[0], int(parts[1]), int(parts[2])
    body = parts[4]
    ch = 3 if kind == b"P6" else 1
    a = np.frombuffer(body[:w * h * ch], np.uint8).reshape(h, w, ch)
    return np.moveaxis(a, 2, 0)


@pytest.fixture(scope="module")
def rnd():
    r = abi.Renderer(0)
    yield r
    r.close()


def test_depth_view_matches_cimg_normalize(rnd, port):
    sc = S.config_displaced_sphere(128, 64, 320, 200)
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    _, depth, _, _ = port.draw(sc, cam, nm, lights)
    assert np.array_equal(rnd.depth_view(depth), cimg_normalize_u8(depth))
    rng = np.random.default_rng(4)
    odd = (rng.random((37, 53)) * 3 - 2).astype(np.float32)
    assert np.array_equal(rnd.depth_view(odd), cimg_normalize_u8(odd))
    const = np.full((9, 11), 0.25, np.float32)
    assert (rnd.depth_view(const) == 0).all()


def test_spin_last_frame_is_the_frame_at_its_angle(rnd, port):
    sc = S.config_displaced_sphere(96, 48, 256, 160)
    n, step = 7, 0.05
    frame, depth, sec = rnd.spin(sc, n, step)
    ry = np.float32(sc.angles[1]) + np.float32(n - 1) * np.float32(step)  # float arithmetic, as the loop
    last = sc.with_view(angles=(sc.angles[0], float(np.float32(ry)), sc.angles[2]))
    cam, nm, lights, _ = abi.scene_frame_inputs(last)
    of, od, _, _ = port.draw(last, cam, nm, lights)
    assert np.array_equal(frame, of)
    assert np.array_equal(depth.view(np.uint32), od.view(np.uint32))
    assert sec > 0


def run_cli(args, cwd):
    exe = _build.cli_path()
    r = subprocess.run([exe] + args, cwd=cwd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr + r.stdout
    return r.stdout


def write_lights(path, lights7):
    with open(path, "w") as fh:
        for L in lights7:
            fh.write(",".join(repr(float(v)) for v in L) + "\n")


def test_cli_default_square(port, tmp_path):
    write_lights(tmp_path / "l.csv", S.rig_threepoint_csv())
    run_cli(["-l", "l.csv", "--out", str(tmp_path)], tmp_path)
    sc = S.square_scene()  # renderer.cpp's add_square, 540 x 304, 45 deg projection
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    of, od, _, _ = port.draw(sc, cam, nm, lights)
    assert np.array_equal(read_pnm(tmp_path / "frame.ppm"), of)
    assert np.array_equal(read_pnm(tmp_path / "depth.pgm")[0], cimg_normalize_u8(od))


def write_obj(path, sc):
    with open(path, "w") as fh:
        for p in sc.pos:
            fh.write("v %r %r %r\n" % tuple(float(v) for v in p))
        for n in sc.nrm:
            fh.write("vn %r %r %r\n" % tuple(float(v) for v in n))
        fh.write("mtllib m.mtl\nusemtl M\n")
        for t in sc.tris:
            fh.write("f %d//%d %d//%d %d//%d\n" % (t[0] + 1, t[3] + 1, t[1] + 1, t[4] + 1, t[2] + 1, t[5] + 1))
    with open(os.path.join(os.path.dirname(path), "m.mtl"), "w") as fh:
        fh.write("newmtl M\nKd %r %r %r\n" % tuple(float(v) for v in sc.kd[0]))


def test_cli_obj_frame_and_spin(port, tmp_path):
    sc = S.icosphere(3).with_view(width=200, height=150, angles=(0.3, 0.4, 0.0), scale=0.8, disp=(0.1, 0.0, -0.5))
    write_obj(tmp_path / "m.obj", sc)
    write_lights(tmp_path / "l.csv", sc.lights)
    common = ["-l", "l.csv", "-o", "m.obj", "--mats-dir", str(tmp_path) + "/", "-x", "200", "-y", "150",
              "--rx", "0.3", "--ry", "0.4", "--scale", "0.8", "--dx", "0.1", "--dz", "-0.5", "--out", str(tmp_path)]
    run_cli(common, tmp_path)
    loaded = abi.obj_load(str(tmp_path / "m.obj"), str(tmp_path) + "/")
    sc2 = S.Scene("obj", loaded["pos"], loaded["tris"], loaded["nrm"], loaded["uv"], loaded["kd"], sc.lights,
                  width=200, height=150, angles=(np.float32(0.3), np.float32(0.4), 0.0), scale=np.float32(0.8),
                  disp=(np.float32(0.1), 0.0, np.float32(-0.5)))
    cam, nm, lights, _ = abi.scene_frame_inputs(sc2)
    of, od, _, _ = port.draw(sc2, cam, nm, lights)
    assert np.array_equal(read_pnm(tmp_path / "frame.ppm"), of)
    assert np.array_equal(read_pnm(tmp_path / "depth.pgm")[0], cimg_normalize_u8(od))
    # spin, every frame dumped: frame k is the frame at ry = 0.4 + k * step
    out = run_cli(common + ["--spin", "--frames", "3", "--step", "0.25", "--dump"], tmp_path)
    assert "frames/s" in out
    for k in range(3):
        ry = float(np.float32(np.float32(0.4) + np.float32(k * 0.25)))
        sk = sc2.with_view(angles=(np.float32(0.3), ry, 0.0))
        cam, nm, lights, _ = abi.scene_frame_inputs(sk)
        of, _, _, _ = port.draw(sk, cam, nm, lights)
        assert np.array_equal(read_pnm(tmp_path / ("frame_%04d.ppm" % k)), of), k


def test_cli_rejects_bad_arguments(tmp_path):
    exe = _build.cli_path()
    r = subprocess.run([exe, "-x", "100"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "lights" in r.stderr


def test_cli_flat_projection_and_light_scale(port, tmp_path):
    """--flat shades with face normals computed in the path; --fovy/--near/--far replace the
    reference's hard-coded 45 deg / 0.1 / 6 projection (geometry.cpp:30); --light-scale multiplies
    every light's intensity as it is loaded."""
    sc = S.icosphere(3).with_view(width=200, height=150, angles=(0.3, 0.4, 0.0), fovy_deg=60.0, z_near=0.5,
                                  z_far=50.0)
    write_obj(tmp_path / "m.obj", sc)
    write_lights(tmp_path / "l.csv", sc.lights)
    run_cli(["-l", "l.csv", "-o", "m.obj", "--mats-dir", str(tmp_path) + "/", "-x", "200", "-y", "150",
             "--rx", "0.3", "--ry", "0.4", "--flat", "--fovy", "60", "--near", "0.5", "--far", "50",
             "--light-scale", "2", "--out", str(tmp_path)], tmp_path)
    loaded = abi.obj_load(str(tmp_path / "m.obj"), str(tmp_path) + "/")
    lights = np.asarray(sc.lights, np.float32).copy()
    lights[:, 3] *= np.float32(2.0)
    sc2 = S.Scene("obj", loaded["pos"], loaded["tris"], loaded["nrm"], loaded["uv"], loaded["kd"], lights,
                  width=200, height=150, angles=(np.float32(0.3), np.float32(0.4), 0.0), fovy_deg=60.0, z_near=0.5,
                  z_far=50.0)
    cam, nm, l7, _ = abi.scene_frame_inputs(sc2)
    of, od, _, _ = port.draw(sc2, cam, nm, l7, flat=True)
    assert np.array_equal(read_pnm(tmp_path / "frame.ppm"), of)
    assert np.array_equal(read_pnm(tmp_path / "depth.pgm")[0], cimg_normalize_u8(od))
    smooth, _, _, _ = port.draw(sc2, cam, nm, l7)
    assert not np.array_equal(smooth, of)  # the flag changes the picture
