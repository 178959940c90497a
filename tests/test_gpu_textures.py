"""Textured materials on the GPU against the oracle port (whose texture sampling is pinned to the
reference's draw_frame in test_textures.py): depth, coverage and RGB bit for bit."""
import subprocess

import numpy as np
import pytest

import oracle
from test_textures import textured_cases, normalised, write_ppm
from rasteriser_gb300 import _build, abi
from rasteriser_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rnd():
    r = abi.Renderer(0)
    yield r
    r.close()


def raw_chw(raw_hwc):
    return np.moveaxis(raw_hwc.astype(np.float32), 2, 0)


@pytest.mark.parametrize("shader", [abi.SHADER_EXACT, abi.SHADER_EXACT_DEFERRED])
@pytest.mark.parametrize("case", ["square", "sphere_16bit", "sphere_clamped_uvs", "constant_texture",
                                  "textured_and_plain"])
def test_textures_match_port(rnd, port, tmp_path, case, shader):
    sc, _, raws = textured_cases(tmp_path)[case]
    rnd.upload_scene_mesh(sc)
    for m, r in enumerate(raws):
        rnd.upload_texture(m, None if r is None else raw_chw(r))
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    rnd.set_lights(lights)
    rnd.set_option(abi.OPT_SHADER, shader)
    try:
        f, d, ids = rnd.draw(cam, nm, sc.width, sc.height, abi.CLEAR, want_ids=True)
    finally:
        rnd.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)
    of, od, oids, _ = port.draw(sc, cam, nm, lights, textures=[normalised(r) for r in raws])
    assert np.array_equal(d.view(np.uint32), od.view(np.uint32))
    assert np.array_equal(ids, oids)
    assert np.array_equal(f, of), f"RGB differs at {np.argwhere(f != of)[:5]}"
    rnd._mesh_digest = None


def test_texture_removed_and_validated(rnd, port, tmp_path):
    sc, _, raws = textured_cases(tmp_path)["square"]
    rnd.upload_scene_mesh(sc)
    rnd.upload_texture(0, raw_chw(raws[0]))
    rnd.upload_texture(0, None)
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    rnd.set_lights(lights)
    f, _, _ = rnd.draw(cam, nm, sc.width, sc.height, abi.CLEAR)
    of, _, _, _ = port.draw(sc, cam, nm, lights)
    assert np.array_equal(f, of)
    with pytest.raises(abi.RastError):
        rnd.upload_texture(0, np.zeros((1, 4, 4), np.float32))   # one channel
    with pytest.raises(abi.RastError):
        rnd.upload_texture(5, np.zeros((3, 4, 4), np.float32))   # no such material
    rnd._mesh_digest = None


def test_cli_renders_obj_texture(port, tmp_path):
    sc = S.with_spherical_uvs(S.icosphere(3)).with_view(width=160, height=120)
    rng = np.random.default_rng(9)
    raw = rng.integers(0, 256, (12, 20, 3), dtype=np.uint16)
    write_ppm(tmp_path / "tex.ppm", raw)
    with open(tmp_path / "m.obj", "w") as fh:
        for p in sc.pos:
            fh.write("v %r %r %r\n" % tuple(float(v) for v in p))
        for t in sc.uv:
            fh.write("vt %r %r\n" % tuple(float(v) for v in t))
        for n in sc.nrm:
            fh.write("vn %r %r %r\n" % tuple(float(v) for v in n))
        fh.write("mtllib m.mtl\nusemtl T\n")
        for t in sc.tris:
            fh.write("f %d/%d/%d %d/%d/%d %d/%d/%d\n" % (t[0] + 1, t[6] + 1, t[3] + 1, t[1] + 1, t[7] + 1, t[4] + 1,
                                                         t[2] + 1, t[8] + 1, t[5] + 1))
    with open(tmp_path / "m.mtl", "w") as fh:
        fh.write("newmtl T\nKd 0.5 0.5 0.5\nmap_Kd tex.ppm\n")
    with open(tmp_path / "l.csv", "w") as fh:
        for L in sc.lights:
            fh.write(",".join(repr(float(v)) for v in L) + "\n")
    r = subprocess.run([_build.cli_path(), "-l", "l.csv", "-o", "m.obj", "--mats-dir", str(tmp_path) + "/",
                        "-x", "160", "-y", "120", "--out", str(tmp_path)], cwd=tmp_path, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    loaded = abi.obj_load(str(tmp_path / "m.obj"), str(tmp_path) + "/")
    sc2 = S.Scene("obj", loaded["pos"], loaded["tris"], loaded["nrm"], loaded["uv"], loaded["kd"], sc.lights,
                  width=160, height=120)
    cam, nm, lights, _ = abi.scene_frame_inputs(sc2)
    of, _, _, _ = port.draw(sc2, cam, nm, lights, textures=[normalised(raw)])
    with open(tmp_path / "frame.ppm", "rb") as fh:
        data = fh.read()
    img = np.frombuffer(data[-160 * 120 * 3:], np.uint8).reshape(120, 160, 3)
    assert np.array_equal(np.moveaxis(img, 2, 0), of)
