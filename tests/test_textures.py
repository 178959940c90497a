"""Texture sampling (Material::sample with a texture, material.cpp:11-26): the oracle port against
the reference's own draw_frame, which loads each texture through CImg (PPM read natively),
normalises it to 0..1 and samples it with linear_atXY at the perspective-correct uv."""
import os

import numpy as np
import pytest

import oracle
from rasteriser_gb300 import abi
from rasteriser_gb300 import scenes as S


def write_ppm(path, img_hwc, maxval=255):
    h, w, c = img_hwc.shape
    assert c == 3
    with open(path, "wb") as fh:
        fh.write(b"P6\n%d %d\n%d\n" % (w, h, maxval))
        fh.write(img_hwc.astype(">u2" if maxval > 255 else np.uint8).tobytes())
    return str(path)


def textured_cases(tmp_path):
    rng = np.random.default_rng(7)
    t1 = rng.integers(0, 256, (13, 21, 3), dtype=np.uint16)
    t1[0, 0] = [0, 0, 0]
    t2 = rng.integers(1000, 60000, (8, 5, 3), dtype=np.uint16)
    t3 = np.full((4, 4, 3), 77, np.uint16)  # constant: normalises to 0
    p1 = write_ppm(tmp_path / "t1.ppm", t1)
    p2 = write_ppm(tmp_path / "t2.ppm", t2, 65535)
    p3 = write_ppm(tmp_path / "t3.ppm", t3)
    sq = S.square_scene().with_view(width=160, height=120, angles=(0.2, -0.4, 0.1))
    sph = S.with_spherical_uvs(S.icosphere(3)).with_view(width=200, height=150, angles=(0.3, 1.1, 0.0))
    wide = S.with_spherical_uvs(S.icosphere(2), scale=1.6, offset=-0.3).with_view(width=180, height=140)
    two = S.with_spherical_uvs(S.icosphere(3)).with_view(width=170, height=130, angles=(-0.2, 0.7, 0.0))
    tris = two.tris.copy()
    tris[::2, 9] = 1
    two = two.with_view(tris=tris, kd=np.array([[0.8, 0.8, 0.8], [0.2, 0.9, 0.4]], np.float32))
    return {
        "square": (sq, [p1], [t1]),
        "sphere_16bit": (sph, [p2], [t2]),
        "sphere_clamped_uvs": (wide, [p1], [t1]),
        "constant_texture": (sph, [p3], [t3]),
        "textured_and_plain": (two, [p1, None], [t1, None]),
    }


def normalised(raw_hwc):
    return None if raw_hwc is None else oracle.cimg_normalize01(np.moveaxis(raw_hwc.astype(np.float32), 2, 0))


@pytest.mark.parametrize("case", ["square", "sphere_16bit", "sphere_clamped_uvs", "constant_texture",
                                  "textured_and_plain"])
def test_port_textures_match_reference(reference, port, tmp_path, case):
    sc, paths, raws = textured_cases(tmp_path)[case]
    rf, rd, td = reference.draw(sc, textures=paths)
    cam = reference.matrices(sc)["camera"]
    nm = reference.matrices(sc)["normal"]
    lights = oracle.lights_with_dirs(sc, td)
    pf, pd, _, _ = port.draw(sc, cam, nm, lights, textures=[normalised(r) for r in raws])
    assert np.array_equal(pd.view(np.uint32), rd.view(np.uint32))
    assert np.array_equal(pf, rf), f"RGB differs at {np.argwhere(pf != rf)[:5]}"


def test_texture_changes_the_frame(port, tmp_path):
    sc, _, raws = textured_cases(tmp_path)["square"]
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    plain, _, _, _ = port.draw(sc, cam, nm, lights)
    tex, _, _, _ = port.draw(sc, cam, nm, lights, textures=[normalised(raws[0])])
    assert (plain != tex).any()
