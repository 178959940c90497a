"""File ingest (OBJ / MTL / lights CSV / raw images) against the reference's own loaders.

The reference's load_obj (fileloader.cpp with the vendored tinyobjloader) and load_lights run from
oracle/_ref; the same files go through librast's parallel loader, and the arrays must be equal
bit for bit: positions, normals, uvs, the Triangle records in order, and untextured materials' Kd.
"""
import os
import shutil

import numpy as np
import pytest

from rasteriser_gb300 import abi

import oracle

# the reference's sample data, where its source tree is present (RAST_REFERENCE)
REF_DATA = os.path.join(oracle.REFERENCE_TREE, "sampledata")


def write(path, text, newline="\n"):
    with open(path, "w", newline="") as fh:
        fh.write(text.replace("\n", newline))
    return path


def assert_same(ours, ref, textured=()):
    for k in ("pos", "nrm", "uv", "tris"):
        assert ours[k].shape == ref[k].shape, k
        assert np.array_equal(ours[k].view(np.uint32) if ours[k].dtype == np.float32 else ours[k],
                              ref[k].view(np.uint32) if ref[k].dtype == np.float32 else ref[k]), k
    assert ours["kd"].shape == ref["kd"].shape
    for i in range(ours["kd"].shape[0]):
        if i not in textured:
            assert np.array_equal(ours["kd"][i], ref["kd"][i]), i


MTL = """# two materials
newmtl A
Kd 0.25 0.5 0.75
newmtl B
Ka 1 1 1
Kd 1e-1 2.5E-1 +0.3
"""

CASES = {
    "fans_and_corners": """v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 0.5 1.5 0
vt 0 0
vt 1 0
vt 1 1
vn 0 0 1
vn 0 1 0
f 1/1/1 2/2/1 3/3/1 4/1/2 5/2/2
f -5//1 -4//2 -3//1
f 1 2 3
f 1/1 2/2 3/3
f\t2/3/2\t3/1/1   4/2/2
""",
    "numbers": """v 1e-3 -2.5E+2 +3
v -.5 .25 1.
v 123456789.123456789 0.000000001 7e10
v 0.1 0.2 0.30000000000000004
v 1
vn 0.57735026918962576451 -0.57735026918962576451 5e-324
vt 0.999999999 1.00000001
f 1//1 2//1 3//1 4//1 5//1
""",
    "materials_and_groups": """mtllib mats.mtl
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
vn 0 0 1
o first
usemtl A
f 1//1 2//1 3//1
usemtl B
f 1//1 3//1 4//1
g second
f 2//1 3//1 4//1
usemtl A
f 1//1 2//1 4//1
usemtl B
g third
f 1//1 2//1 3//1
usemtl missing
f 2//1 3//1 4//1
usemtl A
usemtl A
f 3//1 4//1 1//1
""",
    "comments_blank_lines": """# a comment

   v 0 0 0
v 1 0 0 # trailing words are ignored
v 0 1 0
vn 0 0 1

f 1//1 2//1 3//1
  # indented comment
f 3//1 2//1 1//1
""",
}


@pytest.mark.parametrize("newline", ["\n", "\r\n"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_obj_cases_match_reference(reference, tmp_path, case, newline):
    write(tmp_path / "mats.mtl", MTL, newline)
    obj = write(tmp_path / f"{case}.obj", CASES[case], newline)
    mats_dir = str(tmp_path) + os.sep
    ours = abi.obj_load(obj, mats_dir)
    ref = reference.load_obj(str(obj), mats_dir)
    assert_same(ours, ref)


def test_fan_and_indices_explicit(tmp_path):
    obj = write(tmp_path / "f.obj", CASES["fans_and_corners"])
    d = abi.obj_load(obj)
    t = d["tris"]
    # pentagon 1/1/1 2/2/1 3/3/1 4/1/2 5/2/2 -> fan (0,1,2), (0,2,3), (0,3,4)
    assert t[:3, 0:3].tolist() == [[0, 1, 2], [0, 2, 3], [0, 3, 4]]
    assert t[:3, 3:6].tolist() == [[0, 0, 0], [0, 0, 1], [0, 1, 1]]  # normals
    assert t[:3, 6:9].tolist() == [[0, 1, 2], [0, 2, 0], [0, 0, 1]]  # uvs
    assert t[3, 0:9].tolist() == [0, 1, 2, 0, 1, 0, -1, -1, -1]      # -5//1 -4//2 -3//1 with 5 vertices
    assert t[4, 3:9].tolist() == [-1] * 6                              # f 1 2 3
    assert t[5, 3:6].tolist() == [-1] * 3 and t[5, 6:9].tolist() == [0, 1, 2]
    assert (t[:, 9] == -1).all()                                       # no usemtl


def test_number_quirks(tmp_path):
    """The vendored parser: no digit before '.' is not a number (0), '1.' is 1, exponents scale."""
    d = abi.obj_load(write(tmp_path / "n.obj", CASES["numbers"]))
    p = d["pos"]
    assert p[1].tolist() == [0.0, 0.0, 1.0]
    assert p[0].tolist() == [np.float32(1e-3), np.float32(-250.0), 3.0]
    assert p[4].tolist() == [1.0, 0.0, 0.0]


def test_usemtl_group_quirk(tmp_path):
    """Faces flushed by `usemtl` just before a `g` with no faces of its own are dropped, as by the
    vendored tinyobjloader."""
    write(tmp_path / "mats.mtl", MTL)
    d = abi.obj_load(write(tmp_path / "g.obj", CASES["materials_and_groups"]), str(tmp_path) + os.sep)
    mats = d["tris"][:, 9].tolist()
    # shape 'first': A, B (kept by 'g second'); shape 'second': f 2 3 4 with B kept? no: its group
    # was flushed by 'usemtl A', then 'f 1 2 4' (A) flushed by 'usemtl B', then 'g third' had no
    # faces of its own, so shape 'second' is dropped; the rest: B, missing (-1), A.
    assert mats == [0, 1, 1, -1, 0]
    assert d["kd"].tolist() == [[0.25, 0.5, 0.75], [np.float32(0.1), 0.25, np.float32(0.3)]]
    assert d["textures"] == ["", ""]


def test_suzanne_matches_reference(reference, tmp_path):
    """Suzanne with its map_Kd pointed at a PPM (CImg reads PPM natively; PNG needs a codec)."""
    src = os.path.join(REF_DATA, "Suzanne.obj")
    if not os.path.exists(src):
        pytest.skip("reference sample data not present")
    shutil.copy(src, tmp_path / "Suzanne.obj")
    mtl = open(os.path.join(REF_DATA, "Suzanne.mtl")).read().replace("SuzanneTex.png", "tex.ppm")
    write(tmp_path / "Suzanne.mtl", mtl)
    rng = np.random.default_rng(1)
    img = rng.integers(0, 256, (16, 24, 3), dtype=np.uint8)
    with open(tmp_path / "tex.ppm", "wb") as fh:
        fh.write(b"P6\n24 16\n255\n" + img.tobytes())
    d = str(tmp_path) + os.sep
    ours = abi.obj_load(str(tmp_path / "Suzanne.obj"), d)
    ref = reference.load_obj(str(tmp_path / "Suzanne.obj"), d)
    assert_same(ours, ref, textured={0})
    assert ours["tris"].shape[0] == 968 or ours["tris"].shape[0] > 0
    assert ours["textures"] == [d + "tex.ppm"]


def big_obj(path, n=420, m=380, seed=5):
    """A grid of quads with normals, uvs, material switches and groups; > 1 MB so the loader
    splits it over threads."""
    rng = np.random.default_rng(seed)
    lines = ["mtllib mats.mtl"]
    xs = rng.random((n * m, 3)) * 4 - 2
    lines += ["v %.9f %.9f %.9f" % tuple(x) for x in xs]
    lines += ["vn %.6f %.6f %.6f" % tuple(x) for x in rng.normal(size=(97, 3))]
    lines += ["vt %.7f %.7f" % tuple(x) for x in rng.random((131, 2))]
    for j in range(m - 1):
        if j % 37 == 0:
            lines.append("usemtl %s" % ("A" if (j // 37) % 2 == 0 else "B"))
        if j % 53 == 11:
            lines.append("g band%d" % j)
        for i in range(n - 1):
            a, b, c, dd = j * n + i + 1, j * n + i + 2, (j + 1) * n + i + 2, (j + 1) * n + i + 1
            k = (i * 7 + j * 3) % 97 + 1
            u = (i + j) % 131 + 1
            if (i + j) % 5 == 0:
                lines.append("f %d/%d/%d %d/%d/%d %d/%d/%d" % (a, u, k, b, u, k, c, u, k))
            else:
                lines.append("f %d/%d/%d %d/%d/%d %d/%d/%d %d/%d/%d" % (a, u, k, b, u, k, c, u, k, dd, u, k))
    write(path, "\n".join(lines) + "\n")
    return path


def test_large_obj_parallel_matches_reference(reference, tmp_path):
    write(tmp_path / "mats.mtl", MTL)
    obj = big_obj(tmp_path / "big.obj")
    assert os.path.getsize(obj) > (1 << 20)
    d = str(tmp_path) + os.sep
    assert_same(abi.obj_load(str(obj), d), reference.load_obj(str(obj), d))


def test_missing_obj_is_an_error(tmp_path):
    with pytest.raises(abi.RastError):
        abi.obj_load(str(tmp_path / "nope.obj"))


@pytest.mark.parametrize("name", ["threepoint.csv", "normalmap.csv"])
def test_lights_match_reference(reference, name):
    path = os.path.join(REF_DATA, name)
    if not os.path.exists(path):
        pytest.skip("reference sample data not present")
    ours = abi.lights_load(path)
    assert np.array_equal(ours, reference.load_lights(path))


def test_lights_variants(tmp_path):
    p = write(tmp_path / "l.csv", "1, -0.5,-1,512,1,1,0.9\n\n-1,0,-1,256,1,1,0.5\n", "\r\n")
    li = abi.lights_load(p)
    assert li.shape == (2, 7)
    assert li[0].tolist() == [1.0, -0.5, -1.0, 512.0, 1.0, 1.0, np.float32(0.9)]
    with pytest.raises(abi.RastError):
        abi.lights_load(write(tmp_path / "bad.csv", "1,2,3\n"))


def test_images(tmp_path):
    rng = np.random.default_rng(2)
    img = rng.integers(0, 256, (5, 7, 3), dtype=np.uint8)
    with open(tmp_path / "a.ppm", "wb") as fh:
        fh.write(b"P6\n# comment\n7 5\n255\n" + img.tobytes())
    got = abi.image_load(str(tmp_path / "a.ppm"))
    assert got.shape == (3, 5, 7)
    assert np.array_equal(got, np.moveaxis(img, 2, 0).astype(np.float32))
    img16 = rng.integers(0, 65536, (4, 3, 3), dtype=np.uint16)
    with open(tmp_path / "b.ppm", "wb") as fh:
        fh.write(b"P6 3 4 65535\n" + img16.astype(">u2").tobytes())
    assert np.array_equal(abi.image_load(str(tmp_path / "b.ppm")), np.moveaxis(img16, 2, 0).astype(np.float32))
    g = rng.integers(0, 256, (3, 4), dtype=np.uint8)
    write(tmp_path / "c.pgm", "P2\n4 3\n255\n" + " ".join(str(v) for v in g.ravel()) + "\n")
    assert np.array_equal(abi.image_load(str(tmp_path / "c.pgm"))[0], g.astype(np.float32))
    f = rng.random((3, 2, 3)).astype(np.float32)
    with open(tmp_path / "d.pfm", "wb") as fh:
        fh.write(b"PF\n2 3\n-1.0\n" + f[::-1].astype("<f4").tobytes())  # PFM rows bottom first
    assert np.array_equal(abi.image_load(str(tmp_path / "d.pfm")), np.moveaxis(f, 2, 0))
    with pytest.raises(abi.RastError):
        abi.image_load(write(tmp_path / "x.txt", "hello"))
