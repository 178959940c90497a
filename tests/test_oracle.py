"""The CPU oracle: the C restatement (port) pinned against the golden fixtures made by the
reference's own draw_frame, and against the compiled reference directly where it is present."""
import numpy as np
import pytest

import golden_io
from rasteriser_gb300 import scenes as S
import edge_scenes as E
import oracle


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("name", golden_io.names())
def test_port_matches_golden(port, name):
    sc, g = golden_io.load(name)
    fr, dp, ids, stats = port.draw(sc, g["camera"], g["normal"], g["lights7"])
    assert np.array_equal(bits(dp), bits(g["depth"])), "depth differs from the reference"
    assert np.array_equal(fr, g["frame"]), "RGB differs from the reference"
    # every pixel the port attributes to a triangle was written by the reference, and vice versa
    changed = (bits(g["depth"]) != bits(np.ones_like(g["depth"]))) | (g["frame"].reshape(3, -1).T.any(1).reshape(
        g["depth"].shape))
    assert np.all((ids != 0xFFFFFFFF) >= changed)


def _live_scenes():
    out = [S.square_scene(), S.plane_scene(), S.config_icosphere_small()]
    for seed in range(4):
        out.append(S.soup(4000 + 997 * seed, 300 + 37 * seed, 200 + 11 * seed, seed=100 + seed,
                          area_range=(0.3, 2000.0)).with_view(wind_clockwise=bool(seed & 1)))
    out.append(S.config_displaced_sphere(96, 48, 333, 222).with_view(angles=(0.7, -0.4, 1.9), scale=0.8,
                                                                      disp=(0.3, 0.1, -0.5)))
    out += E.all_edge_scenes()
    return out


@pytest.mark.parametrize("idx", range(len(_live_scenes())))
def test_port_matches_reference_live(reference, port, idx):
    sc = _live_scenes()[idx]
    fr, dr, td = reference.draw(sc)
    m = reference.matrices(sc)
    fp, dp, _, _ = port.draw(sc, m["camera"], m["normal"], oracle.lights_with_dirs(sc, td))
    assert np.array_equal(bits(dp), bits(dr))
    assert np.array_equal(fp, fr)


def test_port_rmw_matches_reference(reference, port):
    """draw_frame reads the caller's buffers: pixels keep their colour and depth unless beaten."""
    sc = S.soup(6000, 256, 192, seed=11)
    rng = np.random.default_rng(3)
    depth = rng.uniform(-1.5, 1.5, (sc.height, sc.width)).astype(np.float32)
    depth[::7, ::5] = -0.0
    depth[3::11, ::3] = np.nan
    depth[5::13, 1::4] = -np.inf
    frame = rng.integers(0, 256, (3, sc.height, sc.width), dtype=np.uint8)
    fr, dr, td = reference.draw(sc, frame, depth)
    m = reference.matrices(sc)
    fp, dp, _, _ = port.draw(sc, m["camera"], m["normal"], oracle.lights_with_dirs(sc, td), frame, depth)
    assert np.array_equal(bits(dp), bits(dr))
    assert np.array_equal(fp, fr)


def test_camera_override_reproduces_reference_projection(reference):
    """The harness's camera_matrix with 45 deg / 0.1 / 6 is the reference's own (geometry.cpp:30)."""
    sc = S.config_icosphere_small().with_view(fovy_deg=45.0, z_near=0.1, z_far=6.0, angles=(0.2, 0.5, 0.1))
    m = reference.matrices(sc)
    assert np.array_equal(bits(m["camera"]), bits(m["camera45"]))


def test_port_vertex_stage_matches_reference(reference, port):
    rng = np.random.default_rng(0)
    pos = rng.uniform(-2, 2, (5000, 3)).astype(np.float32)
    sc = S.config_icosphere_small()
    cam = reference.matrices(sc)["camera"]
    assert np.array_equal(bits(port.raster_vertices(cam, pos, 640, 480)),
                          bits(reference.raster_vertices(cam, pos, 640, 480)))


def test_port_shade_matches_reference(reference, port):
    rng = np.random.default_rng(1)
    for _ in range(300):
        n = rng.normal(size=3).astype(np.float32)
        n /= np.float32(np.linalg.norm(n))
        alb = rng.uniform(0, 1, 3).astype(np.float32)
        nl = int(rng.integers(0, 9))
        li = np.concatenate([rng.normal(size=(nl, 3)), rng.uniform(0, 300, (nl, 1)), rng.uniform(0, 1, (nl, 3))],
                            axis=1).astype(np.float32)
        assert np.array_equal(port.shade(n, alb, li), reference.shade(n, alb, li))


def _random_views(n, seed):
    rng = np.random.default_rng(seed)
    for _ in range(n):
        yield (int(rng.integers(1, 4000)), int(rng.integers(1, 3000)), float(rng.uniform(0.1, 3.0)),
               rng.uniform(-2, 2, 3).astype(np.float32), rng.uniform(-7, 7, 3).astype(np.float32),
               float(rng.uniform(10, 120)), float(rng.uniform(0.01, 1.0)), float(rng.uniform(2.0, 200.0)))


def test_port_frame_inputs_match_reference(reference, port):
    """The port's restatement of drawing.cpp:221-238 (matrices and Light::transform) gives the
    reference's matrices and transformed lights bit for bit."""
    for sc in _live_scenes()[:8]:
        m = reference.matrices(sc)
        cam, nm, l7, mp = port.frame_inputs(sc)
        for k in ("model", "view", "modelview", "camera", "normal"):
            assert np.array_equal(bits(mp[k]), bits(m[k])), k
        _, _, td = reference.draw(S.square_scene().with_view(lights=sc.lights, width=sc.width, height=sc.height))
        assert np.array_equal(bits(l7[:, :3]), bits(td))


def test_port_frame_inputs_match_librast_host_code(port):
    """librast's host matrices (rast_frame_matrices, rast_transform_lights) and the port's agree
    bit for bit on random views and projections (no GPU is needed for these two calls)."""
    from rasteriser_gb300 import abi
    rng = np.random.default_rng(7)
    for W, H, scale, d, a, fov, zn, zf in _random_views(300, 5):
        mp = port.matrices(W, H, scale, d, a, fov, zn, zf)
        ml = abi.frame_matrices(W, H, scale, d, a, fov, zn, zf)
        for k in mp:
            assert np.array_equal(bits(mp[k]), bits(ml[k])), k
        li = rng.normal(size=(4, 7)).astype(np.float32)
        assert np.array_equal(bits(port.transform_lights(mp["view"], li)), bits(abi.transform_lights(ml["view"], li)))


def test_port_flat_matches_reference_with_face_normals(reference, port):
    """The port's flat mode equals the reference's draw_frame on the same mesh whose vertex normals
    are the per-face normals cross(p1 - p0, p2 - p0) (the reference parses --flat but ignores it,
    so the face normals are given to it as data)."""
    from test_gpu_parity import face_normal_scene
    for sc in (S.config_icosphere_small(),
               S.soup(5000, 300, 200, seed=61, area_range=(0.5, 2000.0)).with_view(wind_clockwise=True),
               S.config_displaced_sphere(96, 48, 333, 222).with_view(angles=(0.7, -0.4, 1.9))):
        fr, dr, td = reference.draw(face_normal_scene(sc))
        m = reference.matrices(sc)
        fp, dp, _, _ = port.draw(sc, m["camera"], m["normal"], oracle.lights_with_dirs(sc, td), flat=True)
        assert np.array_equal(bits(dp), bits(dr))
        assert np.array_equal(fp, fr)
