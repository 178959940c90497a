"""The seeded workloads have the named shapes and are reproducible."""
import numpy as np

import golden_io
from rasteriser_gb300 import scenes as S


def test_icosphere_level4_counts():
    sc = S.config_icosphere_small()
    assert sc.pos.shape == (2562, 3) and sc.ntri == 5120
    assert (sc.width, sc.height) == (640, 480)
    np.testing.assert_allclose(np.linalg.norm(sc.pos, axis=1), 1.0, atol=1e-6)


def test_displaced_sphere_counts():
    sc = S.config_displaced_sphere()
    assert sc.pos.shape == (523_266, 3) and sc.ntri == 1_046_528
    assert sc.nrm.shape == (1_046_528, 3)
    r = np.linalg.norm(sc.pos.astype(np.float64), axis=1)
    assert abs(r.mean() - 1.0) < 1e-3 and 0.015 < r.std() < 0.025


def test_soup_shape_statistics():
    sc = S.soup(50_000, 3840, 2160, seed=2)
    assert sc.ntri == 50_000 and sc.pos.shape == (150_000, 3)
    z = -(sc.pos[:, 2].astype(np.float64) - 3.0)
    assert z.min() > 1.8 and z.max() < 52.5


def test_generators_are_deterministic():
    a, b = S.soup(5000, 640, 480, seed=9), S.soup(5000, 640, 480, seed=9)
    assert a.mesh_digest() == b.mesh_digest()
    assert S.config_displaced_sphere(64, 32).mesh_digest() == S.config_displaced_sphere(64, 32).mesh_digest()


def test_full_size_inputs_match_the_golden_digests():
    """The full-size meshes regenerate bit for bit (this also holds across x86 and aarch64)."""
    full = golden_io.full_size()
    e = full["displaced_sphere_frame0"]
    assert golden_io.full_size_scene(e).mesh_digest() == e["mesh"]


def test_det_sincos_accuracy():
    t = np.linspace(-20, 20, 10001)
    s, c = S.det_sincos(t)
    assert np.max(np.abs(s - np.sin(t))) < 1e-14 and np.max(np.abs(c - np.cos(t))) < 1e-14
    x = np.linspace(-5, 7, 1001)
    assert np.max(np.abs(S.det_exp(x) / np.exp(x) - 1)) < 1e-14
