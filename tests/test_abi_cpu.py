"""The C ABI library without a GPU: it builds, loads, exports every declared entry point, and its
host-side geometry (matrices, light transform) equals the reference's."""
import ctypes
import os
import re

import numpy as np
import pytest

import golden_io
from rasteriser_gb300 import abi
from rasteriser_gb300 import scenes as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    """Every function include/*.h declares."""
    names = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            src = open(os.path.join(inc, f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"^[a-z_][a-z_0-9 \*]*?\b(rast_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    lib = abi.load()
    decl = declared_functions()
    assert len(decl) >= 15
    for name in decl:
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_binding_covers_header_exactly():
    assert sorted(abi.SIGNATURES) == declared_functions()


def test_abi_version():
    assert abi.load().rast_abi_version() == 1


def test_frame_matrices_match_reference_bitwise(reference):
    for sc in [S.square_scene(), S.config_icosphere_small(),
               S.config_displaced_sphere(64, 32, 333, 222).with_view(angles=(0.3, 1.1, -0.2), scale=1.7,
                                                                     disp=(0.1, -0.2, 0.3))]:
        mine = abi.frame_matrices(sc.width, sc.height, sc.scale, sc.disp, sc.angles, sc.fovy_deg, sc.z_near, sc.z_far)
        ref = reference.matrices(sc)
        for k in mine:
            assert np.array_equal(mine[k].view(np.uint32), ref[k].view(np.uint32)), k


@pytest.mark.parametrize("name", golden_io.names())
def test_frame_matrices_close_to_golden(name):
    """The goldens were made on x86; another libm may move sin/cos/tan by an ulp."""
    sc, g = golden_io.load(name)
    cam, nm, lights, m = abi.scene_frame_inputs(sc)
    np.testing.assert_allclose(cam, g["camera"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(nm, g["normal"], rtol=1e-5, atol=1e-6)
    # the light transform is a translation-only view and a normalize: exact everywhere
    assert np.array_equal(abi.transform_lights(g["view"], sc.lights).view(np.uint32), g["lights7"].view(np.uint32))


def test_frame_matrices_rejects_zero_size():
    lib = abi.load()
    out = np.zeros(16, np.float32)
    d = np.zeros(3, np.float32)
    p = d.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    o = out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    assert lib.rast_frame_matrices(0, 10, 1.0, p, p, 45.0, 0.1, 6.0, o, o, o, o, o) == 1


def test_status_strings():
    lib = abi.load()
    for s in range(9):
        assert lib.rast_status_string(s)


def test_create_without_gpu_reports_no_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(abi.RastError) as ei:
        abi.Renderer(0)
    assert ei.value.status == 8
