"""Full-size parity of the two added workloads, through the C ABI, against the oracle port.

- The many-light frame: the 1,046,528-triangle displaced sphere with smooth normals and per-vertex
  albedo at 1920x1080 under 256 lights. The exact shaders (fused into the resolve pass, and the
  deferred plain per-light shader) give the port's depth, triangle ids and colour bit for bit
  (shading.cpp:20-34 in its order). The learned shader, with either network, keeps depth and ids
  bit-exact, and its colour stays within mean 0.5/255 and max 1/255 of the port's.
- The uneven batch: all 256 frames (icospheres L2-L7, soups of 1k-500k triangles, four
  resolutions, 1-8 lights) drawn by rast_draw_batch as one CUDA graph over 8 lanes with the
  autotuner's options; eight frames, among them the L7 icosphere and the largest soup at 1920x1080,
  are compared with the port's draw_frame (drawing.cpp:205-258) bit for bit.
"""
import numpy as np
import pytest

from rasteriser_gb300 import abi
from rasteriser_gb300 import scenes as S

pytestmark = pytest.mark.gpu

MEAN_TOL = 0.5  # learned shader: mean absolute channel error over covered pixels, 1/255 units
MAX_TOL = 1     # learned shader: largest channel error, 1/255 units


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def many_lights(port):
    """The many-light frame, the port's draw of it, and a renderer holding the mesh and lights."""
    sc = S.config_many_lights()
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    of, od, oids, _ = port.draw(sc, cam, nm, lights)
    r = abi.Renderer(0)
    r.upload_scene_mesh(sc)
    r.set_lights(lights)
    yield sc, cam, nm, (of, od, oids), r
    r.close()


@pytest.mark.parametrize("shader", [abi.SHADER_EXACT, abi.SHADER_EXACT_DEFERRED])
def test_many_lights_exact_shaders_full_size(many_lights, shader):
    sc, cam, nm, (of, od, oids), r = many_lights
    assert sc.ntri == 1_046_528 and (sc.width, sc.height) == (1920, 1080) and sc.lights.shape[0] == 256
    r.set_option(abi.OPT_SHADER, shader)
    try:
        f, d, ids = r.draw(cam, nm, sc.width, sc.height, abi.CLEAR, want_ids=True)
    finally:
        r.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)
    assert np.array_equal(bits(d), bits(od)), "depth"
    assert np.array_equal(ids, oids), "triangle ids"
    assert np.array_equal(f, of), f"RGB differs at {np.argwhere(f != of)[:5]}"


@pytest.mark.parametrize("network", [abi.MLP_COMPACT, abi.MLP_WIDE])
def test_many_lights_learned_shader_full_size(many_lights, network):
    """Both networks: the compact default and the 16-frequency 64-64 one the workload names."""
    sc, cam, nm, (of, od, oids), r = many_lights
    r.set_option(abi.OPT_MLP_NETWORK, network)
    try:
        st = r.mlp_train(samples=4 << 20, epochs=24, seed=3)
    finally:
        r.set_option(abi.OPT_MLP_NETWORK, abi.MLP_COMPACT)
    r.set_option(abi.OPT_SHADER, abi.SHADER_LEARNED)
    try:
        f, d, ids = r.draw(cam, nm, sc.width, sc.height, abi.CLEAR, want_ids=True)
        checks = r.shade_stats()
    finally:
        r.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)
    assert np.array_equal(bits(d), bits(od)), "depth must stay exact"
    assert np.array_equal(ids, oids), "coverage must stay exact"
    cov = oids != abi.NO_TRIANGLE
    diff = np.abs(f.astype(np.int16) - of.astype(np.int16))
    print("training", st, "checks", checks, "mean", diff[:, cov].mean(), "max", diff.max())
    assert np.all(diff[:, ~cov] == 0)
    assert diff[:, cov].mean() <= MEAN_TOL
    assert diff.max() <= MAX_TOL


# batch frames compared with the port: the L7 icosphere and the largest soup (381,010 triangles)
# at 1920x1080 and at 1280x720, a 1920x1080 frame, and three more
BATCH_SAMPLE = [189, 210, 71, 62, 1, 0, 100, 255]


def test_uneven_batch_full_size(port):
    torch = pytest.importorskip("torch")
    meshes, frames = S.batch_workload()
    assert len(frames) == 256 and frames[189][0] == 5 and meshes[5].ntri == 327_680
    assert meshes[frames[210][0]].ntri == max(m.ntri for m in meshes) and frames[210][1:3] == (1920, 1080)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        r = abi.Renderer(0)
        r.set_stream(s.cuda_stream)
        try:
            ids = [r.add_mesh(m.pos, m.nrm, m.uv, m.tris, m.kd) for m in meshes]
            descs, keep = [], []
            for fr in frames:
                mi, W, H = fr[0], fr[1], fr[2]
                sc = S.batch_frame_scene(meshes, fr)
                cam, nm, l7, _ = abi.scene_frame_inputs(sc)
                d = {"sc": sc, "cam": cam, "nm": nm, "l7": l7, "d_l7": torch.from_numpy(l7).cuda(),
                     "rgb": torch.empty(3 * W * H, dtype=torch.uint8, device="cuda"),
                     "dep": torch.empty(W * H, dtype=torch.float32, device="cuda"),
                     "ids": torch.empty(W * H, dtype=torch.int32, device="cuda")}
                keep.append(d)
                descs.append(r.frame_desc(ids[mi], W, H, abi.CLEAR, cam, nm, d["d_l7"].data_ptr(), l7.shape[0],
                                          d["rgb"].data_ptr(), d["dep"].data_ptr(), d["ids"].data_ptr()))
            tuned = r.autotune(descs, lanes=8, repeats=1)
            print("autotuned", tuned)
            for _ in range(2):  # recorded, then replayed
                for d in keep:
                    d["rgb"].fill_(7)
                    d["dep"].fill_(-5.0)
                r.draw_batch(descs, lanes=8, graph=True)
                r.sync()
                for i in BATCH_SAMPLE:
                    d = keep[i]
                    sc = d["sc"]
                    fp, dp, ip, _ = port.draw(sc, d["cam"], d["nm"], d["l7"])
                    H, W = sc.height, sc.width
                    assert np.array_equal(bits(d["dep"].cpu().numpy().reshape(H, W)), bits(dp)), f"frame {i} depth"
                    assert np.array_equal(d["ids"].cpu().numpy().view(np.uint32).reshape(H, W), ip), f"frame {i} ids"
                    assert np.array_equal(d["rgb"].cpu().numpy().reshape(3, H, W), fp), f"frame {i} rgb"
        finally:
            r.close()
