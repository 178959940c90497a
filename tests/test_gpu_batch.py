"""Batched drawing (rast_draw_batch, rast_autotune): every frame of a mixed batch equals the
reference's draw_frame on the same inputs (checked against the oracle port)."""
import numpy as np
import pytest

from rasteriser_gb300 import abi
from rasteriser_gb300 import scenes as S

pytestmark = pytest.mark.gpu

RGB_TOL = 1


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def make_batch(torch, r, n=12, seed=5):
    rng = np.random.default_rng(seed)
    meshes = [S.icosphere(3), S.uv_sphere(96, 48, seed=3), S.soup(5000, 640, 480, seed=8),
              S.soup(3000, 320, 240, seed=9, area_range=(100.0, 4000.0))]
    ids = [r.add_mesh(m.pos, m.nrm, m.uv, m.tris, m.kd) for m in meshes]
    sizes = [(256, 256), (320, 200), (640, 480), (97, 61)]
    frames, keep = [], []
    for i in range(n):
        mi = int(rng.integers(len(meshes)))
        W, H = sizes[int(rng.integers(len(sizes)))]
        nl = int(rng.integers(1, 9))
        sc = meshes[mi].with_view(width=W, height=H, fovy_deg=60.0, z_near=0.1, z_far=100.0,
                                  angles=(float(rng.uniform(-1, 1)), float(rng.uniform(-3, 3)), 0.0),
                                  wind_clockwise=bool(rng.random() < 0.2), lights=S.rig_random(nl, seed=100 + i))
        cam, nm, lights, _ = abi.scene_frame_inputs(sc)
        clear = bool(rng.random() < 0.7)
        init_rgb = rng.integers(0, 256, (3, H, W), dtype=np.uint8)
        init_dep = rng.uniform(-1, 2, (H, W)).astype(np.float32)
        d = {"sc": sc, "cam": cam, "nm": nm, "lights": lights, "clear": clear, "init_rgb": init_rgb,
             "init_dep": init_dep,
             "d_lights": torch.from_numpy(lights).cuda(), "rgb": torch.from_numpy(init_rgb.copy()).cuda(),
             "dep": torch.from_numpy(init_dep.copy()).cuda(), "ids": torch.empty((H, W), dtype=torch.int32).cuda()}
        flags = (abi.CLEAR if clear else 0) | (abi.WIND_CLOCKWISE if sc.wind_clockwise else 0)
        frames.append(r.frame_desc(ids[mi], W, H, flags, cam, nm, d["d_lights"].data_ptr(), nl, d["rgb"].data_ptr(),
                                   d["dep"].data_ptr(), d["ids"].data_ptr()))
        keep.append(d)
    return frames, keep


def reset_outputs(torch, keep):
    for d in keep:
        d["rgb"].copy_(torch.from_numpy(d["init_rgb"]))
        d["dep"].copy_(torch.from_numpy(d["init_dep"]))


def check_against_port(port, keep, stats=None):
    for i, d in enumerate(keep):
        sc = d["sc"]
        f0 = None if d["clear"] else d["init_rgb"]
        d0 = None if d["clear"] else d["init_dep"]
        fp, dp, ip, st = port.draw(sc, d["cam"], d["nm"], d["lights"], f0, d0)
        assert np.array_equal(bits(d["dep"].cpu().numpy()), bits(dp)), f"frame {i} depth"
        assert np.array_equal(d["ids"].cpu().numpy().view(np.uint32), ip), f"frame {i} ids"
        assert np.abs(d["rgb"].cpu().numpy().astype(int) - fp.astype(int)).max() <= RGB_TOL, f"frame {i} rgb"
        if stats is not None:
            assert int(stats[i, 2]) == int(st[2]), f"frame {i} inside fragments"


@pytest.mark.parametrize("lanes,graph", [(1, False), (4, False), (4, True), (3, True)])
def test_batch_matches_port(port, lanes, graph):
    torch = pytest.importorskip("torch")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        r = abi.Renderer(0)
        r.set_stream(s.cuda_stream)
        try:
            frames, keep = make_batch(torch, r)
            for rep in range(2):  # the second run replays the recorded graph
                reset_outputs(torch, keep)
                r.draw_batch(frames, lanes=lanes, graph=graph)
                r.sync()
                check_against_port(port, keep, r.batch_stats(len(frames)))
        finally:
            r.close()


def test_autotune_keeps_results_exact(port):
    torch = pytest.importorskip("torch")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        r = abi.Renderer(0)
        r.set_stream(s.cuda_stream)
        try:
            frames, keep = make_batch(torch, r, n=8, seed=11)
            best = r.autotune(frames, lanes=4, repeats=1)
            assert best["tile"] in (8, 16, 32) and best["row_chunk"] in (4, 8, 32)
            assert best["tile_threads"] in (64, 128, 256, 512)
            assert r.get_option(abi.OPT_TILE_SIZE) == best["tile"]
            reset_outputs(torch, keep)
            r.draw_batch(frames, lanes=4, graph=True)
            r.sync()
            check_against_port(port, keep)
        finally:
            r.close()
