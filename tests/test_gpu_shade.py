"""Deferred and learned shading through the C ABI.

- EXACT_DEFERRED gives the reference's colour bit for bit (oracle port), like the fused EXACT mode.
- Per-vertex albedo (the many-light workload's material) matches the oracle port bit for bit.
- The tensor-core MLP kernel matches a float64 numpy forward pass of the same BF16 network.
- LEARNED keeps depth and triangle ids bit-exact and the colour within the error bound.
"""
import numpy as np
import pytest

import mlp_ref
from rasteriser_gb300 import abi
from rasteriser_gb300 import scenes as S

pytestmark = pytest.mark.gpu

RGB_TOL = 1          # per channel, 1/255 units, for the learned shader's frame
MEAN_TOL = 0.5       # mean absolute channel error over covered pixels, learned shader


@pytest.fixture(scope="module")
def rnd():
    r = abi.Renderer(0)
    yield r
    r.close()


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def draw(r, sc, shader, clear=True):
    r.set_option(abi.OPT_SHADER, shader)
    try:
        return r.draw_scene(sc, clear=clear)
    finally:
        r.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)


def oracle_frame(port, sc):
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    f, d, ids, _ = port.draw(sc, cam, nm, lights)
    return f, d, ids


def small_many_lights(n_lights=16, w=320, h=240, seg=(96, 48)):
    return S.config_many_lights(seg[0], seg[1], w, h, n_lights).with_view(angles=(0.2, 0.7, 0.0))


SCENES = {
    "icosphere4": lambda: S.config_icosphere_small(),
    "soup": lambda: S.soup(20000, 320, 200, seed=31, area_range=(0.5, 2000.0)),
    "many_lights16": lambda: small_many_lights(16),
    "sphere_cw": lambda: S.config_displaced_sphere(128, 64, 257, 131).with_view(wind_clockwise=True),
}


@pytest.mark.parametrize("name", sorted(SCENES))
@pytest.mark.parametrize("shader", [abi.SHADER_EXACT, abi.SHADER_EXACT_DEFERRED])
def test_exact_modes_match_oracle(rnd, port, name, shader):
    sc = SCENES[name]()
    f, d, ids = draw(rnd, sc, shader)
    of, od, oids = oracle_frame(port, sc)
    assert np.array_equal(bits(d), bits(od))
    assert np.array_equal(ids, oids)
    assert np.array_equal(f, of), f"RGB differs at {np.argwhere(f != of)[:5]}"


def test_deferred_read_modify_write(rnd, port):
    """Without RAST_CLEAR the frame and depth coming in are kept where nothing wins."""
    sc = small_many_lights(8)
    rng = np.random.default_rng(3)
    frame0 = rng.integers(0, 256, (3, sc.height, sc.width), dtype=np.uint8)
    depth0 = np.where(rng.random((sc.height, sc.width)) < 0.5, 1.0, 0.97).astype(np.float32)
    rnd.set_option(abi.OPT_SHADER, abi.SHADER_EXACT_DEFERRED)
    try:
        f, d, ids = rnd.draw_scene(sc, frame=frame0.copy(), depth=depth0.copy())
    finally:
        rnd.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    of, od, oids, _ = port.draw(sc, cam, nm, lights, frame=frame0, depth=depth0)
    assert np.array_equal(bits(d), bits(od))
    assert np.array_equal(ids, oids)
    assert np.array_equal(f, of)


def test_vertex_albedo_removed(rnd, port):
    sc = small_many_lights(4)
    rnd.upload_scene_mesh(sc)
    rnd.upload_vertex_albedo(None)  # back to Kd
    plain = sc.with_view(vertex_albedo=None)
    cam, nm, lights, _ = abi.scene_frame_inputs(plain)
    rnd.set_lights(lights)
    f, d, ids = rnd.draw(cam, nm, plain.width, plain.height, abi.CLEAR, want_ids=True)
    of, od, oids = oracle_frame(port, plain)
    assert np.array_equal(f, of) and np.array_equal(bits(d), bits(od))
    rnd._mesh_digest = None


def test_vertex_albedo_size_checked(rnd):
    sc = small_many_lights(4)
    rnd.upload_scene_mesh(sc)
    with pytest.raises(abi.RastError):
        rnd.upload_vertex_albedo(np.zeros((sc.pos.shape[0] - 1, 3), np.float32))
    rnd._mesh_digest = None


def test_options_validated(rnd):
    for opt, bad in [(abi.OPT_SHADER, 3), (abi.OPT_MLP_SAMPLES, 5), (abi.OPT_MLP_SAMPLES, -1),
                     (abi.OPT_MLP_BOUND_MILLI, -1), (abi.OPT_MLP_NETWORK, 2), (abi.OPT_MLP_NETWORK, -1)]:
        with pytest.raises(abi.RastError):
            rnd.set_option(opt, bad)
    assert rnd.get_option(abi.OPT_SHADER) == abi.SHADER_EXACT
    assert rnd.get_option(abi.OPT_MLP_SAMPLES) == 2
    assert rnd.get_option(abi.OPT_MLP_BOUND_MILLI) == 500


@pytest.mark.parametrize("net", sorted(mlp_ref.NETWORKS))
def test_mlp_kernel_matches_numpy(rnd, net):
    """The tcgen05 path against a float64 forward pass of the same BF16 weights, for each network."""
    w = mlp_ref.random_weights(7, net=net)
    rnd.mlp_load(mlp_ref.make_blob(w))
    rng = np.random.default_rng(11)
    n = 5000  # 40 tiles, the last one partial
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    nv = v.astype(np.float32)
    alb = rng.random((n, 3)).astype(np.float32)
    got = rnd.mlp_eval(nv, alb)
    want = mlp_ref.forward(w, nv, alb)
    err = np.abs(got - want)
    scale = float(w["scale"])
    # Sums agree to FP32 rounding except where a feature or hidden value sits on a BF16 rounding
    # boundary and the kernel's feature recurrence (hardware sine, FP32) rounds it the other way
    # than numpy's float64 sine: one BF16 step in one input moves the output by ~1e-2 * scale.
    tight = err <= 1e-4 * scale + 1e-4 * np.abs(want)
    assert tight.mean() > 0.95, f"only {tight.mean():.4f} of the outputs agree to FP32 rounding"
    tol = 0.02 * np.abs(want) + 0.01 * scale
    assert np.all(err <= tol), f"max err {err.max()} at {np.unravel_index(err.argmax(), err.shape)}"


@pytest.mark.parametrize("net", sorted(mlp_ref.NETWORKS))
def test_mlp_blob_round_trip(rnd, net):
    w = mlp_ref.random_weights(8, net=net)
    blob = mlp_ref.make_blob(w, n_lights=3, lights_hash=12345, loss=0.25)
    rnd.mlp_load(blob)
    assert rnd.mlp_save() == blob
    back = mlp_ref.parse_blob(rnd.mlp_save())
    for k in ("w1", "w2", "w3"):
        assert np.array_equal(back[k], np.asarray(w[k], np.float32))


def test_mlp_blob_refused(rnd):
    blob = bytearray(mlp_ref.make_blob(mlp_ref.random_weights(9)))
    with pytest.raises(abi.RastError):
        rnd.mlp_load(bytes(blob[:-4]))
    bad = bytearray(blob)
    bad[0:4] = b"XMLP"
    with pytest.raises(abi.RastError):
        rnd.mlp_load(bytes(bad))
    other = bytearray(blob)
    other[8:12] = (102).to_bytes(4, "little")  # n_in of no network
    with pytest.raises(abi.RastError):
        rnd.mlp_load(bytes(other))
    mixed = bytearray(blob)
    mixed[12:16] = (64).to_bytes(4, "little")  # the compact inputs with the wide hidden width
    with pytest.raises(abi.RastError):
        rnd.mlp_load(bytes(mixed))


def test_exact_eval_matches_oracle_shade(rnd, port):
    lights = S.rig_random(256, 21)
    rnd.set_lights(lights)
    rng = np.random.default_rng(5)
    n = 700
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    nv = v.astype(np.float32)
    alb = rng.random((n, 3)).astype(np.float32)
    got = rnd.mlp_eval(nv, alb, exact=True)
    gb = np.minimum(got, 255.0).astype(np.uint32)
    for i in range(n):
        assert np.array_equal(gb[i], port.shade(nv[i], alb[i], lights)), i


@pytest.fixture(scope="module")
def trained(rnd):
    """A learned shader for a 256-light rig, trained on 4M samples for 24 epochs."""
    sc = small_many_lights(256, 640, 480, (256, 128))
    _, _, lights, _ = abi.scene_frame_inputs(sc)
    rnd.set_lights(lights)
    stats = rnd.mlp_train(samples=4 << 20, epochs=24, seed=3)
    return sc, lights, stats, rnd.mlp_save()


def test_training_converges(trained):
    _, _, st, _ = trained
    print("training:", st)
    assert st["mean_err"] < 0.25, st
    assert st["max_err"] < 2.0, st


def test_learned_frame(rnd, port, trained):
    sc, lights, _, blob = trained
    rnd.mlp_load(blob)
    rnd.set_option(abi.OPT_SHADER, abi.SHADER_LEARNED)
    try:
        f, d, ids = rnd.draw_scene(sc, clear=True)
        st = rnd.shade_stats()
    finally:
        rnd.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)
    of, od, oids = oracle_frame(port, sc)
    assert np.array_equal(bits(d), bits(od)), "depth must stay exact"
    assert np.array_equal(ids, oids), "coverage must stay exact"
    cov = oids != 0xFFFFFFFF
    diff = np.abs(f.astype(np.int16) - of.astype(np.int16))
    print("learned frame: max", diff.max(), "mean", diff[:, cov].mean(), "stats", st)
    assert np.all(diff[:, ~cov] == 0)
    assert diff.max() <= RGB_TOL
    assert diff[:, cov].mean() <= MEAN_TOL
    # tiles: 128 consecutive covered pixels (in block order, which is raster order) each
    assert st["tiles"] == (int(cov.sum()) + 127) // 128


def test_wide_network_trains_and_shades(rnd, port, trained):
    """RAST_OPT_MLP_NETWORK 1 trains the 16-frequency network with hidden layers of 64; its frame
    keeps coverage and depth exact and its colour within the same bounds. Weights keep their own
    network: the compact blob loaded afterwards shades as the compact network again."""
    sc, lights, _, blob = trained
    rnd.set_lights(lights)
    assert rnd.get_option(abi.OPT_MLP_NETWORK) == abi.MLP_COMPACT
    rnd.set_option(abi.OPT_MLP_NETWORK, abi.MLP_WIDE)
    try:
        st = rnd.mlp_train(samples=4 << 20, epochs=24, seed=3)
        wide_blob = rnd.mlp_save()
    finally:
        rnd.set_option(abi.OPT_MLP_NETWORK, abi.MLP_COMPACT)
    print("wide training:", st)
    assert st["mean_err"] < 0.25 and st["max_err"] < 2.0, st
    hdr = mlp_ref.parse_blob(wide_blob)
    assert hdr["w1"].shape == (64, 103) and hdr["n_freq"] == 16
    assert len(wide_blob) != len(blob)
    rnd.set_option(abi.OPT_SHADER, abi.SHADER_LEARNED)
    try:
        f, d, ids = rnd.draw_scene(sc, clear=True)
        st = rnd.shade_stats()
    finally:
        rnd.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)
    of, od, oids = oracle_frame(port, sc)
    assert np.array_equal(bits(d), bits(od)) and np.array_equal(ids, oids)
    cov = oids != 0xFFFFFFFF
    diff = np.abs(f.astype(np.int16) - of.astype(np.int16))
    print("wide frame: max", diff.max(), "mean", diff[:, cov].mean(), "stats", st)
    assert diff.max() <= RGB_TOL and diff[:, cov].mean() <= MEAN_TOL
    assert st["tiles"] == (int(cov.sum()) + 127) // 128
    rnd.mlp_load(blob)
    assert rnd.mlp_save() == blob


def test_learned_fallback_gives_exact_colour(rnd, port, trained):
    """With a bound below any error every checked tile falls back: the exact colour everywhere."""
    sc, lights, _, blob = trained
    rnd.mlp_load(blob)
    rnd.set_option(abi.OPT_SHADER, abi.SHADER_LEARNED)
    rnd.set_option(abi.OPT_MLP_BOUND_MILLI, 0)
    rnd.set_option(abi.OPT_MLP_SAMPLES, 4)
    try:
        f, d, ids = rnd.draw_scene(sc, clear=True)
        st = rnd.shade_stats()
    finally:
        rnd.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)
        rnd.set_option(abi.OPT_MLP_BOUND_MILLI, 500)
        rnd.set_option(abi.OPT_MLP_SAMPLES, 2)
    of, _, _ = oracle_frame(port, sc)
    # a tile keeps the MLP colour only where all four checked fragments match to the bit
    fell = st["fallback_tiles"]
    assert fell >= st["tiles"] - 2, st
    diff = np.abs(f.astype(np.int16) - of.astype(np.int16))
    assert diff.max() <= RGB_TOL


@pytest.mark.parametrize("samples", [1, 3, 4])
def test_learned_each_sample_count(rnd, port, trained, samples):
    """Each number of checked records per tile is its own kernel: every tile checks that many
    records, depth and ids stay exact, the colour within tolerance, and tiles fall back exactly
    when a checked error exceeds the bound (max checked error <= 0.5/255 <=> no fallback)."""
    sc, lights, _, blob = trained
    rnd.mlp_load(blob)
    rnd.set_option(abi.OPT_SHADER, abi.SHADER_LEARNED)
    rnd.set_option(abi.OPT_MLP_SAMPLES, samples)
    try:
        f, d, ids = rnd.draw_scene(sc, clear=True)
        st = rnd.shade_stats()
    finally:
        rnd.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)
        rnd.set_option(abi.OPT_MLP_SAMPLES, 2)
    of, od, oids = oracle_frame(port, sc)
    print("samples", samples, "stats", st)
    assert np.array_equal(bits(d), bits(od)) and np.array_equal(ids, oids)
    cov = oids != 0xFFFFFFFF
    diff = np.abs(f.astype(np.int16) - of.astype(np.int16))
    assert diff.max() <= RGB_TOL and diff[:, cov].mean() <= MEAN_TOL
    assert st["checked"] == st["tiles"] * samples
    assert 0.0 < st["max_checked_err"]
    assert (st["max_checked_err"] <= 0.5) == (st["fallback_tiles"] == 0), st


def test_learned_checks_catch_a_wrong_network(rnd, port, trained):
    """The trained network with its output layer scaled by 1.5 is wrong by more than the bound
    wherever a pixel is lit: at the default bound the sampled checks send the tiles to the exact
    shader, and only tiles whose checked records are all (nearly) dark keep the network's colour."""
    sc, lights, _, blob = trained
    w = mlp_ref.parse_blob(blob)
    w["w3"] = mlp_ref.bf16_round(w["w3"] * 1.5)
    rnd.mlp_load(mlp_ref.make_blob(w, n_lights=w["n_lights"], lights_hash=w["lights_hash"], loss=w["loss"]))
    rnd.set_option(abi.OPT_SHADER, abi.SHADER_LEARNED)
    try:
        f, d, ids = rnd.draw_scene(sc, clear=True)
        st = rnd.shade_stats()
    finally:
        rnd.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)
        rnd.mlp_load(blob)
    of, od, oids = oracle_frame(port, sc)
    print("wrong network:", st)
    assert np.array_equal(bits(d), bits(od)) and np.array_equal(ids, oids)
    assert st["max_checked_err"] > 1.0, st
    assert st["fallback_tiles"] >= 0.8 * st["tiles"], st
    cov = oids != 0xFFFFFFFF
    exact = np.all(f == of, axis=0)
    assert exact[cov].mean() >= 0.8


def test_learned_checks_with_lights_beyond_the_shared_table(rnd, port):
    """600 lights: more than the shared check table holds, so the checks read the light records
    from global memory. At a bound of 0 every
    tile whose checked records differ at all falls back: the exact colour; at the default bound the
    verdicts agree with the largest checked error."""
    sc = small_many_lights(600, 320, 240)
    _, _, lights, _ = abi.scene_frame_inputs(sc)
    rnd.upload_scene_mesh(sc)
    rnd.set_lights(lights)
    rnd.mlp_train(samples=1 << 20, epochs=4, seed=5)
    of, od, oids = oracle_frame(port, sc)
    rnd.set_option(abi.OPT_SHADER, abi.SHADER_LEARNED)
    try:
        rnd.set_option(abi.OPT_MLP_BOUND_MILLI, 0)
        f0, _, _ = rnd.draw_scene(sc, clear=True)
        st0 = rnd.shade_stats()
        rnd.set_option(abi.OPT_MLP_BOUND_MILLI, 500)
        f1, d1, ids1 = rnd.draw_scene(sc, clear=True)
        st1 = rnd.shade_stats()
    finally:
        rnd.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)
        rnd.set_option(abi.OPT_MLP_BOUND_MILLI, 500)
    print("600 lights, bound 0:", st0, "bound 0.5:", st1)
    assert st0["fallback_tiles"] >= st0["tiles"] - 2, st0
    assert np.abs(f0.astype(np.int16) - of.astype(np.int16)).max() <= RGB_TOL
    assert np.array_equal(bits(d1), bits(od)) and np.array_equal(ids1, oids)
    assert st1["checked"] == 2 * st1["tiles"] and st1["max_checked_err"] > 0.0
    assert (st1["max_checked_err"] <= 0.5) == (st1["fallback_tiles"] == 0), st1


def test_learned_needs_matching_rig(rnd, trained):
    sc, lights, _, blob = trained
    rnd.mlp_load(blob)
    rnd.upload_scene_mesh(sc)
    other = lights.copy()
    other[0, 3] *= 1.5
    rnd.set_lights(other)
    rnd.set_option(abi.OPT_SHADER, abi.SHADER_LEARNED)
    try:
        cam, nm, _, _ = abi.scene_frame_inputs(sc)
        with pytest.raises(abi.RastError):
            rnd.draw(cam, nm, sc.width, sc.height, abi.CLEAR)
    finally:
        rnd.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)
    hdr = mlp_ref.parse_blob(blob)
    assert hdr["lights_hash"] == mlp_ref.lights_hash(lights)


def _pinned(torch, shape, dtype):
    tdt = {np.uint8: torch.uint8, np.float32: torch.float32, np.uint32: torch.int32}[dtype]
    a = torch.zeros(shape, dtype=tdt).pin_memory().numpy()
    return a.view(np.uint32) if dtype is np.uint32 else a


@pytest.mark.parametrize("clear", [False, True])
def test_deferred_in_place_pinned(rnd, port, clear):
    """Page-locked buffers with the deferred shader: drawn in place, bit for bit the oracle's, and
    after a bin-pool overflow the redraw starts from untouched buffers."""
    torch = pytest.importorskip("torch")
    sc = S.soup(5000, 320, 240, seed=43, area_range=(100.0, 4000.0))
    rng = np.random.default_rng(7)
    frame0 = rng.integers(0, 256, (3, sc.height, sc.width), dtype=np.uint8)
    depth0 = rng.uniform(-1.0, 1.5, (sc.height, sc.width)).astype(np.float32)
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    rnd.upload_scene_mesh(sc)
    rnd.set_lights(lights)
    f = _pinned(torch, (3, sc.height, sc.width), np.uint8)
    d = _pinned(torch, (sc.height, sc.width), np.float32)
    i = _pinned(torch, (sc.height, sc.width), np.uint32)
    f[...] = frame0
    d[...] = depth0
    rnd.set_option(abi.OPT_SHADER, abi.SHADER_EXACT_DEFERRED)
    rnd.set_option(abi.OPT_BIN_CAPACITY, 16)
    try:
        rnd.draw(cam, nm, sc.width, sc.height, abi.CLEAR if clear else 0, f, d, ids=i)
        assert rnd.get_option(abi.OPT_BIN_CAPACITY) > 16
    finally:
        rnd.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)
        rnd.set_option(abi.OPT_BIN_CAPACITY, 0)
    of, od, oids, _ = port.draw(sc, cam, nm, lights, None if clear else frame0, None if clear else depth0)
    assert np.array_equal(bits(d), bits(od))
    assert np.array_equal(i, oids)
    assert np.array_equal(f, of)


def test_learned_in_place_pinned(rnd, trained):
    """The learned shader writes page-locked buffers in place: the same frame as the copy path."""
    torch = pytest.importorskip("torch")
    sc, lights, _, blob = trained
    rnd.mlp_load(blob)
    rnd.set_option(abi.OPT_SHADER, abi.SHADER_LEARNED)
    try:
        f0, d0, i0 = rnd.draw_scene(sc, clear=True)
        cam, nm, l7, _ = abi.scene_frame_inputs(sc)
        f = _pinned(torch, (3, sc.height, sc.width), np.uint8)
        d = _pinned(torch, (sc.height, sc.width), np.float32)
        i = _pinned(torch, (sc.height, sc.width), np.uint32)
        rnd.draw(cam, nm, sc.width, sc.height, abi.CLEAR | (abi.WIND_CLOCKWISE if sc.wind_clockwise else 0),
                 f, d, ids=i)
    finally:
        rnd.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)
    assert np.array_equal(bits(d), bits(d0))
    assert np.array_equal(i, i0)
    assert np.array_equal(f, f0)


def test_learned_shader_wait_timeout_recovers(rnd, trained):
    """The bounded tensor-core waits: with the test-only stall option the first MMA wait of every
    CTA gives up (it polls an mbarrier nothing arrives on). Each CTA then waits for its MMA in
    flight with the full bound, frees its tensor memory and returns; the draw reports
    RAST_ERR_TIMEOUT, and the context draws the same frame as before once the option is off."""
    sc, lights, _, blob = trained
    rnd.mlp_load(blob)
    rnd.set_option(abi.OPT_SHADER, abi.SHADER_LEARNED)
    try:
        f0, d0, i0 = rnd.draw_scene(sc, clear=True)
        rnd.set_option(abi.OPT_TEST_SHADE_STALL, 1)
        with pytest.raises(abi.RastError) as err:
            rnd.draw_scene(sc, clear=True)
        assert err.value.status == 7, str(err.value)  # RAST_ERR_TIMEOUT
        rnd.set_option(abi.OPT_TEST_SHADE_STALL, 0)
        for _ in range(2):
            f, d, i = rnd.draw_scene(sc, clear=True)
            assert np.array_equal(bits(d), bits(d0))
            assert np.array_equal(i, i0)
            assert np.array_equal(f, f0)
    finally:
        rnd.set_option(abi.OPT_TEST_SHADE_STALL, 0)
        rnd.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)


def test_time_shading_replays_the_same_pass(rnd, port):
    """rast_time_shading re-runs the last draw's deferred shading pass: positive times, and the
    frame it rewrites is the same; after an exact (fused) draw there is no pass to time."""
    torch = pytest.importorskip("torch")
    sc = small_many_lights(32)
    cam, nm, lights, _ = abi.scene_frame_inputs(sc)
    rnd.upload_scene_mesh(sc)
    rnd.set_lights(lights)
    W, H = sc.width, sc.height
    rgb = torch.empty(3 * W * H, dtype=torch.uint8, device="cuda")
    dep = torch.empty(W * H, dtype=torch.float32, device="cuda")
    rnd.set_option(abi.OPT_SHADER, abi.SHADER_EXACT_DEFERRED)
    try:
        rnd.draw_device(cam, nm, W, H, abi.CLEAR, rgb.data_ptr(), dep.data_ptr())
        rnd.sync()
        first = rgb.cpu().numpy().copy()
        us = rnd.time_shading(5)
        assert us > 0.0
        assert np.array_equal(rgb.cpu().numpy(), first)
        of, _, _, _ = port.draw(sc, cam, nm, lights)
        assert np.array_equal(first.reshape(3, H, W), of)
    finally:
        rnd.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)
    rnd.draw_device(cam, nm, W, H, abi.CLEAR, rgb.data_ptr(), dep.data_ptr())
    rnd.sync()
    with pytest.raises(abi.RastError):
        rnd.time_shading(1)
