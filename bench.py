#!/usr/bin/env python
"""Benchmark of the rasteriser hot path (draw_frame) on GB300.

Workload (default): the displaced UV sphere, 1024x512 segments (523,266 vertices, 1,046,528
triangles, flat per-face normals), 1920x1080, 3 directional lights, spun about y by 1/60 rad per
frame (the reference's spin loop at 60 frames/s). A step is one frame: the spin loop's clear plus
draw_frame, on device-resident buffers, with L2 flushed (a 256 MiB write) between steps outside
the timed region.

One JSON line on rank 0: value = frames/s over all ranks; e2e = the same through the C ABI with
host buffers (rast_draw, read-modify-write as draw_frame, mesh resident) on page-locked buffers,
which the exact shader's kernels read and write in place over the link; e2e_pageable = the same on
ordinary pageable numpy arrays, used in place too where the device translates host addresses (Grace),
else copied host->device and back; roofline of the dominant kernel from
per-stage CUDA events; the CPU baseline (the oracle port, one core) on a bounded sample of the same
frames.

--impl reference times the reference's CPU path on the host cores instead (the oracle port, one
frame per thread on all cores; the reference's own sources are not present on the GPU host).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "frames/s @1080p 1M-tri (1 GB300); shade px/s learned vs plain @≤1/255 err"
FLUSH_BYTES = 256 << 20
SPIN_FRAMES = 60


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["displaced_sphere", "soup", "soup_1m", "icosphere", "many_lights"],
                    default="displaced_sphere")
    ap.add_argument("--shader", choices=["exact", "deferred", "learned"], default="exact",
                    help="shading mode (learned: the MLP is trained on 4M samples first)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU-baseline sample")
    ap.add_argument("--device-only", action="store_true", help="only the device-resident timed loop (profiling)")
    ap.add_argument("--no-soak", action="store_true", help="skip the clock-sampling soak loop (profiling)")
    ap.add_argument("--small-max", type=int, default=None)
    ap.add_argument("--tile", type=int, default=None)
    ap.add_argument("--row-chunk", type=int, default=None)
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the extra workloads (4M-triangle soup, 256-frame batch) reported beside the line")
    return ap.parse_args()


def make_scene(name):
    from rasteriser_gb300 import scenes as S
    if name == "displaced_sphere":
        return S.config_displaced_sphere(), "displaced_sphere_1024x512_1080p_spin60"
    if name == "soup":
        return S.config_soup(), "triangle_soup_4M_2160p"
    if name == "soup_1m":  # a cropped soup for profiling: 1M triangles at 1920x1080
        return S.config_soup(1_000_000, 1920, 1080), "triangle_soup_1M_1080p"
    if name == "many_lights":
        return S.config_many_lights(), "displaced_sphere_1M_1080p_256_lights"
    return S.config_icosphere_small(), "icosphere_l4_480p"


def rank_frame(rank, world, k, n_frames):
    """The spin frame that rank `rank` of `world` draws at its step k: the ranks take consecutive
    frames of the spin (replicas, no exchange between them)."""
    return (rank + k * world) % n_frames


def max_over_ranks(dist, seconds, device):
    """The slowest rank's time (the job's time), or the time itself without a process group."""
    if dist is None:
        return seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def frame_inputs(scene, n_frames, source=None):
    """(scene, camera, normal matrix, transformed lights) of each spin frame. The matrices and
    lights come from librast's host code, or from `source.frame_inputs` (the oracle port, for the
    reference arm, which loads nothing of this package's native code)."""
    from rasteriser_gb300 import scenes as S
    if source is None:
        from rasteriser_gb300 import abi
        source_fn = abi.scene_frame_inputs
    else:
        source_fn = source.frame_inputs
    out = []
    for f in range(n_frames):
        sc = scene.with_view(angles=S.spin_angles(f))
        cam, nm, lights, _ = source_fn(sc)
        out.append((sc, cam, nm, lights))
    return out


def workload_config(scene, workload, n_frames, n_lights, world, shader):
    """The `config` object of both arms' lines: the workload, its sizes and the draw mode."""
    return {"workload": workload, "width": scene.width, "height": scene.height, "triangles": scene.ntri,
            "vertices": int(scene.pos.shape[0]), "lights": int(n_lights), "frames_cycled": n_frames,
            "l2": "GPU arm: flushed between steps (256 MiB write, outside the timed events)",
            "parallelism": f"replicas x{world}", "mode": "RAST_CLEAR (spin-loop clear + draw_frame)",
            "shader": shader}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()
        return False

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        rows = [r.split(", ") for r in self.out.strip().splitlines() if r.count(",") >= 8]
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes(stage, sc, st):
    """Compulsory bytes each stage must move for one frame (inputs read once, outputs written once)."""
    W, H = sc.width, sc.height
    npx = W * H
    nv, ntri = sc.pos.shape[0], sc.ntri
    if stage == "vertex":
        return 12 * nv + 16 * nv
    if stage == "setup_raster":
        # indices + three gathered raster vertices per triangle, an 8-byte atomic per inside fragment
        # of the per-triangle path, a 64-byte record per binned triangle
        small_frags = max(0, st["inside"] - st.get("tile_inside", 0))
        return 12 * ntri + 48 * ntri + 8 * small_frags + 64 * st["binned_tris"]
    if stage == "bin_scan":
        tiles = -(-W // 16) * -(-H // 16)
        return 8 * tiles
    if stage == "bin_scatter":
        return 64 * st["binned_tris"] + 4 * st["bin_entries"]
    if stage == "tile_raster":
        return 68 * st["bin_entries"] + 16 * npx
    if stage == "shade":
        # the deferred pass: one 32-byte record read and an RGB8 pixel written per covered pixel
        return (32 + 3) * st["written"]
    if stage == "resolve":
        # key read + re-arm, planar RGB8 + depth written, and per covered pixel the winner's indices,
        # vertices, normal indices and normals
        return (8 + 8 + 3 + 4) * npx + st["written"] * (12 + 48 + 16 + 36)
    return 0


def load_traffic(kernel, workload):
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as fh:
        d = json.load(fh)
    e = d.get(workload, {}).get(kernel)
    return None if e is None else float(e["dram_bytes_per_launch"])


def oracle_port():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    return oracle.Port()


def cpu_baseline(frames, seconds, threads=1):
    """The oracle port (C restatement of the reference's draw_frame) on the host cores."""
    port = oracle_port()
    done = []
    lock = threading.Lock()
    t0 = time.perf_counter()
    stop = t0 + seconds

    def worker(k):
        i = k
        while time.perf_counter() < stop:
            sc, cam, nm, lights = frames[i % len(frames)]
            port.draw(sc, cam, nm, lights, want_ids=False)
            with lock:
                done.append(i)
            i += threads

    ts = [threading.Thread(target=worker, args=(k,)) for k in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    dt = time.perf_counter() - t0
    return len(done) / dt, len(done), dt


def parallel_steps(frames, steps, threads, first=0):
    """`steps` rounds; in each, `threads` threads render one frame each of the spin (the port
    releases the GIL inside its C call). Returns the wall seconds of all rounds."""
    port = oracle_port()

    def render(i):
        sc, cam, nm, lights = frames[i % len(frames)]
        port.draw(sc, cam, nm, lights, want_ids=False)

    t0 = time.perf_counter()
    for s in range(steps):
        ts = [threading.Thread(target=render, args=(first + s * threads + k,)) for k in range(threads)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
    return time.perf_counter() - t0


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    scene, workload = make_scene(args.workload)
    n_frames = SPIN_FRAMES if args.workload == "displaced_sphere" else 1
    # matrices and lights from the oracle port's restatement of drawing.cpp:221-238
    frames = frame_inputs(scene, n_frames, source=oracle_port())
    world = int(os.environ.get("WORLD_SIZE", "1"))
    threads = os.cpu_count() or 1
    warm = parallel_steps(frames, max(1, min(args.warmup, 2)), threads)
    per_step = warm / max(1, min(args.warmup, 2))
    # bounded sample: at most ~90 s of timed work whatever --steps asks for
    steps = max(1, min(args.steps, int(90.0 / max(per_step, 1e-3))))
    dt = parallel_steps(frames, steps, threads, first=threads)
    value = steps * threads / dt
    line = {"metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": args.gpus, "steps": steps,
            "steps_requested": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dt / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": workload_config(scene, workload, n_frames, frames[0][3].shape[0], world, args.shader),
            "cpu_baseline": {"value": value, "unit": "frames/s", "cores": threads, "kind": "port",
                             "sample": f"{steps} steps x {threads} threads, one full frame of the 60-frame spin per "
                                       f"thread per step, {dt:.1f} s"},
            "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def time_scene_device(torch, abi, r, stream, frames_in, steps, warmup, flush):
    """Device-resident loop over one scene's frames (clear + draw), L2 flushed between frames, each
    frame timed with CUDA events on the draw's stream. Returns (frames/s, stats, stage ms)."""
    sc0 = frames_in[0][0]
    W, H = sc0.width, sc0.height
    r.upload_scene_mesh(sc0)
    r.set_lights(frames_in[0][3])
    d_rgb = torch.empty(3 * W * H, dtype=torch.uint8, device="cuda")
    d_depth = torch.empty(W * H, dtype=torch.float32, device="cuda")

    def step(k):
        _, cam, nm, _ = frames_in[k % len(frames_in)]
        r.draw_device(cam, nm, W, H, abi.CLEAR, d_rgb.data_ptr(), d_depth.data_ptr())

    for k in range(warmup):
        step(k)
        flush.zero_()
    r.sync()
    stats = r.stats()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for k in range(steps):
        ev[k][0].record(stream)
        step(k)
        ev[k][1].record(stream)
        flush.zero_()
    r.sync()
    total = sum(a.elapsed_time(b) for a, b in ev) / 1000.0
    r.set_option(abi.OPT_STAGE_TIMING, 1)
    acc = {}
    for k in range(min(steps, 20)):
        step(k)
        r.sync()
        for name, ms in r.stage_times().items():
            acc[name] = acc.get(name, 0.0) + ms
        flush.zero_()
    r.set_option(abi.OPT_STAGE_TIMING, 0)
    n = min(steps, 20)
    return steps / total, stats, {k: v / n for k, v in acc.items()}


def extra_soup(torch, abi, stream, flush, steps=30):
    """The 4M-triangle soup at 3840x2160 (one frame drawn repeatedly)."""
    from rasteriser_gb300 import scenes as S
    sc = S.config_soup()
    fr = frame_inputs(sc, 1)
    r = abi.Renderer(0)
    r.set_stream(stream.cuda_stream)
    try:
        fps, st, stage = time_scene_device(torch, abi, r, stream, fr, steps, 3, flush)
    finally:
        r.close()
    # the dominant pass (setup, which also performs the depth test's 64-bit atomicMins): HBM
    # roofline of its algorithmic bytes, its DRAM traffic scaled from the 1M-triangle 1080p capture
    # (a quarter of the triangles and of the pixels), and the atomic rate
    peak, peak_kind = peaks()
    alg = algorithmic_bytes("setup_raster", sc, st)
    achieved = alg / (stage["setup_raster"] / 1000.0) / 1e9
    small = load_traffic("k_setup_raster", "triangle_soup_1M_1080p")
    return {"workload": "triangle_soup_4M_2160p", "frames_per_s": fps, "fragments_per_s": st["inside"] * fps,
            "ms_per_frame": 1000.0 / fps, "stage_ms": stage,
            "roofline": {"kernel": "k_setup_raster", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "algorithmic_bytes_per_launch": alg,
                         "traffic": None if small is None else 4.0 * small,
                         "traffic_note": "4 x the DRAM bytes of the 1M-triangle 1920x1080 capture"},
            "depth_atomics_per_s": st["inside"] / (stage["setup_raster"] / 1000.0),
            "frame_stats": {k: st[k] for k in ("front", "tested", "inside", "written", "binned_tris", "bin_entries")}}


def bf16_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            return float(json.load(fh)["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


def extra_many_lights(torch, abi, stream, flush, steps=30):
    """The 1M-triangle displaced sphere with smooth normals and per-vertex albedo at
    1920x1080 under 256 lights. The plain per-light shader (deferred exact; fused exact beside it)
    against the learned shader, which is trained here on 4M samples the exact shader labels: the
    compact network (the default) and the wide one the workload's description names."""
    from rasteriser_gb300 import scenes as S
    sc = S.config_many_lights()
    fr = frame_inputs(sc, 1)
    _, cam, nm, lights = fr[0]
    W, H = sc.width, sc.height
    r = abi.Renderer(0)
    r.set_stream(stream.cuda_stream)
    out = {"workload": "displaced_sphere_1M_1080p_256_lights", "lights": int(lights.shape[0])}
    try:
        r.upload_scene_mesh(sc)
        r.set_lights(lights)
        t0 = time.perf_counter()
        out["training"] = r.mlp_train(samples=4 << 20, epochs=24, seed=3)
        out["training"]["wall_s"] = time.perf_counter() - t0
        out["training"]["samples"] = 4 << 20
        # the networks measured here: the compact default, and the wide one the workload's
        # description names (the compact one was chosen for about equal held-out error)
        out["network"] = {
            "learned": {"features": "3 Fourier frequencies per normal component, normal, albedo, 1 (25)",
                        "layers": "25 -> 32 -> 32 -> 3", "dtype": "bf16 weights, fp32 accumulation"},
            "learned_wide": {"features": "16 Fourier frequencies per normal component, normal, albedo, 1 (103)",
                             "layers": "103 -> 64 -> 64 -> 3", "dtype": "bf16 weights, fp32 accumulation"},
            "named_in_workload": "16 Fourier frequencies, 64 -> 64 -> 3"}
        dims = {abi.MLP_COMPACT: (25, 32, 32), abi.MLP_WIDE: (103, 112, 64)}  # features, K, hidden
        frames, modes = {}, {}
        net_now = abi.MLP_COMPACT
        for name, shader, samples, net in (("exact_fused", abi.SHADER_EXACT, 2, abi.MLP_COMPACT),
                                           ("exact_deferred", abi.SHADER_EXACT_DEFERRED, 2, abi.MLP_COMPACT),
                                           ("learned", abi.SHADER_LEARNED, 2, abi.MLP_COMPACT),
                                           ("learned_unchecked", abi.SHADER_LEARNED, 0, abi.MLP_COMPACT),
                                           ("learned_wide", abi.SHADER_LEARNED, 2, abi.MLP_WIDE),
                                           ("learned_wide_unchecked", abi.SHADER_LEARNED, 0, abi.MLP_WIDE)):
            if net != net_now:
                r.set_option(abi.OPT_MLP_NETWORK, net)
                t0 = time.perf_counter()
                out["training_wide"] = r.mlp_train(samples=4 << 20, epochs=24, seed=3)
                out["training_wide"]["wall_s"] = time.perf_counter() - t0
                net_now = net
            r.set_option(abi.OPT_SHADER, shader)
            r.set_option(abi.OPT_MLP_SAMPLES, samples)
            fps, st, stage = time_scene_device(torch, abi, r, stream, fr, steps, 3, flush)
            shade_ms = stage["resolve"] if shader == abi.SHADER_EXACT else stage["shade"]
            m = {"frames_per_s": fps, "shade_ms_stage_events": shade_ms, "stage_ms": stage}
            if shader != abi.SHADER_EXACT:
                # the shading pass alone: the same pass (same records and tiles) run back to back
                # 200 times, so each kernel's time excludes the launch gap that events between a
                # frame's unchained kernels add (several microseconds, for any kernel)
                d_rgb = torch.empty(3 * W * H, dtype=torch.uint8, device="cuda")
                d_dep = torch.empty(W * H, dtype=torch.float32, device="cuda")
                r.draw_device(cam, nm, W, H, abi.CLEAR, d_rgb.data_ptr(), d_dep.data_ptr())
                r.sync()
                shade_ms = r.time_shading(200) / 1000.0
            m["shade_ms"] = shade_ms
            f, _, ids = r.draw(cam, nm, W, H, abi.CLEAR, want_ids=True)
            if shader == abi.SHADER_LEARNED:
                m["checks"] = r.shade_stats()  # of this one draw
                m["check_samples_per_tile"] = samples
                m["network"] = net
            frames[name] = (f, ids)
            modes[name] = m
        r.set_option(abi.OPT_SHADER, abi.SHADER_EXACT)
        r.set_option(abi.OPT_MLP_NETWORK, abi.MLP_COMPACT)
        ref, ids = frames["exact_fused"]
        cov = ids != abi.NO_TRIANGLE
        covered = int(cov.sum())
        peak, peak_kind = bf16_peak()
        for name, m in modes.items():
            f, fid = frames[name]
            d = np.abs(f.astype(np.int16) - ref.astype(np.int16))
            m["shade_px_per_s"] = covered / (m["shade_ms"] * 1e-3)
            m["err_vs_exact"] = {"mean": float(d[:, cov].mean()), "max": int(d.max()),
                                 "coverage_identical": bool(np.array_equal(fid, ids))}
            if name.startswith("learned"):
                ck = m["checks"]
                m["fallback_tile_fraction"] = ck["fallback_tiles"] / max(ck["tiles"], 1)
                # algorithmic tensor work: 2 * (F*H + H*H + H*3) FLOP per shaded pixel (F features
                # in use, two hidden layers of H, 3 outputs); executed: K padded to a multiple of
                # 16, N of the last layer 16
                nf, nk, nh = dims[m["network"]]
                alg = covered * 2.0 * (nf * nh + nh * nh + nh * 3)
                executed = ck["tiles"] * 128 * 2.0 * (nk * nh + nh * nh + nh * 16)
                tflops = alg / (m["shade_ms"] * 1e-3) / 1e12
                m["tensor"] = {"algorithmic_flop": alg, "executed_flop": executed, "achieved_tflops": tflops,
                               "peak_tflops": peak, "frac": tflops / peak, "peak_source": peak_kind}
        plain = modes["exact_deferred"]["shade_ms"]
        out["covered_px"] = covered
        out["modes"] = modes
        # the shading passes timed alone (back to back); the stage-event ratio beside it
        out["speedup_learned_vs_plain"] = plain / modes["learned"]["shade_ms"]
        out["speedup_learned_unchecked_vs_plain"] = plain / modes["learned_unchecked"]["shade_ms"]
        out["speedup_stage_events"] = (modes["exact_deferred"]["shade_ms_stage_events"] /
                                       modes["learned"]["shade_ms_stage_events"])
        out["speedup_learned_wide_vs_plain"] = plain / modes["learned_wide"]["shade_ms"]
        out["speedup_learned_wide_unchecked_vs_plain"] = plain / modes["learned_wide_unchecked"]["shade_ms"]
    finally:
        r.close()
    return out


def extra_batch(torch, abi, stream, steps=10):
    """The 256-frame batch as one CUDA graph over 8 lanes after autotuning, against the
    same frames drawn one after another on one stream."""
    from rasteriser_gb300 import scenes as S
    meshes, frames = S.batch_workload()
    r = abi.Renderer(0)
    r.set_stream(stream.cuda_stream)
    keep = []
    try:
        ids = [r.add_mesh(m.pos, m.nrm, m.uv, m.tris, m.kd) for m in meshes]
        descs = []
        for fr in frames:
            mi, W, H = fr[0], fr[1], fr[2]
            sc = S.batch_frame_scene(meshes, fr)
            cam, nm, l7, _ = abi.scene_frame_inputs(sc)
            d = (torch.from_numpy(l7).cuda(), torch.empty(3 * W * H, dtype=torch.uint8, device="cuda"),
                 torch.empty(W * H, dtype=torch.float32, device="cuda"))
            keep.append(d)
            descs.append(r.frame_desc(ids[mi], W, H, abi.CLEAR, cam, nm, d[0].data_ptr(), l7.shape[0],
                                      d[1].data_ptr(), d[2].data_ptr()))
        tuned = r.autotune(descs, lanes=8, repeats=2)

        def timed(lanes, graph):
            r.draw_batch(descs, lanes=lanes, graph=graph)
            r.sync()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(steps):
                r.draw_batch(descs, lanes=lanes, graph=graph)
            b.record(stream)
            r.sync()
            return a.elapsed_time(b) / 1000.0 / steps

        t_graph = timed(8, True)
        st = r.batch_stats(len(descs))
        t_serial = timed(1, False)
        # where the time goes: each frame alone on the stream (tuned options), by mesh kind and size
        per_frame = []
        for d in descs:
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            r.draw_batch([d], lanes=1, graph=False)
            b.record(stream)
            per_frame.append((a, b))
        r.sync()
        frame_ms = [a.elapsed_time(b) for a, b in per_frame]
        # the same two forms with the untuned defaults (tile 16, small-box limit 4096, whole rows,
        # 256 threads per tile): how much of the gain is the lanes' overlap and how much the tuning
        for opt, v in ((abi.OPT_TILE_SIZE, 16), (abi.OPT_SMALL_MAX_PIXELS, 4096), (abi.OPT_ROW_CHUNK, 32),
                       (abi.OPT_TILE_THREADS, 0)):
            r.set_option(opt, v)
        t_graph_default = timed(8, True)
        t_serial_default = timed(1, False)
    finally:
        r.close()
    n = len(descs)
    frags = int(st[:, 2].sum())
    classes = {}
    for fr, ms, row in zip(frames, frame_ms, st):
        kind = f"icosphere_L{fr[0] + 2}" if fr[0] < 6 else "soup"
        key = f"{kind} {fr[1]}x{fr[2]}"
        c = classes.setdefault(key, {"frames": 0, "ms": 0.0, "fragments": 0})
        c["frames"] += 1
        c["ms"] += ms
        c["fragments"] += int(row[2])
    return {"workload": "batch_256_frames_uneven", "frames": n, "meshes": len(meshes),
            "triangles_per_batch": int(sum(meshes[f[0]].ntri for f in frames)),
            "autotuned": tuned, "lanes": 8,
            "graph_frames_per_s": n / t_graph, "graph_fragments_per_s": frags / t_graph,
            "serial_frames_per_s": n / t_serial, "speedup_vs_frame_by_frame": t_serial / t_graph,
            "ms_per_batch_graph": 1000 * t_graph, "ms_per_batch_serial": 1000 * t_serial,
            "untuned": {"ms_per_batch_graph": 1000 * t_graph_default, "ms_per_batch_serial": 1000 * t_serial_default},
            "sum_of_frames_alone_ms": sum(frame_ms),
            "by_class": dict(sorted(classes.items(), key=lambda kv: -kv[1]["ms"])),
            "l2": "not flushed (the batch's working set exceeds L2)"}


def e2e_line(value, shader, W, H, stats, memory="page-locked", in_place=True):
    """The e2e entry for host buffers. Used in place, the resolve pass reads the incoming depth of
    each pixel a fragment landed on and writes the winners' colour (3 B) and depth (4 B), plus the
    4-byte status word; deferred shading writes the colour once more. Copied, the whole frame and
    depth cross the link both ways."""
    if not in_place:
        return {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 7 * W * H,
                "d2h_bytes_per_step": 7 * W * H + 4,
                "path": f"rast_draw with {memory} host frame (planar RGB8) and depth buffers, copied both ways "
                        "(read-modify-write); mesh resident"}
    covered = int(stats["written"])
    colour = 3 * covered if shader != "exact" else 0
    return {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 4 * covered,
            "d2h_bytes_per_step": 7 * covered + colour + 4,
            "path": f"rast_draw with {memory} host frame (planar RGB8) and depth buffers used in place "
                    "(read-modify-write; the kernels read the incoming depth of covered pixels and write "
                    "their colour and depth over the link); mesh resident"}


def run_ours(args):
    import torch
    from rasteriser_gb300 import abi

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    scene, workload = make_scene(args.workload)
    n_frames = SPIN_FRAMES if args.workload == "displaced_sphere" else 1
    frames = frame_inputs(scene, n_frames)
    W, H = scene.width, scene.height

    r = abi.Renderer(local)
    # A created stream: librast and the timing events, L2 flushes and copies all run on it, in order.
    # (Handle 0, torch's default stream, would select librast's own stream instead.)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    r.set_stream(stream.cuda_stream)
    if args.small_max:
        r.set_option(abi.OPT_SMALL_MAX_PIXELS, args.small_max)
    if args.tile:
        r.set_option(abi.OPT_TILE_SIZE, args.tile)
    if args.row_chunk:
        r.set_option(abi.OPT_ROW_CHUNK, args.row_chunk)
    r.upload_scene_mesh(scene)
    r.set_lights(frames[0][3])  # the view is a fixed translation: the lights are the same each frame
    training = None
    if args.shader == "learned":
        training = r.mlp_train(samples=4 << 20, epochs=24, seed=3)
    r.set_option(abi.OPT_SHADER, {"exact": abi.SHADER_EXACT, "deferred": abi.SHADER_EXACT_DEFERRED,
                                  "learned": abi.SHADER_LEARNED}[args.shader])
    d_rgb = torch.empty(3 * W * H, dtype=torch.uint8, device="cuda")
    d_depth = torch.empty(W * H, dtype=torch.float32, device="cuda")
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def frame_of(k):
        return frames[rank_frame(rank, world, k, n_frames)]

    def step(k):
        _, cam, nm, _ = frame_of(k)
        r.draw_device(cam, nm, W, H, abi.CLEAR, d_rgb.data_ptr(), d_depth.data_ptr())

    for k in range(args.warmup):
        step(k)
        flush.zero_()
    r.sync()
    stats = r.stats()

    # timed region: K steps, each bracketed by events; L2 flushed between steps, outside the events
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(local)
    with sampler:
        # keep the GPU busy for >= 0.5 s so the 100 ms clock samples see the load
        t_soak = time.perf_counter()
        while not args.no_soak and time.perf_counter() - t_soak < 0.5:
            step(0)
            flush.zero_()
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        wall0 = time.perf_counter()
        for k in range(args.steps):
            starts[k].record(stream)
            step(k)
            ends[k].record(stream)
            flush.zero_()
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    r.sync()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_s = max_over_ranks(dist, sum(step_ms) / 1000.0, "cuda")
    value = world * args.steps / total_s
    launches_per_step = stats["launches"]

    if args.device_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "frames/s", "steps": args.steps,
                              "ms_per_step": 1000 * total_s / args.steps, "device_only": True}))
        return

    # per-stage device times (CUDA events recorded by librast between its kernels)
    r.set_option(abi.OPT_STAGE_TIMING, 1)
    n_st = min(args.steps, 200)
    acc = {}
    for k in range(n_st):
        step(k)
        r.sync()
        for name, ms in r.stage_times().items():
            acc[name] = acc.get(name, 0.0) + ms
        flush.zero_()
    r.set_option(abi.OPT_STAGE_TIMING, 0)
    stage_ms = {k: v / n_st for k, v in acc.items()}

    # End to end through the C ABI with host buffers (read-modify-write, as draw_frame), mesh
    # resident. Page-locked buffers are used in place (the kernels read and write them over the
    # link); ordinary pageable arrays too where the device translates host addresses, else they
    # are copied both ways. Both are timed; the draw's statistics say which path ran.
    def e2e_run(pinned):
        if pinned:
            h_rgb = torch.zeros(3 * W * H, dtype=torch.uint8).pin_memory().numpy().reshape(3, H, W)
            h_depth = torch.ones(W * H, dtype=torch.float32).pin_memory().numpy().reshape(H, W)
        else:
            h_rgb = np.zeros((3, H, W), np.uint8)
            h_depth = np.ones((H, W), np.float32)
        n_e2e = min(args.steps, 500)
        e2e_s = 0.0
        for k in range(n_e2e + 3):
            h_rgb[...] = 0
            h_depth[...] = 1.0
            flush.zero_()
            torch.cuda.synchronize()
            _, cam, nm, _ = frame_of(k)
            t0 = time.perf_counter()
            r.draw(cam, nm, W, H, 0, h_rgb, h_depth)
            if k >= 3:
                e2e_s += time.perf_counter() - t0
        return world * n_e2e / max_over_ranks(dist, e2e_s, "cuda"), r.stats()["host_in_place"] == 1

    e2e_value, e2e_in_place = e2e_run(True)
    e2e_pageable, pageable_in_place = e2e_run(False)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    # roofline of the dominant kernel
    peak, peak_kind = peaks()
    stage_names = ["vertex", "setup_raster", "bin_scan", "bin_scatter", "tile_raster", "resolve"]
    if args.shader != "exact":
        stage_names.append("shade")
    dom = max(stage_names, key=lambda s: stage_ms.get(s, 0.0))
    sc0 = frames[0][0]
    alg = algorithmic_bytes(dom, sc0, stats)
    achieved = alg / (stage_ms[dom] / 1000.0) / 1e9
    kernel_names = {"vertex": "k_vertex", "setup_raster": "k_setup_raster", "bin_scan": "k_bin_scan",
                    "bin_scatter": "k_bin_scatter", "tile_raster": "k_tile_raster", "resolve": "k_resolve",
                    "shade": "k_shade_mlp" if args.shader == "learned" else "k_shade_exact"}
    traffic = load_traffic(kernel_names[dom], workload)

    cpu = None
    if world == 1 or rank == 0:
        v, n, dt = cpu_baseline(frames, args.cpu_seconds, 1)
        cpu = {"value": v, "unit": "frames/s", "cores": 1, "kind": "port",
               "sample": f"{n} frames of the same spin ({W}x{H}, {scene.ntri} triangles) in {dt:.1f} s, one thread"}

    clocks = sampler.summary()
    line = {
        "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * total_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(scene, workload, n_frames, frames[0][3].shape[0], world, args.shader),
        "e2e": e2e_line(e2e_value, args.shader, W, H, stats, in_place=e2e_in_place),
        "e2e_pageable": e2e_line(e2e_pageable, args.shader, W, H, stats, "pageable numpy", pageable_in_place),
        "gpu_launches": launches_per_step * args.steps,
        "roofline": {"kernel": kernel_names[dom], "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": alg, "launch_ms": stage_ms[dom]},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "wall_s_timed_loop": wall,
        "stage_ms": stage_ms,
        "frame_stats": {k: stats[k] for k in ("front", "tested", "inside", "written", "binned_tris", "bin_entries")},
        "fragments_per_s": stats["inside"] * value,
    }
    if training is not None:
        line["training"] = training
        line["shade_checks"] = r.shade_stats()
    if not args.no_extras and world == 1 and args.workload == "displaced_sphere":
        line["extras"] = {"soup": extra_soup(torch, abi, stream, flush), "batch": extra_batch(torch, abi, stream),
                          "many_lights": extra_many_lights(torch, abi, stream, flush)}
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
