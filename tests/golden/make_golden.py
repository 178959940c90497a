"""Generates the golden fixtures in this directory from canmom/rasteriser's own draw_frame,
compiled from the reference sources (oracle/Makefile ``ref`` -> oracle/_ref/libref.so).

Small scenes are stored whole (inputs, matrices, transformed lights, reference frame and depth
buffers) in ``<name>.npz``. The full-size workloads are stored as digests in ``full_size.json``:
the SHA-256 of the generated inputs and of the reference's depth and RGB outputs, with the
matrices used, so a machine without the reference can still check a full 1920x1080 or 3840x2160
frame against it.

Run from the repository root on a machine that has the reference tree:
    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from rasteriser_gb300 import scenes as S  # noqa: E402
import edge_scenes as E  # noqa: E402


def small_scenes():
    out = [S.square_scene(), S.plane_scene(),
           S.config_icosphere_small(),
           S.config_icosphere_small().with_view(name="icosphere4_cw", wind_clockwise=True),
           S.config_displaced_sphere(128, 64, 480, 270).with_view(name="uvsphere_small_tf", angles=(0.3, 1.1, 0.2),
                                                                 scale=1.3, disp=(0.1, -0.2, 0.3)),
           S.soup(20000, 640, 360, seed=5).with_view(name="soup20k"),
           S.soup(3000, 200, 120, seed=7, area_range=(50.0, 5000.0)).with_view(name="soup_big_tris")]
    out += E.all_edge_scenes()
    names = set()
    for sc in out:
        if sc.name in names:
            sc.name = sc.name + ("_cw" if sc.wind_clockwise else "_ccw")
        names.add(sc.name)
    return out


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def main():
    oracle.build(with_reference=True)
    ref = oracle.Reference()
    for sc in small_scenes():
        fr, dr, td = ref.draw(sc)
        m = ref.matrices(sc)
        np.savez_compressed(os.path.join(HERE, sc.name + ".npz"), pos=sc.pos, tris=sc.tris, nrm=sc.nrm, uv=sc.uv,
                            kd=sc.kd, lights=sc.lights, lights7=oracle.lights_with_dirs(sc, td),
                            camera=m["camera"], normal=m["normal"], view=m["view"],
                            width=sc.width, height=sc.height, cw=int(sc.wind_clockwise),
                            params=np.array([sc.scale, *sc.disp, *sc.angles, sc.fovy_deg, sc.z_near, sc.z_far],
                                            np.float32),
                            frame=fr, depth=dr)
        print("wrote", sc.name, sc.ntri, "tris")

    full = {}
    sphere = S.config_displaced_sphere()
    for f in (0, 30, 59):
        sc = sphere.with_view(angles=S.spin_angles(f))
        fr, dr, td = ref.draw(sc)
        m = ref.matrices(sc)
        full[f"displaced_sphere_frame{f}"] = dict(
            generator="config_displaced_sphere", frame=f, mesh=sc.mesh_digest(), width=sc.width, height=sc.height,
            camera=m["camera"].tolist(), normal=m["normal"].tolist(),
            lights7=oracle.lights_with_dirs(sc, td).tolist(), depth=digest(dr), frame_rgb=digest(fr),
            covered=int((fr.reshape(3, -1).max(axis=0) > 0).sum()))
        print("full", f)
    soup = S.config_soup()
    fr, dr, td = ref.draw(soup)
    m = ref.matrices(soup)
    full["soup_4m_4k"] = dict(generator="config_soup", frame=0, mesh=soup.mesh_digest(), width=soup.width,
                              height=soup.height, camera=m["camera"].tolist(), normal=m["normal"].tolist(),
                              lights7=oracle.lights_with_dirs(soup, td).tolist(), depth=digest(dr),
                              frame_rgb=digest(fr))
    with open(os.path.join(HERE, "full_size.json"), "w") as fh:
        json.dump(full, fh, indent=1)
    print("wrote full_size.json")


if __name__ == "__main__":
    main()
