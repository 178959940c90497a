"""Loading of the golden fixtures written by tests/golden/make_golden.py."""
import glob
import json
import os

import numpy as np

from rasteriser_gb300 import scenes as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    """(scene, inputs) where inputs holds camera, normal, lights7 and the reference's frame/depth."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    prm = z["params"]
    sc = S.Scene(name, z["pos"], z["tris"], z["nrm"], z["uv"], z["kd"], z["lights"], width=int(z["width"]),
                 height=int(z["height"]), wind_clockwise=bool(z["cw"]), scale=float(prm[0]),
                 disp=tuple(float(v) for v in prm[1:4]), angles=tuple(float(v) for v in prm[4:7]),
                 fovy_deg=float(prm[7]), z_near=float(prm[8]), z_far=float(prm[9]))
    return sc, {k: z[k] for k in ("camera", "normal", "view", "lights7", "frame", "depth")}


def full_size():
    with open(os.path.join(GOLDEN, "full_size.json")) as fh:
        return json.load(fh)


def full_size_scene(entry):
    if entry["generator"] == "config_displaced_sphere":
        sc = S.config_displaced_sphere().with_view(angles=S.spin_angles(entry["frame"]))
    else:
        sc = S.config_soup()
    return sc
