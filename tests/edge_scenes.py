"""Hand-built scenes for the edge cases of the reference's raster loop (drawing.cpp:77-203):
depth ties between triangles, vertices behind the camera, off-screen and clamped bounding boxes,
degenerate triangles drawn under --wind-clockwise, and NaN / infinite vertices."""
import numpy as np

from rasteriser_gb300 import scenes as S


def _scene(name, pos, tris, kd, nrm=None, **view):
    pos = np.asarray(pos, np.float32)
    tris = np.asarray(tris, np.int32)
    nrm = np.array([[0, 0, 1]], np.float32) if nrm is None else np.asarray(nrm, np.float32)
    sc = S.Scene(name, pos, tris, nrm, np.zeros((0, 2), np.float32), np.asarray(kd, np.float32),
                 S.rig_three_point())
    return sc.with_view(**view)


def _t(v, mat=0, n=(0, 0, 0)):
    return [v[0], v[1], v[2], n[0], n[1], n[2], -1, -1, -1, mat]


def ties():
    """Identical and edge-sharing triangles: equal depths go to the lowest triangle index."""
    pos = [[-1, -1, 0], [1, -1, 0], [-1, 1, 0], [1, 1, 0], [0, 0, 0.2]]
    tris = [_t((0, 1, 3), 1), _t((0, 1, 3), 0), _t((0, 3, 2), 2), _t((0, 3, 2), 1), _t((0, 1, 4), 2),
            _t((1, 3, 4), 0)]
    kd = [[0.9, 0.2, 0.2], [0.2, 0.9, 0.2], [0.2, 0.2, 0.9]]
    return _scene("ties", pos, tris, kd, width=320, height=240, fovy_deg=60.0, z_near=0.1, z_far=100.0)


def behind_camera():
    """Triangles with vertices behind the eye (w < 0) and across the near plane; the reference does
    no clipping, so these project through the divide as they are."""
    pos = [[-0.5, -0.5, 0], [0.5, -0.5, 0], [0, 0.5, 4.0], [-2, -0.2, 1.0], [2, -0.3, 1.0], [0, 0.7, 3.2],
           [-0.3, 0.1, 2.95], [0.4, 0.2, 2.95], [0.0, -0.4, 2.85]]
    tris = [_t((0, 1, 2)), _t((3, 4, 5)), _t((6, 8, 7)), _t((6, 7, 8))]
    return _scene("behind_camera", pos, tris, [[0.8, 0.8, 0.8]], width=320, height=200, fovy_deg=60.0,
                  z_near=0.1, z_far=100.0)


def off_screen():
    """Triangles partly and wholly outside the frame: clamped boxes test border rows/columns."""
    pos = []
    tris = []
    for k, (cx, cy) in enumerate([(-3.5, 0), (3.5, 0.2), (0.1, 2.8), (-0.2, -2.9), (-2.4, 1.6), (2.6, -1.5),
                                  (-1.85, 0.3), (1.9, -0.4), (0.3, 1.45)]):
        b = len(pos)
        pos += [[cx - 0.6, cy - 0.5, 0], [cx + 0.6, cy - 0.4, 0], [cx, cy + 0.7, 0]]
        tris.append(_t((b, b + 1, b + 2)))
    return _scene("off_screen", pos, tris, [[0.7, 0.8, 0.9]], width=256, height=160, fovy_deg=60.0,
                  z_near=0.1, z_far=100.0)


def degenerate_clockwise():
    """Zero-area and sliver triangles drawn with --wind-clockwise, which makes them front faces: the
    reference divides by a zero area and keeps whatever the IEEE results say."""
    pos = [[-1, -1, 0], [1, -1, 0], [0, 1, 0], [0.5, 0.5, 0], [-0.5, 0.5, 0], [0.25, 0.25, 0],
           [0.25, 0.2500001, 0], [-0.8, 0.8, 0.1], [0.8, -0.8, 0.1], [0.0, 0.0, 0.1]]
    tris = [_t((0, 0, 0)), _t((0, 1, 1)), _t((0, 5, 3)), _t((5, 6, 3)), _t((7, 8, 9)), _t((0, 2, 1)),
            _t((4, 3, 2))]
    return _scene("degenerate_cw", pos, tris, [[0.8, 0.8, 0.8]], width=200, height=200, wind_clockwise=True,
                  fovy_deg=60.0, z_near=0.1, z_far=100.0)


def nonfinite():
    """Vertices at NaN and +-inf mixed with ordinary triangles."""
    nan, inf = np.nan, np.inf
    pos = [[-1, -1, 0], [1, -1, 0], [0, 1, 0], [nan, 0, 0], [0.5, nan, 0], [inf, 0.2, 0], [-inf, 0.1, 0],
           [0.1, 0.2, nan]]
    tris = [_t((0, 1, 2)), _t((0, 3, 2)), _t((4, 1, 2)), _t((0, 1, 5)), _t((6, 1, 2)), _t((0, 1, 7)),
            _t((5, 6, 2))]
    return _scene("nonfinite", pos, tris, [[0.8, 0.8, 0.8]], width=160, height=120, fovy_deg=60.0,
                  z_near=0.1, z_far=100.0)


def all_edge_scenes():
    return [ties(), behind_camera(), off_screen(), degenerate_clockwise(), degenerate_clockwise().with_view(
        wind_clockwise=False), nonfinite(), nonfinite().with_view(wind_clockwise=True)]
