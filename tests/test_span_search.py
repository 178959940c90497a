"""The whole-item interval search of k_setup_raster (rast_kernels.cu), restated in numpy float32
(one rounding per operation, as the kernel's __f*_rn steps) and checked against a brute-force scan
of the same items. For every item whose ends verify, the interval must be exactly the set of
pixels whose three staged edge values pass the early reject; items that do not verify fall back
to the scan in the kernel, so they only count towards the verification rate.

Also checks the column remap: (U, V, W, Z) = (-B, X, -A, Y) gives the reference's rounded edge
value A*(py - Y) - B*(px - X) (drawing.cpp:36-39) bit for bit."""
import numpy as np
import pytest

f32 = np.float32


def edge_ref(A, B, X, Y, px, py):
    """sgn(area) * the reference's edge function, each operation rounded."""
    return ((A * (py - Y)).astype(f32) - (B * (px - X)).astype(f32)).astype(f32)


def edge_item(K, W, Z, t):
    """The kernel's f(t) = K - W * (t - Z) along an item."""
    return (K - (W * (t - Z)).astype(f32)).astype(f32)


def triangles(rng, n, spread, integer=False):
    c = np.stack([rng.uniform(0, 640, n), rng.uniform(0, 480, n)], 1)[:, None, :]
    p = (c + rng.normal(0, 1, (n, 3, 2)) * np.asarray(spread)).astype(f32)
    if integer:
        p = np.round(p).astype(f32)
    return p


def items(p, W_px, H_px, columns):
    """The items of each front- or back-facing triangle with a normal area, staged as the kernel
    stages them: per edge (U, V, W, Z), thr, and the item's range and fixed coordinate."""
    a, b, c = p[:, 0], p[:, 1], p[:, 2]
    d12x, d12y = c[:, 0] - b[:, 0], c[:, 1] - b[:, 1]
    d20x, d20y = a[:, 0] - c[:, 0], a[:, 1] - c[:, 1]
    d01x, d01y = b[:, 0] - a[:, 0], b[:, 1] - a[:, 1]
    area = ((d01x * (c[:, 1] - a[:, 1])).astype(f32) - (d01y * (c[:, 0] - a[:, 0])).astype(f32)).astype(f32)
    keep = (np.abs(area) >= 2.0 ** -26) & np.isfinite(area)
    sg = np.where(area > 0, f32(1), f32(-1))
    thr = (-(np.abs(area) * f32(2.0 ** -100))).astype(f32)
    A = [sg * d12x, sg * d20x, sg * d01x]
    B = [sg * d12y, sg * d20y, sg * d01y]
    X = [b[:, 0], c[:, 0], a[:, 0]]
    Y = [b[:, 1], c[:, 1], a[:, 1]]
    xs, ys = p[:, :, 0], p[:, :, 1]
    tlx = np.clip(xs.min(1), 0, W_px - 1).astype(np.int64)
    brx = np.clip(np.ceil(xs.max(1)), 0, W_px - 1).astype(np.int64)
    tly = np.clip(ys.min(1), 0, H_px - 1).astype(np.int64)
    bry = np.clip(np.ceil(ys.max(1)), 0, H_px - 1).astype(np.int64)
    if columns:
        U, V, Wc, Z = [-x for x in B], X, [-x for x in A], Y
        lo, hi, f0, f1 = tly, bry, tlx, brx
    else:
        U, V, Wc, Z = A, Y, B, X
        lo, hi, f0, f1 = tlx, brx, tly, bry
    n = np.where(keep, f1 - f0 + 1, 0)
    idx = np.repeat(np.arange(len(p)), n)
    fixed = f0[idx] + np.concatenate([np.arange(k) for k in n]) if len(idx) else np.zeros(0, np.int64)
    ff = fixed.astype(f32)
    K = [(U[k][idx] * (ff - V[k][idx])).astype(f32) for k in range(3)]
    coef = dict(K=K, W=[Wc[k][idx] for k in range(3)], Z=[Z[k][idx] for k in range(3)], thr=thr[idx],
                lo=lo[idx], hi=hi[idx], fixed=fixed)
    ref = dict(A=[A[k][idx] for k in range(3)], B=[B[k][idx] for k in range(3)],
               X=[X[k][idx] for k in range(3)], Y=[Y[k][idx] for k in range(3)])
    return coef, ref


def search(K, W, Z, thr, lo, hi):
    """The kernel's branch-free crossing checks: (verified, L, U)."""
    lof, hif = lo.astype(f32), hi.astype(f32)
    L, U = lof.copy(), hif.copy()
    ok = np.ones(len(lo), bool)
    with np.errstate(all="ignore"):
        for k in range(3):
            R = (f32(1) / W[k]).astype(f32)
            pos = W[k] >= 0
            est = (Z[k] + (K[k] * R).astype(f32)).astype(f32)
            fl = np.floor(est).astype(f32)
            mf = np.where(~pos & (fl == est), fl - f32(1), fl).astype(f32)
            mf = np.where(W[k] == 0, np.where(K[k] >= thr, hif, lof - f32(1)), mf).astype(f32)
            mf = np.fmin(np.fmax(mf, lof - f32(1)), hif).astype(f32)
            mf1 = (mf + f32(1)).astype(f32)
            p0 = edge_item(K[k], W[k], Z[k], mf) >= thr
            p1 = edge_item(K[k], W[k], Z[k], mf1) >= thr
            in0, in1 = mf >= lof, mf1 <= hif
            ok &= (~in0 | (p0 == pos)) & (~in1 | (p1 != pos))
            U = np.where(pos, np.fmin(U, mf), U)
            L = np.where(pos, L, np.fmax(L, mf1))
    return ok, L.astype(np.int64), U.astype(np.int64)


def brute(coef, ref, columns):
    lo, hi, fixed, thr = coef["lo"], coef["hi"], coef["fixed"], coef["thr"]
    L = np.full(len(lo), 1 << 40)
    U = np.full(len(lo), -1)
    for d in range(int((hi - lo).max()) + 1 if len(lo) else 0):
        t = lo + d
        px, py = (fixed, t) if columns else (t, fixed)
        ok = t <= hi
        with np.errstate(all="ignore"):
            for k in range(3):
                ok &= edge_ref(ref["A"][k], ref["B"][k], ref["X"][k], ref["Y"][k],
                               px.astype(f32), py.astype(f32)) >= thr
        L = np.where(ok & (L == 1 << 40), t, L)
        U = np.where(ok, t, U)
    return L, U


@pytest.mark.parametrize("columns", [False, True])
@pytest.mark.parametrize("spread,integer", [((3.0, 3.0), False), ((1.0, 12.0), False), ((12.0, 1.0), False),
                                            ((0.3, 0.3), False), ((4.0, 4.0), True), ((40.0, 2.0), False)])
def test_interval_search_matches_scan(columns, spread, integer):
    rng = np.random.default_rng(11 + int(spread[0] * 7) + 3 * int(integer) + 5 * int(columns))
    p = triangles(rng, 20000, spread, integer)
    coef, ref = items(p, 640, 480, columns)
    ok, L, U = search(coef["K"], coef["W"], coef["Z"], coef["thr"], coef["lo"], coef["hi"])
    bL, bU = brute(coef, ref, columns)
    empty = bU < 0
    agree = np.where(empty, L > U, (L == bL) & (U == bU))
    assert len(ok) > 10000
    assert not (ok & ~agree).any()        # every verified interval is exact
    assert ok.mean() > (0.9 if integer else 0.995)


@pytest.mark.parametrize("scale", [1.0, 1e-3, 1e3, 1e-30, 1e30])
def test_column_remap_is_bit_identical(scale):
    rng = np.random.default_rng(5)
    n = 500000
    A = (rng.normal(0, 1, n) * scale).astype(f32)
    B = (rng.normal(0, 1, n) * scale).astype(f32)
    X = rng.uniform(-100, 2000, n).astype(f32)
    Y = rng.uniform(-100, 1200, n).astype(f32)
    px = rng.integers(0, 1920, n).astype(f32)
    py = rng.integers(0, 1080, n).astype(f32)
    with np.errstate(all="ignore"):
        r = edge_ref(A, B, X, Y, px, py)
        K = (-B * (px - X)).astype(f32)                 # U * (fixed - V) with U = -B, V = X
        c = edge_item(K, -A, Y, py)                     # W = -A, Z = Y, t = py
    assert np.array_equal(r.view(np.uint32), c.view(np.uint32))
