"""The warp-level work distribution of k_setup_raster (rast_kernels.cu), restated in Python and
checked on random layouts:

- the item windows: a warp's 32 triangles lay their items end to end and take them 32 at a time;
  the owner of item k is the last triangle whose items start at or before k within the window (an
  OR-reduction of start positions), else the owner of the window's first item carried over from
  the previous window. It must be the triangle the item belongs to;
- the ring of candidate runs: each window pushes up to 32 runs; drain rounds take exactly 32
  pending pixels (a run left partly done stays at the head with its done pixels counted), so at
  most 63 runs are ever pending in the 64-entry ring, and every pixel of every run is processed
  exactly once.
"""
import random

import numpy as np
import pytest


def owners_by_window(n_items):
    """Owner of every item, computed window by window as the kernel does."""
    incl = np.cumsum(n_items)
    start = incl - n_items
    total = int(incl[-1]) if len(incl) else 0
    out = []
    carry = 0
    slot = [None] * 32
    for base in range(0, total, 32):
        starts = 0
        for lane in range(32):
            if n_items[lane] and base <= start[lane] < base + 32:
                slot[start[lane] - base] = lane
                starts |= 1 << int(start[lane] - base)
        owners = []
        for lane in range(32):
            upto = starts & (0xFFFFFFFF >> (31 - lane))
            owners.append(slot[upto.bit_length() - 1] if upto else carry)
        for lane in range(32):
            if base + lane < total:
                out.append(owners[lane])
        carry = owners[31]
    return out


@pytest.mark.parametrize("seed", range(4))
def test_item_owners(seed):
    rng = np.random.default_rng(seed)
    for trial in range(2000):
        n = rng.integers(0, 6, 32) * (rng.random(32) < 0.6)
        if trial % 7 == 0:
            n = rng.integers(0, 80, 32) * (rng.random(32) < 0.3)
        if trial % 11 == 0:
            n = np.zeros(32, np.int64)
            n[rng.integers(0, 32)] = rng.integers(1, 200)
        truth = np.repeat(np.arange(32), n).tolist()
        assert owners_by_window(n) == truth


class Ring:
    """The warp's ring of candidate runs and its drain rounds."""

    def __init__(self):
        self.xy = [None] * 64
        self.om = [None] * 64
        self.n = [None] * 64
        self.head = self.count = self.skip = self.pix = 0
        self.done = []

    def push(self, runs):
        """runs: up to 32 (owner, first pixel, length) entries of one window, in lane order."""
        assert self.count + len(runs) <= 64
        for k, (own, x0, n) in enumerate(runs):
            e = (self.head + self.count + k) & 63
            self.xy[e], self.om[e], self.n[e] = x0, own, n
        self.count += len(runs)
        self.pix += sum(r[2] for r in runs)
        while self.pix >= 32:
            self.round()
        assert self.count < 32 and self.count <= self.pix

    def round(self):
        cnt = [0] * 32
        xy = [0] * 32
        own = [0] * 32
        for lane in range(min(self.count, 32)):
            e = (self.head + lane) & 63
            xy[lane], own[lane], cnt[lane] = self.xy[e], self.om[e], self.n[e]
            if lane == 0:
                xy[lane] += self.skip
                cnt[lane] -= self.skip
        incl = [int(v) for v in np.cumsum(cnt)]
        excl = [incl[i] - cnt[i] for i in range(32)]
        slot = {}
        starts = 0
        for lane in range(32):
            if cnt[lane] and excl[lane] < 32:
                slot[excl[lane]] = lane
                starts |= 1 << excl[lane]
        avail = min(self.pix, 32)
        for lane in range(avail):
            src = slot[(starts & ((1 << (lane + 1)) - 1)).bit_length() - 1]
            off = lane - excl[src]
            assert 0 <= off < cnt[src]
            self.done.append((own[src], xy[src] + off))
        nd = sum(1 for lane in range(32) if lane < self.count and incl[lane] <= avail)
        sk = excl[nd & 31]
        self.skip = self.skip + avail if nd == 0 else (avail - sk if (nd < self.count and nd < 32) else 0)
        self.head = (self.head + nd) & 63
        self.count -= nd
        self.pix -= avail


@pytest.mark.parametrize("seed", range(6))
def test_run_ring_processes_every_pixel_once(seed):
    rnd = random.Random(seed)
    ring = Ring()
    want = []
    for w in range(rnd.randint(20, 200)):
        runs = []
        for lane in range(32):
            r = rnd.random()
            if r < 0.4:
                continue
            n = 1 if seed % 3 == 0 else (rnd.randint(1, 3) if r < 0.9 else rnd.randint(1, 64))
            x0 = rnd.randint(0, 30000)
            runs.append(((w, lane), x0, n))
            want += [((w, lane), x0 + i) for i in range(n)]
        ring.push(runs)
    if ring.pix:
        ring.round()
    assert ring.pix == 0 and ring.count == 0
    assert sorted(ring.done) == sorted(want) and len(ring.done) == len(set(ring.done))
