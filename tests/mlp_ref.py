"""Plain numpy restatement of the learned shader's network, the float reference for the
tensor-core kernel, and the "RMLP" weight blob format (rasteriser_gb300/csrc/rast_mlp.h)."""
import struct

import numpy as np

HEADER = struct.Struct("<4s7IQff")  # magic, version, n_in, n_hidden, n_out, n_freq, n_lights, reserved,
                                    # lights_hash, out_scale, train_loss
N_OUT = 3
VERSION = 3
# the networks of RAST_OPT_MLP_NETWORK: (Fourier frequencies, hidden width); inputs are 6F + 7,
# the constant-1 feature included
NETWORKS = {0: (3, 32), 1: (16, 64)}
N_FREQ, N_HID = NETWORKS[0]
N_IN = 6 * N_FREQ + 7


def dims(net):
    """(n_in, n_hidden, n_freq) of network `net`."""
    f, h = NETWORKS[net]
    return 6 * f + 7, h, f


def bf16_round(a):
    """float32 -> nearest-even BF16, returned as float32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def bf16_bits(a):
    return (bf16_round(a).view(np.uint32) >> 16).astype(np.uint16)


def features(n, alb, n_freq=N_FREQ):
    """(m, 6F + 7): sin / cos(f * pi * n_c) for c in xyz, f = 1..F (pairs), then n, albedo and 1."""
    n = np.asarray(n, np.float64)
    f = np.arange(1, n_freq + 1, dtype=np.float64)
    cols = []
    for c in range(3):
        ang = np.pi * f[None, :] * n[:, c:c + 1]
        cols.append(np.stack([np.sin(ang), np.cos(ang)], axis=2).reshape(-1, 2 * n_freq))
    ones = np.ones((n.shape[0], 1))
    return np.concatenate(cols + [n, np.asarray(alb, np.float64), ones], axis=1)


def random_weights(seed, scale=12.0, net=0):
    """Arbitrary BF16 weights of network `net`'s shapes (biases folded in: W1's last column)."""
    n_in, n_hid, n_freq = dims(net)
    rng = np.random.default_rng(seed)
    return {
        "w1": bf16_round(rng.uniform(-1, 1, (n_hid, n_in)) * np.sqrt(6.0 / n_in)),
        "w2": bf16_round(rng.uniform(-1, 1, (n_hid, n_hid)) * np.sqrt(6.0 / n_hid)),
        "w3": bf16_round(rng.uniform(-1, 1, (N_OUT, n_hid)) * np.sqrt(6.0 / n_hid) * 0.5),
        "scale": np.float32(scale),
        "n_freq": n_freq,
    }


def make_blob(w, n_lights=0, lights_hash=0, loss=0.0):
    n_hid, n_in = w["w1"].shape
    head = HEADER.pack(b"RMLP", VERSION, n_in, n_hid, N_OUT, w["n_freq"], n_lights, 0, lights_hash,
                       float(w["scale"]), loss)
    return head + b"".join([bf16_bits(w["w1"]).tobytes(), bf16_bits(w["w2"]).tobytes(), bf16_bits(w["w3"]).tobytes()])


def parse_blob(blob):
    h = HEADER.unpack_from(blob, 0)
    assert h[0] == b"RMLP" and h[1] == VERSION and (h[2], h[3], h[5]) in [dims(k) for k in NETWORKS]
    n_in, n_hid = h[2], h[3]
    off = HEADER.size

    def take(count):
        nonlocal off
        a = np.frombuffer(blob, np.uint16, count, off)
        off += a.nbytes
        return (a.astype(np.uint32) << 16).view(np.float32)

    w = {"w1": take(n_hid * n_in).reshape(n_hid, n_in), "w2": take(n_hid * n_hid).reshape(n_hid, n_hid),
         "w3": take(N_OUT * n_hid).reshape(N_OUT, n_hid), "n_freq": h[5],
         "scale": np.float32(h[9]), "n_lights": h[6], "lights_hash": h[8], "loss": h[10]}
    assert off == len(blob)
    return w


def forward(w, n, alb):
    """Radiance (m, 3) before clamping: BF16 inputs and hidden activations, float64 sums."""
    x = bf16_round(features(n, alb, w["n_freq"]).astype(np.float32)).astype(np.float64)
    h1 = bf16_round(np.maximum(x @ w["w1"].T.astype(np.float64), 0).astype(np.float32)).astype(np.float64)
    h2 = bf16_round(np.maximum(h1 @ w["w2"].T.astype(np.float64), 0).astype(np.float32)).astype(np.float64)
    o = h2 @ w["w3"].T.astype(np.float64)
    return np.asarray(alb, np.float64) * (o * float(w["scale"]))


def lights_hash(lights7):
    """FNV-1a 64 of the light records' bytes."""
    h = 0xcbf29ce484222325
    for b in np.ascontiguousarray(lights7, np.float32).tobytes():
        h ^= b
        h = (h * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    return h
