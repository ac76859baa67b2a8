"""CPU oracle of the learned closure's network -- TEST INFRASTRUCTURE ONLY.

The network is 6 -> 64 -> 64 -> 64 -> 64 -> 2 with SiLU after every hidden
layer, parameters in the flat layout of include/tsr_capi.h (tsr_mlp_*).
The GPU kernels round every GEMM operand to BF16 (round to nearest even)
where they load it and accumulate in FP32; with ``bf16=True`` this oracle
rounds at exactly the same points and accumulates in FP64, so the two
differ only by FP32 accumulation order.  With ``bf16=False`` it is the plain
FP64 network, whose gradient is checked against finite differences.
"""
import numpy as np

N_IN, N_IN_PAD, HID, N_OUT, N_OUT_PAD = 6, 16, 64, 2, 8
SHAPES = [(HID, N_IN_PAD), (HID, HID), (HID, HID), (HID, HID), (N_OUT_PAD, HID)]


def layout():
    """(weight offset, bias offset, n_out, n_in) per layer and the total."""
    out, off = [], 0
    for no, ni in SHAPES:
        w = off
        off += no * ni
        b = off
        off += no
        out.append((w, b, no, ni))
    return out, off


LAYOUT, N_PARAMS = layout()


def unpack(p):
    """Views (W [out][in], b [out]) of a flat parameter block."""
    p = np.asarray(p)
    return [(p[w:b].reshape(no, ni), p[b:b + no]) for (w, b, no, ni) in LAYOUT]


def init_params(seed):
    """Seeded initial parameters: uniform(+-1/sqrt(fan_in)) weights on the
    real inputs / outputs, zero biases, zero padding."""
    rng = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, dtype=np.float32)
    for li, (w, b, no, ni) in enumerate(LAYOUT):
        fan_in = N_IN if li == 0 else ni
        W = rng.uniform(-1.0, 1.0, size=(no, ni)) / np.sqrt(fan_in)
        if li == 0:
            W[:, N_IN:] = 0.0
        if li == len(LAYOUT) - 1:
            W[N_OUT:, :] = 0.0
        p[w:b] = W.astype(np.float32).ravel()
    return p


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32)


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, x, bf=True):
    """Outputs (n x 2) and the saved pre-activations / activations."""
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    f32 = (lambda a: np.asarray(a, dtype=np.float32)) if bf else (lambda a: a)
    layers = unpack(p)
    n = x.shape[0]
    a = np.zeros((n, N_IN_PAD), dtype=np.float64)
    a[:, :N_IN] = x[:, :N_IN]
    acts, zs = [f32(a)], []
    for li, (W, b) in enumerate(layers):
        z = r(acts[-1]).astype(np.float64) @ r(W).astype(np.float64).T + b
        z = f32(z)
        zs.append(z)
        if li < len(layers) - 1:
            s = _silu(np.asarray(z, dtype=np.float64))
            acts.append(f32(s))
    return np.asarray(zs[-1][:, :N_OUT], dtype=np.float64), (acts, zs)


def loss_grad(p, x, y, bf=True):
    """Mean squared error over rows and the 2 outputs, and its gradient."""
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    out, (acts, zs) = forward(p, x, bf)
    n = x.shape[0]
    layers = unpack(p)
    d = out - y[:, :N_OUT]
    loss = float(np.mean(d * d))
    dz = np.zeros((n, N_OUT_PAD))
    dz[:, :N_OUT] = 2.0 * d / (n * N_OUT)
    if bf:
        dz = dz.astype(np.float32)
    g = np.zeros(N_PARAMS)
    for li in range(len(layers) - 1, -1, -1):
        w, b, no, ni = LAYOUT[li]
        W = layers[li][0]
        g[w:b] = (r(dz).astype(np.float64).T @ r(acts[li]).astype(np.float64)).ravel()
        g[b:b + no] = np.asarray(dz, dtype=np.float64).sum(axis=0)
        if li > 0:
            da = r(dz).astype(np.float64) @ r(W).astype(np.float64)
            dz = da * _dsilu(np.asarray(zs[li - 1], dtype=np.float64))
            if bf:
                dz = dz.astype(np.float32)
    return loss, g
