"""CPU restatement of the proposal network's forward pass, pinball loss and
backward pass (numpy), for checking the GPU kernels of
ncrystal_gb300/csrc/ncgb_mlp.cu.  TEST INFRASTRUCTURE ONLY.

The GPU rounds GEMM operands to BF16 (weights, activations, output gradients)
and accumulates in FP32; this restatement rounds the same tensors to BF16 at
the same places and accumulates in FP64, so the two differ by accumulation
order only (and by the rare BF16 rounding or ReLU / pinball-indicator flip
that this causes).
"""
import numpy as np

K_IN, K_IN_USED, K_HID, K_OUT, K_OUT_PAD = 32, 19, 128, 62, 64
DIN = [K_IN, K_HID, K_HID, K_HID, K_HID]
DOUT = [K_HID, K_HID, K_HID, K_HID, K_OUT_PAD]


def layout():
    """Offsets of W_l ([din][dout] row-major) and b_l in the flat parameters."""
    off, w, b = 0, [], []
    for di, do in zip(DIN, DOUT):
        w.append(off)
        off += di * do
        b.append(off)
        off += do
    return w, b, off


def unpack(p):
    w, b, _ = layout()
    Ws = [p[w[l]:w[l] + DIN[l] * DOUT[l]].reshape(DIN[l], DOUT[l]).astype(np.float64) for l in range(5)]
    bs = [p[b[l]:b[l] + DOUT[l]].astype(np.float64) for l in range(5)]
    return Ws, bs


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def features(loge, temp, ranges):
    lmin, lmax, tmin, tmax = ranges
    loge = np.asarray(loge, dtype=np.float32)
    temp = np.asarray(temp, dtype=np.float32)
    x0 = (np.float32(2) * (loge - np.float32(lmin)) / np.float32(lmax - lmin) - np.float32(1)).astype(np.float32)
    x1 = (np.float32(2) * (temp - np.float32(tmin)) / np.float32(tmax - tmin) - np.float32(1)).astype(np.float32)
    f = np.zeros((len(loge), K_IN), dtype=np.float64)
    f[:, 0] = x0
    f[:, 1] = x1
    f[:, 2] = (x0 * x1).astype(np.float32)
    for k in range(1, 9):
        f[:, 1 + 2 * k] = np.sin(np.pi * k * x0.astype(np.float64))
        f[:, 2 + 2 * k] = np.cos(np.pi * k * x0.astype(np.float64))
    return bf16(f)


def softplus(x):
    return np.where(x > 20, x, np.log1p(np.exp(np.minimum(x, 20))))


def forward(p, loge, temp, ranges, emulate_bf16=True):
    """-> (raw outputs [n, 64], activations list)."""
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    Ws, bs = unpack(p)
    x = features(loge, temp, ranges)
    acts = [x]
    for l in range(5):
        z = x @ r(Ws[l]) + bs[l]
        if l < 4:
            x = r(np.maximum(z, 0.0))
            acts.append(x)
        else:
            out = z
    return out, acts


def knots(p, loge, temp, ranges, emulate_bf16=True):
    out, _ = forward(p, loge, temp, ranges, emulate_bf16)
    o = out[:, :K_OUT]
    g = np.empty_like(o)
    g[:, 0] = o[:, 0]
    g[:, 1:] = o[:, :1] + np.cumsum(softplus(o[:, 1:]), axis=1)
    return g


def loss_and_gradients(p, loge, temp, target, ranges):
    """Mean pinball loss over the 62 levels and its gradient (flat layout)."""
    Ws, bs = unpack(p)
    out, acts = forward(p, loge, temp, ranges)
    n = out.shape[0]
    o = out[:, :K_OUT]
    g = np.empty_like(o)
    g[:, 0] = o[:, 0]
    g[:, 1:] = o[:, :1] + np.cumsum(softplus(o[:, 1:]), axis=1)
    tau = np.arange(1, K_OUT + 1) / (K_OUT + 1.0)
    a = np.asarray(target, dtype=np.float64)[:, None]
    rr = a - g
    loss = np.sum(rr * np.where(rr < 0, tau - 1.0, tau)) / n
    dg = (a < g).astype(np.float64) - tau
    suffix = np.cumsum(dg[:, ::-1], axis=1)[:, ::-1]
    do = suffix.copy()
    do[:, 1:] *= 1.0 / (1.0 + np.exp(-o[:, 1:]))
    dz = np.zeros((n, K_OUT_PAD))
    dz[:, :K_OUT] = do / n
    dz = bf16(dz)
    w, b, total = layout()
    grad = np.zeros(total)
    for l in range(4, -1, -1):
        a_in = acts[l]
        grad[w[l]:w[l] + DIN[l] * DOUT[l]] = (a_in.T @ dz).ravel()
        grad[b[l]:b[l] + DOUT[l]] = dz.sum(axis=0)
        if l == 0:
            break
        dh = dz @ bf16(Ws[l]).T
        dz = bf16(dh * (acts[l] > 0))
    return loss, grad
