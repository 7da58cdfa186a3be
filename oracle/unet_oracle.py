"""FP64 CPU oracle for the U-Net denoiser's operators (TEST INFRASTRUCTURE ONLY).

RenderToy has no learned part (its demos call Intel OIDN, a closed binary),
so there is no reference to pin against: these are the textbook definitions,
written for clarity in float64 numpy, used to check the GPU kernels' forward
values and gradients on small shapes.  Layout NHWC; a 3x3 convolution weight
is [Cout, 3, 3, Cin]; "same" zero padding, stride 1.
"""
from __future__ import annotations

import numpy as np


def conv3x3(x, w, b=None):
    """y[n,y,x,o] = b[o] + sum_{i,j,c} x[n, y+i-1, x+j-1, c] * w[o,i,j,c]."""
    x = np.asarray(x, np.float64)
    w = np.asarray(w, np.float64)
    n, h, wd, c = x.shape
    xp = np.zeros((n, h + 2, wd + 2, c))
    xp[:, 1:-1, 1:-1] = x
    y = np.zeros((n, h, wd, w.shape[0]))
    for i in range(3):
        for j in range(3):
            y += np.einsum("nhwc,oc->nhwo", xp[:, i:i + h, j:j + wd], w[:, i, j, :])
    if b is not None:
        y += np.asarray(b, np.float64)
    return y


def conv3x3_dgrad(dy, w):
    """d x = conv of dy with the spatially flipped, channel-transposed weight."""
    dy = np.asarray(dy, np.float64)
    w = np.asarray(w, np.float64)
    n, h, wd, o = dy.shape
    dyp = np.zeros((n, h + 2, wd + 2, o))
    dyp[:, 1:-1, 1:-1] = dy
    dx = np.zeros((n, h, wd, w.shape[3]))
    for i in range(3):
        for j in range(3):
            # x[y+i-1] contributed to dy[y] with w[i]; so dx[y] gets dy[y-i+1] w[i]
            dx += np.einsum("nhwo,oc->nhwc", dyp[:, 2 - i:2 - i + h, 2 - j:2 - j + wd], w[:, i, j, :])
    return dx


def conv3x3_wgrad(x, dy):
    """dw[o,i,j,c] = sum_{n,y,x} dy[n,y,x,o] x[n, y+i-1, x+j-1, c]; db = sum dy."""
    x = np.asarray(x, np.float64)
    dy = np.asarray(dy, np.float64)
    n, h, wd, c = x.shape
    xp = np.zeros((n, h + 2, wd + 2, c))
    xp[:, 1:-1, 1:-1] = x
    dw = np.zeros((dy.shape[3], 3, 3, c))
    for i in range(3):
        for j in range(3):
            dw[:, i, j, :] = np.einsum("nhwo,nhwc->oc", dy, xp[:, i:i + h, j:j + wd])
    return dw, dy.sum(axis=(0, 1, 2))


def relu(x):
    return np.maximum(x, 0.0)


def relu_grad(x, dy):
    return np.where(x > 0.0, dy, 0.0)


def avgpool2(x):
    n, h, w, c = x.shape
    return x.reshape(n, h // 2, 2, w // 2, 2, c).mean(axis=(2, 4))


def avgpool2_grad(dy):
    return np.repeat(np.repeat(dy, 2, axis=1), 2, axis=2) * 0.25


def upsample2(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def upsample2_grad(dy):
    n, h, w, c = dy.shape
    return dy.reshape(n, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4))


KP_WIDTH = 5
KP_TAPS = KP_WIDTH * KP_WIDTH
REL_EPS = 1e-2


def sane(x):
    """Radiance made safe to filter: NaN and negatives 0, +inf the BF16 range."""
    x = np.nan_to_num(np.asarray(x, np.float64), nan=0.0, posinf=65504.0, neginf=0.0)
    return np.clip(x, 0.0, 65504.0)


def kp_taps(rad):
    """rad [N][H][W][3] -> [N][H][W][25][3]: tap k = offset
    (k // 5 - 2, k % 5 - 2) in (y, x), clamped to the frame."""
    r = KP_WIDTH // 2
    N, H, W, _ = rad.shape
    pad = np.pad(rad, ((0, 0), (r, r), (r, r), (0, 0)), mode="edge")
    return np.stack([pad[:, k // KP_WIDTH:k // KP_WIDTH + H, k % KP_WIDTH:k % KP_WIDTH + W]
                     for k in range(KP_TAPS)], axis=3)


def softmax(logits):
    z = logits - logits.max(-1, keepdims=True)
    e = np.exp(z)
    return e / e.sum(-1, keepdims=True)


def kp_apply(logits, raw):
    """The denoised radiance: softmax(logits[..., :25]) over the 5 x 5
    neighbourhood of the input radiance."""
    w = softmax(np.asarray(logits, np.float64)[..., :KP_TAPS])
    taps = kp_taps(sane(np.asarray(raw)[..., :3]))
    return (w[..., None] * taps).sum(3)


def kp_loss(logits, raw, target):
    """mean over pixels and channels of (o - t)^2 / (o^2 + eps), o the
    filtered radiance, the denominator held constant; returns the loss and
    its gradient with respect to the logits (zero beyond the 25 taps)."""
    logits = np.asarray(logits, np.float64)
    w = softmax(logits[..., :KP_TAPS])
    taps = kp_taps(sane(np.asarray(raw)[..., :3]))
    o = (w[..., None] * taps).sum(3)
    t = sane(target)
    den = o * o + REL_EPS
    d = o - t
    loss = (d * d / den).mean()
    g = 2.0 * d / den / d.size
    dw = (g[..., None, :] * taps).sum(-1)
    dl = np.zeros_like(logits)
    dl[..., :KP_TAPS] = w * (dw - (w * dw).sum(-1, keepdims=True))
    return loss, dl


def adam(p, g, m, v, step, lr=3e-4, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v


# ---------------------------------------------------------------------------
# The whole network, in FP64.
#
# Architecture (the denoiser's definition): 3 x 3 convolutions with ReLU
# except the last, 2 x 2 average pooling, nearest upsampling, skip
# concatenation after the upsampled channels.  Tensors carry padded channel
# counts (multiples of 8; the 11-channel input is padded to 16, the 25 filter
# logits of the output to 32), and the parameters live in one flat array:
# per layer w [cout_pad][9][cin_pad] then b [cout_pad], each start aligned to
# 4 floats.  With bf16=True every value the GPU stores in BF16 (the encoded
# input, the weights, activations, data gradients) is rounded to BF16
# (round-to-nearest-even) at the same point, so that only the accumulation
# order separates the two.
# ---------------------------------------------------------------------------

# tensor: (channels, level); level l has resolution full >> l
TENSORS = {
    "X": (16, 0), "A0a": (32, 0), "S0": (32, 0), "P1": (32, 1), "A1a": (64, 1), "S1": (64, 1),
    "P2": (64, 2), "A2a": (96, 2), "S2": (96, 2), "P3": (96, 3), "A3a": (128, 3), "S3": (128, 3),
    "P4": (128, 4), "B": (160, 4), "U3": (128, 3), "U2": (96, 2), "U1": (64, 1), "U0": (32, 0),
}
POOLED = {"P1": "S0", "P2": "S1", "P3": "S2", "P4": "S3"}
# (s1, s1 upsampled, s2, out, cout_pad, cout, cin, relu)
LAYERS = [
    ("X", 0, None, "A0a", 32, 32, 11, 1), ("A0a", 0, None, "S0", 32, 32, 32, 1),
    ("P1", 0, None, "A1a", 64, 64, 32, 1), ("A1a", 0, None, "S1", 64, 64, 64, 1),
    ("P2", 0, None, "A2a", 96, 96, 64, 1), ("A2a", 0, None, "S2", 96, 96, 96, 1),
    ("P3", 0, None, "A3a", 128, 128, 96, 1), ("A3a", 0, None, "S3", 128, 128, 128, 1),
    ("P4", 0, None, "B", 160, 160, 128, 1), ("B", 1, "S3", "U3", 128, 128, 288, 1),
    ("U3", 1, "S2", "U2", 96, 96, 224, 1), ("U2", 1, "S1", "U1", 64, 64, 160, 1),
    ("U1", 1, "S0", "U0", 32, 32, 96, 1), ("U0", 0, None, None, 32, KP_TAPS, 32, 0),
]


def layer_table():
    """Per layer: cout_pad, cout, cin_pad, cin, c1_pad, up1, relu, level,
    w_off, b_off (the layout of the flat parameter array); and its size."""
    rows, off = [], 0
    a4 = lambda n: (n + 3) // 4 * 4  # noqa: E731
    for s1, up, s2, out, cop, co, ci, relu in LAYERS:
        c1 = TENSORS[s1][0]
        cip = c1 + (TENSORS[s2][0] if s2 else 0)
        level = TENSORS[out][1] if out else 0
        w_off = off
        off = a4(off + cop * 9 * cip)
        b_off = off
        off = a4(off + cop)
        rows.append(dict(cout_pad=cop, cout=co, cin_pad=cip, cin=ci, c1_pad=c1, up1=up, relu=relu,
                         level=level, w_off=w_off, b_off=b_off))
    return rows, off


def real_param_count():
    return sum(co * 9 * ci + co for _, _, _, _, _, co, ci, _ in LAYERS)


def to_bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def init_params(seed=0):
    """He-normal weights on the real entries, zero padding and biases (the
    values differ from the GPU initialiser's; tests set parameters
    explicitly)."""
    rng = np.random.RandomState(seed)
    rows, n = layer_table()
    p = np.zeros(n)
    for r in rows:
        w = np.zeros((r["cout_pad"], 9, r["cin_pad"]))
        real_in = r["cin"] if r["cin_pad"] == r["c1_pad"] else r["cin_pad"]
        w[:r["cout"], :, :real_in] = rng.normal(0, np.sqrt(2.0 / (9 * r["cin"])), (r["cout"], 9, real_in))
        p[r["w_off"]:r["w_off"] + w.size] = w.ravel()
    return p


def encode_input(raw):
    """raw [N][H][W][11] -> [N][H][W][16]: log(1 + radiance) of the sane
    radiance, albedo / normal / depth as they are, log2(spp) / 16, 5 zero
    channels."""
    raw = np.asarray(raw, np.float64)
    x = np.zeros(raw.shape[:3] + (16,))
    x[..., :3] = np.log1p(sane(raw[..., :3]))
    x[..., 3:10] = raw[..., 3:10]
    x[..., 10] = np.log2(np.maximum(raw[..., 10], 1.0)) / 16.0
    return x


class UNet:
    """Forward / backward of the denoiser on a flat parameter array."""

    def __init__(self, params, bf16=False):
        self.rows, n = layer_table()
        assert params.size == n
        self.p = np.asarray(params, np.float64)
        self.bf16 = bf16
        self.r = to_bf16 if bf16 else (lambda a: a)

    def _wb(self, i):
        r = self.rows[i]
        w = self.p[r["w_off"]:r["w_off"] + r["cout_pad"] * 9 * r["cin_pad"]].reshape(r["cout_pad"], 3, 3, r["cin_pad"])
        b = self.p[r["b_off"]:r["b_off"] + r["cout_pad"]]
        return self.r(w), b

    def _input(self, i, act):
        s1, up, s2 = LAYERS[i][:3]
        x = upsample2(act[s1]) if up else act[s1]
        return np.concatenate([x, act[s2]], axis=3) if s2 else x

    def forward(self, raw):
        act = {"X": self.r(encode_input(raw))}
        for i, (s1, up, s2, out, *_rest) in enumerate(LAYERS):
            if s1 in POOLED:
                act[s1] = self.r(avgpool2(act[POOLED[s1]]))
            w, b = self._wb(i)
            z = conv3x3(self._input(i, act), w, b)
            if out is None:
                act["pred"] = z
            else:
                act[out] = self.r(relu(z))
        self.act = act
        return act["pred"]

    def denoise(self, raw):
        """The denoised radiance of a batch (the predicted filters applied)."""
        return kp_apply(self.forward(raw), raw)

    def loss_and_grads(self, raw, target):
        """The relative squared error of the filtered radiance (kp_loss);
        returns the loss and the gradient of the flat parameter array."""
        pred = self.forward(raw)
        act = self.act
        loss, dpred = kp_loss(pred, raw, target)
        dpred = self.r(dpred)
        grad = np.zeros_like(self.p)
        dact = {}
        for i in range(len(LAYERS) - 1, -1, -1):
            s1, up, s2, out, cop, co, ci, rl = LAYERS[i]
            r = self.rows[i]
            dout = dpred if out is None else dact[out]
            x = self._input(i, act)
            dw, db = conv3x3_wgrad(x, dout)
            grad[r["w_off"]:r["w_off"] + dw.size] = dw.reshape(cop, 9, -1).ravel()
            grad[r["b_off"]:r["b_off"] + cop] = db
            if i == 0:
                break
            w, _ = self._wb(i)
            din = conv3x3_dgrad(dout, w)
            if s1 not in POOLED:
                din = np.where(x > 0.0, din, 0.0)  # the sources are ReLU outputs
            din = self.r(din)
            c1 = TENSORS[s1][0]
            if s2:
                dact[s1] = self.r(upsample2_grad(din[..., :c1]))
                dact[s2] = din[..., c1:]
            elif s1 in POOLED:
                skip = POOLED[s1]
                dact[skip] = self.r(dact[skip] + np.where(act[skip] > 0.0, 0.25 * upsample2(din), 0.0))
            else:
                dact[s1] = din
        return loss, grad
