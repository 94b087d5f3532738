"""Float32/float64 NumPy reference of the learned initializer's network, for the
tests of the tensor-core kernels (test infrastructure, no GPU).

Layouts follow the C ABI (include/ptycho_gb300.h): activations NHWC, 3 x 3
weights (cout, 9, cin) with tap = ky * 3 + kx and offsets (ky - 1, kx - 1).
Values that the GPU holds in bfloat16 are rounded to bfloat16 here with
round-to-nearest-even (bf16_round), so that the comparison sees only the
accumulation order and the float32 arithmetic.
"""

import numpy as np

CIN = (8, 32, 32, 64, 64, 128, 128, 256, 384, 128, 192, 64, 96, 32)
COUT = (32, 32, 64, 64, 128, 128, 256, 256, 128, 128, 64, 64, 32, 32)
LEVEL = (0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0)


def bf16_bits(a):
    """float32 array -> uint16 bfloat16 bits, round to nearest even."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return r.astype(np.uint16)


def bf16_to_f32(bits):
    return (np.asarray(bits, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def bf16_round(a):
    return bf16_to_f32(bf16_bits(a))


def im2col(x):
    """(n, H, W, C) -> (n, H, W, 9, C) with zero padding; tap = ky * 3 + kx."""
    n, H, W, C = x.shape
    xp = np.zeros((n, H + 2, W + 2, C), dtype=x.dtype)
    xp[:, 1:-1, 1:-1] = x
    cols = np.empty((n, H, W, 9, C), dtype=x.dtype)
    for ky in range(3):
        for kx in range(3):
            cols[:, :, :, ky * 3 + kx] = xp[:, ky:ky + H, kx:kx + W]
    return cols


def conv3x3(x, w, b=None, relu=False):
    """x (n, H, W, cin), w (cout, 9, cin) -> (n, H, W, cout) in float64."""
    cols = im2col(x.astype(np.float64))
    y = np.einsum("nhwtc,otc->nhwo", cols, w.astype(np.float64))
    if b is not None:
        y = y + b
    return np.maximum(y, 0.0) if relu else y


def conv3x3_backward_data(dy, w):
    """Gradient wrt the input: the transposed convolution of dy."""
    n, H, W, cout = dy.shape
    dyp = np.zeros((n, H + 2, W + 2, cout))
    dyp[:, 1:-1, 1:-1] = dy
    dx = np.zeros((n, H, W, w.shape[2]))
    w = w.astype(np.float64)
    for ky in range(3):
        for kx in range(3):
            # y[p] += w[tap] x[p + off]  =>  dx[q] += w[tap]^T dy[q - off]
            src = dyp[:, 2 - ky:2 - ky + H, 2 - kx:2 - kx + W]
            dx += np.einsum("nhwo,oc->nhwc", src, w[:, ky * 3 + kx, :])
    return dx


def conv3x3_backward_weight(x, dy):
    cols = im2col(x.astype(np.float64))
    dw = np.einsum("nhwo,nhwtc->otc", dy.astype(np.float64), cols)
    return dw, dy.sum(axis=(0, 1, 2))


def maxpool(x):
    n, H, W, C = x.shape
    v = x.reshape(n, H // 2, 2, W // 2, 2, C).transpose(0, 1, 3, 2, 4, 5).reshape(
        n, H // 2, W // 2, 4, C)
    idx = np.argmax(v, axis=3)
    return np.take_along_axis(v, idx[:, :, :, None], axis=3)[:, :, :, 0], idx


def maxpool_backward(dp, idx, shape):
    n, H, W, C = shape
    out = np.zeros((n, H // 2, W // 2, 4, C))
    np.put_along_axis(out, idx[:, :, :, None], dp[:, :, :, None], axis=3)
    return out.reshape(n, H // 2, W // 2, 2, 2, C).transpose(0, 1, 3, 2, 4, 5).reshape(shape)


def upsample(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def upsample_backward(d):
    n, H, W, C = d.shape
    return d.reshape(n, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


class UNetReference:
    """Forward and backward of the U-Net in float64 from given weights, with the
    activations rounded to bfloat16 where the GPU stores them."""

    def __init__(self, w, b, hw, hb):
        self.w = [np.asarray(x, np.float64) for x in w]
        self.b = [np.asarray(x, np.float64) for x in b]
        self.hw = np.asarray(hw, np.float64)
        self.hb = float(hb)

    def forward(self, inp):
        n, H, W, _ = inp.shape
        x = np.zeros((n, H, W, 8))
        x[..., :2] = bf16_round(inp)
        t = {"in": x}

        def conv(l, src):
            t[l] = bf16_round(conv3x3(src, bf16_round(self.w[l]), self.b[l], relu=True))
            return t[l]

        conv(1, conv(0, x))
        p = {}
        for k, (lo, nxt) in enumerate(((1, 2), (3, 4), (5, 6))):
            p[k], t[("idx", k)] = maxpool(t[lo])
            conv(nxt + 1, conv(nxt, p[k]))
        t["pool"] = p
        cats = {}
        for k, (low, skip, d) in enumerate(((7, 5, 8), (9, 3, 10), (11, 1, 12))):
            cats[d] = np.concatenate([upsample(t[low]), t[skip]], axis=-1)
            conv(d + 1, conv(d, cats[d]))
        t["cat"] = cats
        out = t[13] @ self.hw + self.hb
        self.t = t
        return out

    def gradients(self, inp, target, mask=None):
        """Loss and parameter gradients (float64) for the masked mean squared error."""
        out = self.forward(inp)
        t = self.t
        m = np.ones_like(out) if mask is None else mask
        count = m.sum()
        loss = float(np.sum(m * (out - target) ** 2) / count)
        dout = 2.0 * (out - target) * m / count
        gw, gb = [None] * 14, [None] * 14
        ghw = np.einsum("nhw,nhwc->c", dout, t[13])
        ghb = float(dout.sum())
        g = bf16_round(dout[..., None] * self.hw * (t[13] > 0))

        def back(l, src, g, need_dx=True):
            gw[l], gb[l] = conv3x3_backward_weight(src, g)
            return conv3x3_backward_data(g, bf16_round(self.w[l])) if need_dx else None

        dcat = {}
        for low, d in ((11, 12), (9, 10), (7, 8)):
            dx = back(d + 1, t[d], g)
            g = bf16_round(dx * (t[d] > 0))
            dcat[d] = back(d, t["cat"][d], g)
            c1 = COUT[low]
            g = bf16_round(upsample_backward(dcat[d][..., :c1]) * (t[low] > 0))
        for k, (l, up, d) in enumerate(((6, 5, 8), (4, 3, 10), (2, 1, 12), (0, None, None))):
            dx = back(l + 1, t[l], g)
            g = bf16_round(dx * (t[l] > 0))
            if l == 0:
                back(0, t["in"], g, need_dx=False)
                break
            pool_i = 2 - k
            dp = back(l, t["pool"][pool_i], g)
            dsk = maxpool_backward(dp, t[("idx", pool_i)], t[up].shape)
            c1 = CIN[d] - COUT[up]
            dsk = dsk + dcat[d][..., c1:]
            g = bf16_round(dsk * (t[up] > 0))
        return loss, gw, gb, ghw, ghb
