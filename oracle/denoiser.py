"""CPU restatement (numpy, FP64) of the dose denoiser: a 3D convolutional
encoder-decoder with forward, backward and Adam.

TEST INFRASTRUCTURE ONLY: the tests check the GPU kernels' forward pass, gradients
and optimiser step against this module, and check this module's own gradients by
finite differences.  The product never imports it.  The network has no counterpart
in the reference; its layout is this project's:

  encoder level l (0..L-1), resolution R / 2^l:
      e_la = relu(conv3(x_l)), e_lb = relu(conv3(e_la)),  x_{l+1} = avgpool2(e_lb)
      (x_0 = the input channels)
  decoder level l = L-2..0:
      d_la = relu(conv3(concat(upsample2(d_{l+1}), e_lb))), d_lb = relu(conv3(d_la))
      (d_{L-1} = e_{L-1,b})
  head: pred = conv1(d_0b) (one channel, no activation); loss = mean |pred - target|

conv3 is a 3x3x3 convolution with zero padding; weights are stored [Cout][27][Cin]
with tap t = (dz+1)*9 + (dy+1)*3 + (dx+1).  Tensors are [B][D][H][W][C].

With `bf16=True` the functions round every tensor the GPU stores in bfloat16
(weights, activations, activation gradients) at the same points, so that the
comparison measures accumulation order only.
"""
from __future__ import annotations

import numpy as np

TAPS = [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def round_bf16(a):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    out = r.view(np.float32).astype(np.float64)
    return np.where(np.isnan(f), np.nan, out)


def _shift(xp, tap, D, H, W):
    dz, dy, dx = tap
    return xp[:, 1 + dz:1 + dz + D, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W, :]


def conv3(x, Wt, b):
    """y[v, o] = b[o] + sum_t sum_c x[v + off(t), c] W[o, t, c] (zero padding)."""
    B, D, H, W_, C = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))
    y = np.broadcast_to(b, (B, D, H, W_, Wt.shape[0])).astype(np.float64).copy()
    for t, tap in enumerate(TAPS):
        y += np.einsum("bdhwc,oc->bdhwo", _shift(xp, tap, D, H, W_), Wt[:, t, :], optimize=True)
    return y


def conv3_backward(x, Wt, dz):
    """Gradients of conv3 given dz = dL/dy: (dx, dW, db)."""
    B, D, H, W_, C = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))
    dW = np.zeros_like(Wt, dtype=np.float64)
    dxp = np.zeros(xp.shape)
    for t, tap in enumerate(TAPS):
        dW[:, t, :] = np.einsum("bdhwo,bdhwc->oc", dz, _shift(xp, tap, D, H, W_), optimize=True)
        dz_, dy_, dx_ = tap
        dxp[:, 1 + dz_:1 + dz_ + D, 1 + dy_:1 + dy_ + H, 1 + dx_:1 + dx_ + W_, :] += np.einsum(
            "bdhwo,oc->bdhwc", dz, Wt[:, t, :], optimize=True)
    db = dz.sum(axis=(0, 1, 2, 3))
    return dxp[:, 1:-1, 1:-1, 1:-1, :], dW, db


def avgpool2(x):
    B, D, H, W, C = x.shape
    return x.reshape(B, D // 2, 2, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4, 6))


def avgpool2_backward(dy):
    return upsample2(dy) / 8.0


def upsample2(x):
    return x.repeat(2, axis=1).repeat(2, axis=2).repeat(2, axis=3)


def upsample2_backward(dy):
    B, D, H, W, C = dy.shape
    return dy.reshape(B, D // 2, 2, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4, 6))


class UNet:
    """Parameters in one flat FP64 vector, in layer order: enc0a, enc0b, ...,
    enc(L-1)b, dec(L-2)a, dec(L-2)b, ..., dec0a, dec0b (each W then b), then the
    head (w[C0], b)."""

    def __init__(self, channels, in_channels=16, seed=0, params=None):
        self.ch = list(channels)
        self.L = len(self.ch)
        self.cin = in_channels
        self.layers = []  # (name, cin, cout)
        prev = in_channels
        for l, c in enumerate(self.ch):
            self.layers += [(f"enc{l}a", prev, c), (f"enc{l}b", c, c)]
            prev = c
        for l in range(self.L - 2, -1, -1):
            self.layers += [(f"dec{l}a", self.ch[l + 1] + self.ch[l], self.ch[l]), (f"dec{l}b", self.ch[l], self.ch[l])]
        self.offsets = {}
        o = 0
        for name, ci, co in self.layers:
            self.offsets[name] = (o, o + co * 27 * ci, o + co * 27 * ci + co, ci, co)
            o += co * 27 * ci + co
        self.head = (o, o + self.ch[0], o + self.ch[0] + 1)
        self.n_params = o + self.ch[0] + 1
        if params is None:
            rng = np.random.default_rng(seed)
            params = np.zeros(self.n_params)
            for name, ci, co in self.layers:
                w0, w1, b1, _, _ = self.offsets[name]
                params[w0:w1] = rng.normal(0.0, np.sqrt(2.0 / (27 * ci)), w1 - w0)
            params[self.head[0]:self.head[1]] = rng.normal(0.0, np.sqrt(1.0 / self.ch[0]), self.ch[0])
        self.params = np.asarray(params, dtype=np.float64).copy()

    def weight(self, name, bf16):
        w0, w1, b1, ci, co = self.offsets[name]
        Wt = self.params[w0:w1].reshape(co, 27, ci)
        return (round_bf16(Wt) if bf16 else Wt), self.params[w1:b1]

    def forward(self, x, bf16=False):
        """pred [B,D,H,W] and the stored activations."""
        R = round_bf16 if bf16 else (lambda a: a)
        act = {"x0": R(x)}
        xin = act["x0"]
        for l in range(self.L):
            for s in "ab":
                Wt, b = self.weight(f"enc{l}{s}", bf16)
                xin = R(np.maximum(conv3(xin, Wt, b), 0.0))
                act[f"enc{l}{s}"] = xin
            if l < self.L - 1:
                xin = R(avgpool2(xin))
                act[f"x{l + 1}"] = xin
        d = act[f"enc{self.L - 1}b"]
        for l in range(self.L - 2, -1, -1):
            cat = np.concatenate([upsample2(d), act[f"enc{l}b"]], axis=-1)
            act[f"cat{l}"] = cat
            Wt, b = self.weight(f"dec{l}a", bf16)
            d = R(np.maximum(conv3(cat, Wt, b), 0.0))
            act[f"dec{l}a"] = d
            Wt, b = self.weight(f"dec{l}b", bf16)
            d = R(np.maximum(conv3(d, Wt, b), 0.0))
            act[f"dec{l}b"] = d
        h0, h1, h2 = self.head
        final = act["dec0b"] if self.L > 1 else act["enc0b"]
        act["final"] = final
        pred = final @ self.params[h0:h1] + self.params[h1]
        return pred, act

    def gradient(self, x, target, bf16=False):
        """mean |pred - target| and dL/dparams (backward through decoder, then encoder)."""
        R = round_bf16 if bf16 else (lambda a: a)
        pred, act = self.forward(x, bf16)
        n = pred.size
        loss = np.abs(pred - target).mean()
        g = np.zeros(self.n_params)
        dpred = np.sign(pred - target) / n
        h0, h1, h2 = self.head
        final = act["final"]
        g[h0:h1] = np.einsum("bdhw,bdhwc->c", dpred, final)
        g[h1] = dpred.sum()
        dy = R(dpred[..., None] * self.params[h0:h1])

        def layer_back(name, xin, y, dy_):
            w0, w1, b1, ci, co = self.offsets[name]
            Wt, _ = self.weight(name, bf16)
            dz = R(dy_ * (y > 0))
            dx, dW, db = conv3_backward(xin, Wt, dz)
            g[w0:w1] = dW.ravel()
            g[w1:b1] = db
            return R(dx)

        dskip = {}
        # decoder: level 0 first (closest to the head), then towards the bottleneck
        for l in range(0, self.L - 1):
            dy = layer_back(f"dec{l}b", act[f"dec{l}a"], act[f"dec{l}b"], dy)
            dcat = layer_back(f"dec{l}a", act[f"cat{l}"], act[f"dec{l}a"], dy)
            cu = self.ch[l + 1]
            dskip[l] = dcat[..., cu:]
            # gradient of upsample2(d_{l+1}): d_{l+1} is dec(l+1)b, or enc(L-1)b at the bottom
            dy = R(upsample2_backward(dcat[..., :cu]))
        # encoder: bottleneck first
        for l in range(self.L - 1, -1, -1):
            if l < self.L - 1:
                dy = R(dskip[l] + avgpool2_backward(dx_next))
            dy = layer_back(f"enc{l}b", act[f"enc{l}a"], act[f"enc{l}b"], dy)
            xin = act["x0"] if l == 0 else act[f"x{l}"]
            dx_next = layer_back(f"enc{l}a", xin, act[f"enc{l}a"], dy)
            dy = None
        return loss, g, pred


def adam_step(params, grads, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (Kingma & Ba 2015), in place; `step` counts from 1."""
    m *= b1
    m += (1 - b1) * grads
    v *= b2
    v += (1 - b2) * grads * grads
    mhat = m / (1 - b1 ** step)
    vhat = v / (1 - b2 ** step)
    params -= lr * mhat / (np.sqrt(vhat) + eps)
    return params
