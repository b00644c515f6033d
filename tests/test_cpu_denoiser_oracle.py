"""The denoiser's CPU restatement (oracle/denoiser.py) pinned by finite differences:
its analytic gradient matches central differences of its own loss along random
directions, and its bf16 rounding matches IEEE round-to-nearest-even.  On the same
restatement, the brick sets of the world path's restricted layers are checked to
keep the tissue bricks' outputs exact whatever the other bricks hold."""
import numpy as np
import pytest

from oracle import denoiser as D


def test_gradient_matches_finite_differences():
    net = D.UNet([2, 3, 4], in_channels=3, seed=1)
    rng = np.random.default_rng(0)
    x = rng.normal(size=(2, 8, 8, 8, 3))
    t = rng.normal(size=(2, 8, 8, 8))
    loss, g, _ = net.gradient(x, t)
    assert loss > 0
    p0 = net.params.copy()
    for _ in range(4):
        u = rng.normal(size=net.n_params)
        eps = 1e-6
        net.params = p0 + eps * u
        lp = np.abs(net.forward(x)[0] - t).mean()
        net.params = p0 - eps * u
        lm = np.abs(net.forward(x)[0] - t).mean()
        net.params = p0
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g @ u) <= 1e-6 * max(1.0, abs(fd))


def test_single_level_network_and_adam():
    net = D.UNet([2], in_channels=2, seed=3)
    rng = np.random.default_rng(1)
    x = rng.normal(size=(1, 4, 4, 4, 2))
    t = rng.normal(size=(1, 4, 4, 4))
    loss0, g, _ = net.gradient(x, t)
    m = np.zeros_like(g)
    v = np.zeros_like(g)
    for step in range(1, 30):
        loss, g, _ = net.gradient(x, t)
        D.adam_step(net.params, g, m, v, step, 1e-2)
    assert loss < loss0


def test_round_bf16():
    vals = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e38, 1e-40], dtype=np.float32)
    r = D.round_bf16(vals)
    assert r[0] == 1.0
    assert r[1] == 1.0  # halfway between 1 and 1 + 2^-7: ties to even
    assert r[2] == 1.0078125
    assert r[3] == -2.5
    assert np.isfinite(r[4])


# ---- the world path's brick sets (csrc/denoiser.cpp: networkSpan, brickRanges) ----
# Restated here to check the exactness argument on the CPU: along each axis, the
# outputs of a level-0 brick depend on the outputs of each layer only within a span
# found by following the brick's interval back through every path of the network;
# a layer computed only on the bricks of its grid that some tissue brick's span
# reaches gives the tissue bricks exactly the dense outputs, whatever the other
# bricks hold.

def _encoder_needs(l, kind, level, s, acc):
    if kind != "enc" or l < level:
        return
    if l == level:
        acc[0], acc[1] = min(acc[0], s[0]), max(acc[1], s[1])
        return
    x = (s[0] - 2, s[1] + 2)
    _encoder_needs(l - 1, kind, level, (2 * x[0], 2 * x[1] + 1), acc)


def _decoder_needs(L, l, kind, level, s, acc):
    if l == level and kind in ("decb", "deca"):
        w = 0 if kind == "decb" else 1
        acc[0], acc[1] = min(acc[0], s[0] - w), max(acc[1], s[1] + w)
    i = (s[0] - 2, s[1] + 2)
    _encoder_needs(l, kind, level, i, acc)
    up = (i[0] // 2, i[1] // 2)
    if l + 1 == L - 1:
        _encoder_needs(L - 1, kind, level, up, acc)
    else:
        _decoder_needs(L, l + 1, kind, level, up, acc)


def _brick_set(tissue, L, kind, level, dims, b0, bl):
    """Bricks (z, y, x) of a layer's grid (bl voxels per brick along z, y, x) that the
    tissue bricks (b0 voxels per brick) need."""
    ranges = []
    for a in range(3):
        n0, diml = tissue.shape[a], dims[a] >> level
        nl = -(-diml // bl[a])
        r = np.zeros((nl, n0), bool)
        for c in range(n0):
            acc = [10 ** 9, -10 ** 9]
            for p in range(c * b0[a], min((c + 1) * b0[a], dims[a])):
                _decoder_needs(L, 0, kind, level, (p, p), acc)
            lo, hi = (acc[0] - 1, acc[1] + 1) if kind == "enc" else tuple(acc)
            lo, hi = max(0, lo), min(diml - 1, hi)
            if lo <= hi:
                r[lo // bl[a]:hi // bl[a] + 1, c] = True
        ranges.append(r)
    rz, ry, rx = ranges
    t = np.einsum("zyx,Xx->zyX", tissue.astype(int), rx.astype(int)) > 0
    t = np.einsum("zyX,Yy->zYX", t.astype(int), ry.astype(int)) > 0
    return np.einsum("zYX,Zz->ZYX", t.astype(int), rz.astype(int)) > 0


def _voxel_mask(bricks, bl, shape):
    m = bricks.repeat(bl[0], 0).repeat(bl[1], 1).repeat(bl[2], 2)
    return m[:shape[0], :shape[1], :shape[2]]


@pytest.mark.parametrize("granularity", ["bricks", "voxels"])
def test_world_path_brick_sets_keep_tissue_bricks_exact(granularity):
    """A four-level net on a grid with the body at one end of a long block of air:
    every layer the world path restricts (the encoders of levels 0-2, the decoders of
    levels 1-2, the last two convolutions) gets large random values outside its brick
    set, and the prediction on every voxel of a tissue brick is still the dense one.
    With the library's bricks, and with one-voxel bricks, where every span must be
    exact to the voxel."""
    L = 4
    net = D.UNet([2, 2, 2, 2], in_channels=2, seed=4)
    dims = (32, 32, 192)  # z, y, x
    rng = np.random.default_rng(1)
    x = rng.normal(size=(1, *dims, 2))
    tissue_vox = np.zeros(dims, bool)
    tissue_vox[9:20, 5:27, 3:29] = True
    if granularity == "bricks":
        b0 = (8, 16, 8)  # level-0 bricks of the 16-channel layers: z, y, x
        tissue = tissue_vox.reshape(4, 8, 2, 16, 24, 8).any(axis=(1, 3, 5))
        grid = {0: (8, 16, 8), 1: (8, 16, 8), 2: (4, 16, 8)}  # z, y, x per level
    else:
        b0, tissue = (1, 1, 1), tissue_vox
        grid = {0: (1, 1, 1), 1: (1, 1, 1), 2: (1, 1, 1)}
    sets = {f"enc{l}": _brick_set(tissue, L, "enc", l, dims, b0, grid[l]) for l in range(3)}
    for l in (1, 2):
        sets[f"dec{l}b"] = _brick_set(tissue, L, "decb", l, dims, b0, grid[l])
        sets[f"dec{l}a"] = _brick_set(tissue, L, "deca", l, dims, b0, grid[l])
    grown = np.zeros_like(tissue)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                grown |= np.roll(np.roll(np.roll(tissue, dz, 0), dy, 1), dx, 2) & np.pad(
                    np.ones((tissue.shape[0] - abs(dz), tissue.shape[1] - abs(dy), tissue.shape[2] - abs(dx)), bool),
                    ((max(dz, 0), max(-dz, 0)), (max(dy, 0), max(-dy, 0)), (max(dx, 0), max(-dx, 0))))
    sets["dec0a"], sets["dec0b"] = grown, tissue
    for name, s in sets.items():
        assert 0 < s.mean() < 1, name  # every set leaves bricks out

    def spoil(a, name, level):
        grid_l = grid[level]
        keep = _voxel_mask(sets[name], grid_l, a.shape[1:4])
        noise = 1e3 * rng.normal(size=a.shape)
        return np.where(keep[None, ..., None], a, noise)

    def forward(restricted):
        xin = x
        act = {}
        for l in range(L):
            for s in "ab":
                Wt, b = net.weight(f"enc{l}{s}", False)
                xin = np.maximum(D.conv3(xin, Wt, b), 0.0)
                if restricted and l < 3:
                    xin = spoil(xin, f"enc{l}", l)
            act[l] = xin
            if l < L - 1:
                xin = D.avgpool2(xin)
        d = act[L - 1]
        for l in range(L - 2, -1, -1):
            cat = np.concatenate([D.upsample2(d), act[l]], axis=-1)
            for s, src in (("a", cat), ("b", None)):
                Wt, b = net.weight(f"dec{l}{s}", False)
                d = np.maximum(D.conv3(cat if s == "a" else d, Wt, b), 0.0)
                if restricted:
                    d = spoil(d, f"dec{l}{s}", l)
        h0, h1, h2 = net.head
        return d @ net.params[h0:h1] + net.params[h1]

    dense = forward(False)[0]
    sparse = forward(True)[0]
    inside = _voxel_mask(tissue, b0, dims)
    np.testing.assert_array_equal(sparse[inside], dense[inside])
    assert not np.allclose(sparse[~inside], dense[~inside])  # the garbage is real
