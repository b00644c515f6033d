"""The denoiser's GPU kernels against the FP64 restatement (oracle/denoiser.py),
which rounds to bfloat16 wherever the GPU stores bf16, so that what is left is the
FP32-vs-FP64 accumulation order: forward predictions, every parameter gradient and
the Adam update; plus the input preparation, patch gathering, training progress
and the world-to-denoised-dose path, all through the C ABI."""
import numpy as np
import pytest

from oracle import denoiser as OD
from opendxmc_gb300 import phantoms as P

pytestmark = pytest.mark.gpu

CH = [16, 16, 32]  # three levels: D, H, W multiples of 4
TOL = 1e-2         # relative L2 error allowed against the bf16-emulating FP64 oracle


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, float) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def make_case(seed, B=2, D=16, H=8, W=12):
    rng = np.random.default_rng(seed)
    x = np.zeros((B, D, H, W, 16))
    x[..., 0] = np.log1p(rng.gamma(1.0, 1.0, (B, D, H, W)))
    x[..., 1] = rng.uniform(0.0, 2.0, (B, D, H, W))
    m = rng.integers(0, 6, (B, D, H, W))
    for k in range(6):
        x[..., 2 + k] = m == k
    x = OD.round_bf16(x)
    t = rng.gamma(2.0, 0.5, (B, D, H, W)).astype(np.float32).astype(np.float64)
    return x, t


@pytest.fixture(scope="module", params=[1, 2], ids=["tcgen05", "mma_sync"])
def case(gpu, torch, request):
    """Both convolution paths: tcgen05 (tensor memory accumulators) and mma.sync."""
    net = OD.UNet(CH, in_channels=16, seed=5)
    net.params = net.params.astype(np.float32).astype(np.float64)  # the GPU's FP32 master copy
    dn = gpu.Denoiser(CH, seed=1, conv_path=request.param)
    dn.set_params(net.params)
    x, t = make_case(7)
    xt = torch.tensor(x, dtype=torch.bfloat16, device="cuda")
    tt = torch.tensor(t, dtype=torch.float32, device="cuda")
    return net, dn, x, t, xt, tt


def test_forward_matches_oracle(case):
    net, dn, x, t, xt, tt = case
    got = dn.forward(xt).cpu().numpy()
    ref, _ = net.forward(x, bf16=True)
    assert got.shape == ref.shape
    assert rel(got, ref) < TOL


def test_gradients_match_oracle(case):
    net, dn, x, t, xt, tt = case
    loss = dn.backward(xt, tt)
    g = dn.grads()
    ref_loss, gref, _ = net.gradient(x, t, bf16=True)
    assert abs(loss / ref_loss - 1) < 1e-4
    for name, (w0, w1, b1, ci, co) in net.offsets.items():
        assert rel(g[w0:w1], gref[w0:w1]) < TOL, name
        assert rel(g[w1:b1], gref[w1:b1]) < TOL, name + " bias"
    h0, h1, h2 = net.head
    assert rel(g[h0:h2], gref[h0:h2]) < TOL


def test_tensor_core_convolutions_match_mma_sync(gpu, torch):
    """The full 16/32/64/128 network on both convolution paths with the same
    parameters: every output-channel tile width (16, 32, 64), partial y and z tiles,
    upsampled-and-concatenated decoder inputs and the input-gradient convolutions
    (up to 192 channels) give the same predictions and gradients up to FP32 summation
    order and the bf16 roundings it moves."""
    ch = (16, 32, 64, 128)
    tc = gpu.Denoiser(ch, seed=4, conv_path=1)
    ms = gpu.Denoiser(ch, seed=4, conv_path=2)
    np.testing.assert_array_equal(tc.get_params(), ms.get_params())
    x, t = make_case(13, B=2, D=24, H=40, W=16)
    xt = torch.tensor(x, dtype=torch.bfloat16, device="cuda")
    tt = torch.tensor(t, dtype=torch.float32, device="cuda")
    p1 = tc.forward(xt).cpu().numpy()
    p2 = ms.forward(xt).cpu().numpy()
    assert rel(p1, p2) < 1e-2
    l1 = tc.backward(xt, tt)
    l2 = ms.backward(xt, tt)
    assert abs(l1 / l2 - 1) < 1e-3
    assert rel(tc.grads(), ms.grads()) < 2e-2


def test_tensor_core_wait_limit_gives_up_and_recovers(gpu, torch):
    """The tcgen05 convolution's hand-over waits between its roles are bounded: with
    a limit of one non-blocking poll they run out, every CTA leaves after its copies
    and MMAs in flight have landed, and the call reports DXMCG_ERR_DEVICE; with the
    default limit restored the same network gives the same predictions as before,
    bit for bit, and trains."""
    from opendxmc_gb300 import native as N

    net = gpu.Denoiser((16, 32, 64), seed=2, conv_path=1)
    x, t = make_case(17, B=1, D=24, H=40, W=16)
    xt = torch.tensor(x, dtype=torch.bfloat16, device="cuda")
    tt = torch.tensor(t, dtype=torch.float32, device="cuda")
    ref = net.forward(xt).cpu().numpy()
    net.set_wait_limit(1)
    with pytest.raises(N.DxmcgError) as err:
        net.backward(xt, tt)  # synchronises and reads the convolutions' status
    assert err.value.code == -5
    net.set_wait_limit(0)
    np.testing.assert_array_equal(net.forward(xt).cpu().numpy(), ref)
    loss = net.backward(xt, tt)
    assert np.isfinite(loss) and loss > 0


def test_tensor_core_persistent_bricks_match_mma_sync(gpu, torch):
    """A volume with more output bricks than SMs at level 0 (1 x 64 x 128 x 64: 512
    bricks of 8 x 16 x 8 for the persistent CTAs, three or four each): the tcgen05
    pipeline alternates its two accumulator sets and waits for the epilogue to free
    them, and it agrees with mma.sync on predictions and every gradient."""
    ch = (16, 32)
    tc = gpu.Denoiser(ch, seed=6, conv_path=1)
    ms = gpu.Denoiser(ch, seed=6, conv_path=2)
    x, t = make_case(17, B=1, D=64, H=128, W=64)
    xt = torch.tensor(x, dtype=torch.bfloat16, device="cuda")
    tt = torch.tensor(t, dtype=torch.float32, device="cuda")
    p1 = tc.forward(xt).cpu().numpy()
    p2 = ms.forward(xt).cpu().numpy()
    assert rel(p1, p2) < 1e-2
    l1 = tc.backward(xt, tt)
    l2 = ms.backward(xt, tt)
    assert abs(l1 / l2 - 1) < 1e-3
    assert rel(tc.grads(), ms.grads()) < 2e-2


def test_adam_step_matches_oracle(gpu, torch):
    x, t = make_case(11, B=1, D=8, H=8, W=8)
    dn = gpu.Denoiser(CH, seed=2)
    p0 = dn.get_params().astype(np.float64)
    dn.backward(torch.tensor(x, dtype=torch.bfloat16, device="cuda"),
                torch.tensor(t, dtype=torch.float32, device="cuda"))
    g = dn.grads().astype(np.float64)
    dn.adam(1e-3)
    got = dn.get_params()
    ref = OD.adam_step(p0.copy(), g, np.zeros_like(g), np.zeros_like(g), 1, 1e-3)
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-8)


def test_training_lowers_the_loss(gpu, torch):
    """Overfit one batch of a smoothing task: the loss must fall to well under half."""
    rng = np.random.default_rng(3)
    B, D = 4, 16
    z, y, xx = np.meshgrid(*[np.linspace(-1, 1, D)] * 3, indexing="ij")
    f = np.stack([np.exp(-((z - rng.uniform(-.5, .5)) ** 2 + (y - rng.uniform(-.5, .5)) ** 2 + xx ** 2) * 3)
                  for _ in range(B)])
    x = np.zeros((B, D, D, D, 16))
    x[..., 0] = np.log1p(np.maximum(f + rng.normal(0, 0.2, f.shape), 0))
    x[..., 1] = 1.0
    x[..., 5] = 1.0
    xt = torch.tensor(x, dtype=torch.bfloat16, device="cuda")
    tt = torch.tensor(f, dtype=torch.float32, device="cuda")
    dn = gpu.Denoiser(CH, seed=4)
    losses = [dn.train_step(xt, tt, 2e-3) for _ in range(80)]
    assert np.isfinite(losses).all()
    assert losses[-1] < 0.5 * losses[0]


def test_prepare_input(gpu, torch):
    rng = np.random.default_rng(5)
    n = (10, 12, 14)
    dose = rng.gamma(1.0, 2.0, n).astype(np.float32)
    dose.flat[:5] = [0.0, -1.0, 1e-30, 3.0e4, 7.5]
    dens = rng.uniform(0, 2, n).astype(np.float32)
    mat = rng.integers(0, 8, n).astype(np.uint8)  # 6 and 7 have no channel
    out = gpu.prepare_input(torch.tensor(dose, device="cuda"), torch.tensor(dens, device="cuda"),
                            torch.tensor(mat, device="cuda"), 2.5).float().cpu().numpy()
    assert out.shape == (*n, 16)
    ref0 = OD.round_bf16(np.log1p(np.maximum(dose, 0).astype(np.float64) / 2.5))
    np.testing.assert_allclose(out[..., 0], ref0, rtol=8e-3, atol=0)  # log1pf: within one bf16 step
    np.testing.assert_array_equal(out[..., 1], OD.round_bf16(dens))
    for k in range(6):
        np.testing.assert_array_equal(out[..., 2 + k], (mat == k).astype(np.float64))
    assert not out[..., 8:].any()


def test_gather_patches(gpu, torch):
    import ctypes as C

    from opendxmc_gb300 import native as N

    rng = np.random.default_rng(8)
    dims = [(10, 9, 8), (6, 7, 12)]
    vols = [torch.tensor(rng.normal(size=(*d, 16)), dtype=torch.bfloat16, device="cuda") for d in dims]
    tgts = [torch.tensor(rng.normal(size=d), dtype=torch.float32, device="cuda") for d in dims]
    ptr_in = torch.tensor([v.data_ptr() for v in vols], dtype=torch.int64, device="cuda")
    ptr_t = torch.tensor([v.data_ptr() for v in tgts], dtype=torch.int64, device="cuda")
    dd = torch.tensor(np.array(dims).ravel(), dtype=torch.int32, device="cuda")
    P_ = 4
    origins = [(0, 0, 0, 0), (1, 2, 3, 8), (0, 6, 5, 4), (1, 4, 4, 10), (5, 0, 0, 0)]  # the last two: partly / fully out
    org = torch.tensor(np.array(origins).ravel(), dtype=torch.int32, device="cuda")
    xb = torch.empty((len(origins), P_, P_, P_, 16), dtype=torch.bfloat16, device="cuda")
    tb = torch.empty((len(origins), P_, P_, P_), dtype=torch.float32, device="cuda")
    N.check(N.lib().dxmcg_denoiser_gather_patches(C.c_void_p(ptr_in.data_ptr()), C.c_void_p(ptr_t.data_ptr()),
                                                  C.c_void_p(dd.data_ptr()), len(dims), C.c_void_p(org.data_ptr()),
                                                  len(origins), P_, C.c_void_p(xb.data_ptr()),
                                                  C.c_void_p(tb.data_ptr()), None))
    torch.cuda.synchronize()
    xs = xb.float().cpu().numpy()
    ts = tb.cpu().numpy()
    for k, (v, z, y, x) in enumerate(origins):
        ref_x = np.zeros((P_, P_, P_, 16))
        ref_t = np.zeros((P_, P_, P_))
        if v < len(dims):
            src = vols[v].float().cpu().numpy()
            st = tgts[v].cpu().numpy()
            D, H, W = dims[v]
            for a in range(P_):
                for b in range(P_):
                    for c in range(P_):
                        if z + a < D and y + b < H and x + c < W:
                            ref_x[a, b, c] = src[z + a, y + b, x + c]
                            ref_t[a, b, c] = st[z + a, y + b, x + c]
        np.testing.assert_array_equal(xs[k], ref_x)
        np.testing.assert_array_equal(ts[k], ref_t)


def test_world_denoise_path(gpu, torch):
    ph = P.ellipsoid_phantom((32, 28, 24), (0.4, 0.4, 0.4), seed=6)
    w = gpu.GpuWorld(ph.dims, ph.spacing, ph.materials, 1)
    w.set_data(ph.density, ph.material)
    w.build()
    w.run(P.dx_beam_params(kvp=90.0, field_cm=12.0, particles=20_000, exposures=10), gpu.run_options(seed=9))
    dn = gpu.Denoiser(CH, seed=3)
    out, scale = dn.denoise_world(w)
    d, _, _ = w.dose()
    rho, mat = w.packed_density()
    sel = rho > 0.2
    assert abs(scale / d[sel].mean() - 1) < 1e-6  # the mean forms toDose / rho in FP32
    # the same through the array path: prepare_input + forward, times the scale
    shape = (ph.dims[2], ph.dims[1], ph.dims[0])
    d_in = np.where(mat == 0, 0.0, d)  # air enters with zero dose
    xin = gpu.prepare_input(torch.tensor(d_in.reshape(shape), dtype=torch.float32, device="cuda"),
                            torch.tensor(rho.reshape(shape), device="cuda"),
                            torch.tensor(mat.reshape(shape), device="cuda"), scale)
    pred = dn.forward(xin[None]).cpu().numpy().ravel()
    assert np.isfinite(out).all()
    np.testing.assert_allclose(out, pred.astype(np.float64) * scale, rtol=2e-2, atol=1e-3 * np.abs(out).max())


def test_world_denoise_sparse_bricks_match_dense(gpu, torch):
    """The world path on tcgen05 computes the last convolution only on bricks holding a
    non-air voxel, the one before only on those and their neighbours, and the level-1
    decoder and the encoders only on the bricks that a tissue brick's outputs depend on
    (the body sits at one end of a long block of air, so bricks of every restricted
    layer are skipped).  Every voxel of a tissue
    brick equals the dense array path (prepare_input + forward); the voxels of the other
    bricks are 0."""
    small = P.ellipsoid_phantom((32, 32, 24), (0.4, 0.4, 0.4), seed=8)
    nx, ny, nz = 192, 64, 48
    oz, oy, ox = 12, 16, 8  # the body sits at one end of a larger block of air
    mat = np.zeros((nz, ny, nx), np.uint8)
    rho = np.full((nz, ny, nx), P.SIX_MATERIALS[0][2], np.float32)
    mat[oz:oz + 24, oy:oy + 32, ox:ox + 32] = np.asarray(small.material).reshape(24, 32, 32)
    rho[oz:oz + 24, oy:oy + 32, ox:ox + 32] = np.asarray(small.density).reshape(24, 32, 32)
    w = gpu.GpuWorld((nx, ny, nz), (0.4, 0.4, 0.4), small.materials, 1)
    w.set_data(rho.ravel(), mat.ravel())
    w.build()
    beam = P.dx_beam_params(kvp=90.0, field_cm=14.0, particles=20_000, exposures=10)
    beam["position"] = [(ox + 16) * 0.4 - nx * 0.4 / 2, 100.0, 0.0]  # over the body (the world is centred)
    w.run(beam, gpu.run_options(seed=11))
    dn = gpu.Denoiser(CH, seed=3, conv_path=1)
    out, scale = dn.denoise_world(w)
    d, _, _ = w.dose()
    rho_w, mat_w = w.packed_density()
    d_in = np.where(mat_w == 0, 0.0, d)
    shape = (nz, ny, nx)
    xin = gpu.prepare_input(torch.tensor(d_in.reshape(shape), dtype=torch.float32, device="cuda"),
                            torch.tensor(rho_w.reshape(shape), device="cuda"),
                            torch.tensor(mat_w.reshape(shape), device="cuda"), scale)
    dense = dn.forward(xin[None]).cpu().numpy().astype(np.float64).reshape(shape) * scale
    out = out.reshape(shape)
    # bricks of 8 (x) x 16 (y) x 8 (z) voxels holding a non-air voxel
    tissue = (mat_w.reshape(shape) != 0).reshape(nz // 8, 8, ny // 16, 16, nx // 8, 8).any(axis=(1, 3, 5))
    in_tissue = np.repeat(np.repeat(np.repeat(tissue, 8, 0), 16, 1), 8, 2)
    assert 0.02 < tissue.mean() < 0.5  # the test skips most bricks
    # the level-0 encoder's set lies within the tissue bricks grown by 3, 2, 3 bricks of
    # 8, 16, 8 voxels along x, y, z (a three-level net reaches 21 voxels at most, its
    # first convolution one more)
    enc = np.zeros_like(tissue)
    for dz in range(-3, 4):
        for dy in range(-2, 3):
            for dx in range(-3, 4):
                src = tissue[max(0, -dz):tissue.shape[0] - max(0, dz), max(0, -dy):tissue.shape[1] - max(0, dy),
                             max(0, -dx):tissue.shape[2] - max(0, dx)]
                enc[max(0, dz):tissue.shape[0] - max(0, -dz), max(0, dy):tissue.shape[1] - max(0, -dy),
                    max(0, dx):tissue.shape[2] - max(0, -dx)] |= src
    assert enc.mean() < 0.5  # the encoder skips bricks too
    assert np.isfinite(out).all()
    np.testing.assert_allclose(out[in_tissue], dense[in_tissue], rtol=1e-3, atol=1e-6 * np.abs(dense).max())
    assert (out[~in_tissue] == 0).all()
    # a second call on the same tally reuses the world-path buffers and brick lists
    # and gives the same map
    again, scale2 = dn.denoise_world(w)
    assert scale2 == pytest.approx(scale, rel=1e-12)
    np.testing.assert_allclose(again.reshape(shape), out, rtol=1e-6, atol=1e-9 * np.abs(out).max())


def test_trained_denoiser_beats_plain_monte_carlo(gpu, torch):
    """What the learned part gains: after a short training on two small torsos, a
    held-out torso's 1e6-history dose, denoised, is far closer to the truth than the
    same run without the network (unbiased RMS relative error against two
    independent 1e8-history references, non-air voxels above 10 % of max)."""
    from opendxmc_gb300 import denoise as DN

    out, _ = DN.experiment(torch, dims=(64, 64, 64), spacing=(0.5, 0.5, 0.6), train_seeds=(11, 12),
                           eval_seed=99, lows=(1e6,), high=1e8, steps=200, batch=8, patch=32,
                           channels=(16, 32, 64, 128), log=lambda m: None)
    lv = out["levels"][0]
    assert lv["voxels_scored"] > 10_000
    assert lv["low_rms_rel"] > 0.2                       # the plain short run is noisy
    assert lv["denoised_rms_rel"] < 0.5 * lv["low_rms_rel"], lv
    # the same error level costs plain Monte Carlo many more histories
    assert (lv["low_rms_rel"] / lv["denoised_rms_rel"]) ** 2 > 4.0


def _bf16_bits(x):
    return (np.asarray(x, np.float32).view(np.uint32) >> 16).astype(np.uint16)


def test_time_to_target_falls_back_to_plain_monte_carlo(gpu, torch):
    """The seconds-to-target measurement judges every denoised map against two
    independent reference runs: an untrained network's maps miss the target, so the
    pipeline falls back on plain Monte Carlo, which is run (not extrapolated) until its
    own error crosses the target, and whose time is added to the denoised leg's."""
    from opendxmc_gb300 import denoise as DN

    net = gpu.Denoiser((16, 32, 64, 128), seed=0)
    beam_of = lambda n: DN.spiral_beam(n, scan_cm=8.0, collimation_cm=4.0)  # noqa: E731
    out = DN.time_to_target(torch, net, (64, 64, 48), (0.64, 0.64, 0.8), 5, beam_of, high=2e8, target=0.05,
                            lows=(1e6, 3e6), plain_chunk=1e7, log=lambda m: None)
    dn, plain = out["denoised"], out["plain"]
    assert not dn["accepted"] and len(dn["attempts"]) == 2
    assert all(a["rms_rel"] > 0.05 for a in dn["attempts"])
    assert plain["passed"] and plain["rms_rel"] <= 0.05
    assert plain["checks"][-1]["rms_rel"] <= 0.05 < plain["checks"][0]["rms_rel"] or len(plain["checks"]) == 1
    assert dn["fallback_plain_s"] == plain["s"] and dn["s"] > plain["s"]
    # the reference noise floors the literal mean relative error
    assert 0 < out["mean_rel_floor"] < out["reference_rms_rel"]
    assert plain["crossing_histories"] <= plain["histories"]


@pytest.mark.parametrize("n", [16, 32])
def test_tensor_core_probe_is_exact(gpu, n):
    """The tcgen05 interface (shared-memory descriptors, TMEM accumulators, commit to an
    mbarrier, the A-operand collector) on values whose products and sums are exact in
    FP32: the tensor-core result must equal the FP64 product bit for bit."""
    import ctypes as C
    from opendxmc_gb300 import native as N

    rng = np.random.default_rng(n)
    a = rng.integers(-4, 5, (128, 16)) / 4.0
    b0 = rng.integers(-4, 5, (n, 16)) / 4.0
    b1 = rng.integers(-4, 5, (n, 16)) / 4.0
    A, B0, B1 = (np.ascontiguousarray(_bf16_bits(v)) for v in (a, b0, b1))
    d0 = np.zeros((128, n), np.float32)
    d1 = np.zeros((128, n), np.float32)
    N.check(N.lib().dxmcg_umma_probe(n, A.ctypes.data, B0.ctypes.data, B1.ctypes.data, d0.ctypes.data,
                                     d1.ctypes.data))
    np.testing.assert_array_equal(d1, a @ b1.T)
    np.testing.assert_array_equal(d0, a @ (b0 + b1).T)


def test_world_denoise_sparse_matches_dense_at_full_size(gpu, torch):
    """The 512 x 512 x 400 spiral-CT torso (102,400 level-0 bricks, so the ordered
    brick lists are built over 25 passes of 4096 bricks; the four-level net's
    encoders run on 63 %, 67 % and 72 % of the level-0, -1 and -2 bricks, its level-1
    and level-2 decoders on 44 % and 53-56 %):
    the sparse world path equals the dense array path on every voxel of a tissue
    brick."""
    from opendxmc_gb300 import denoise as DN

    dims, spacing = (512, 512, 400), (0.08, 0.08, 0.1)
    ph = P.torso_phantom(dims=dims, spacing=spacing, seed=99)
    w = gpu.GpuWorld(dims, spacing, [c for _, c, _ in P.SIX_MATERIALS])
    w.set_data(ph.density, ph.material)
    w.build()
    w.run(DN.spiral_beam(1e7), gpu.run_options(seed=5))
    dn = gpu.Denoiser((16, 32, 64, 128), seed=2)
    out, scale = dn.denoise_world(w)
    d, _, _ = w.dose()
    rho, mat = w.packed_density()
    shape = (400, 512, 512)
    xin = gpu.prepare_input(torch.tensor(np.where(mat == 0, 0.0, d).reshape(shape), dtype=torch.float32,
                                         device="cuda"),
                            torch.tensor(rho.reshape(shape), device="cuda"),
                            torch.tensor(mat.reshape(shape), device="cuda"), scale)
    dense = dn.forward(xin[None]).cpu().numpy().reshape(shape).astype(np.float64) * scale
    del xin
    tissue = (mat.reshape(shape) != 0).reshape(50, 8, 32, 16, 64, 8).any(axis=(1, 3, 5))
    in_tissue = np.repeat(np.repeat(np.repeat(tissue, 8, 0), 16, 1), 8, 2)
    out = out.reshape(shape)
    assert 0.2 < tissue.mean() < 0.6
    np.testing.assert_allclose(out[in_tissue], dense[in_tissue], rtol=1e-3, atol=1e-6 * np.abs(dense).max())
    assert (out[~in_tissue] == 0).all()
