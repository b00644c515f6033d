"""GPU passes around the transport against the CPU restatement (oracle/pipelines.py):
CT segmentation (bit-exact material and density), the organ dose table (exact
counts, FP64 sums to 1e-12) and the worker's dose readout (bit-exact), through
the C ABI."""
import ctypes as C

import numpy as np
import pytest

from opendxmc_gb300 import native as N
from opendxmc_gb300 import phantoms as P

pytestmark = pytest.mark.gpu

MATS = [(c, d) for _, c, d in P.SEGMENTATION_MATERIALS]


def table_dict(t):
    n = t.n_materials
    return {"hu": list(t.hu)[:n], "separator": list(t.separator)[:n - 1], "attenuation": list(t.attenuation)[:n],
            "water_attenuation": t.water_attenuation, "water_density": t.water_density,
            "air_attenuation": t.air_attenuation, "air_density": t.air_density}


def hu_volume(n, seed):
    """Fractional and integer CT numbers (the integer ones in [-1024, 3071] take the
    kernel's lookup-table path), including the table's edges and just beyond."""
    rng = np.random.default_rng(seed)
    hu = rng.uniform(-1100.0, 2500.0, n)
    hu[: n // 4] = rng.normal(40.0, 60.0, n // 4)  # soft-tissue-like bulk
    hu[n // 2:] = np.rint(rng.uniform(-1200.0, 3300.0, n - n // 2))
    tail = np.array([-1025.0, -1024.0, 3071.0, 3072.0, -0.0, 0.5])
    k = min(tail.size, n - n // 2)
    hu[n - k:] = tail[:k]
    return hu


@pytest.mark.parametrize("n", [1, 7, 1_000_003])
def test_segment_bit_exact(gpu, n):
    from oracle import pipelines as OP

    t = gpu.ct_segmentation_table(120.0, 2.5, 0.0)
    hu = hu_volume(n, n)
    sep = table_dict(t)["separator"]
    edges = np.array([*sep, *np.nextafter(sep, -np.inf), -1024.0, 3071.0, np.nan, -np.inf, np.inf])
    hu[: min(n, edges.size)] = edges[: min(n, edges.size)]
    m, d = gpu.ct_segment(t, hu)
    rm, rd = OP.ct_segment(table_dict(t), hu)
    np.testing.assert_array_equal(m, rm)
    np.testing.assert_array_equal(d, rd)  # NaN == NaN in assert_array_equal


def test_segment_device_arrays_and_unaligned(gpu):
    """The device-array entry point, once on aligned arrays (vector path) and once
    on views offset by one element (scalar path)."""
    torch = pytest.importorskip("torch")
    from oracle import pipelines as OP

    t = gpu.ct_segmentation_table(90.0, 3.0, 0.2)
    n = 300_001
    hu = hu_volume(n + 1, 5)
    dev = torch.from_numpy(hu).cuda()
    mat = torch.zeros(n + 1, dtype=torch.uint8, device="cuda")
    dens = torch.zeros(n + 1, dtype=torch.float64, device="cuda")
    for off in (0, 1):
        rc = N.lib().dxmcg_ct_segment_device(C.byref(t), dev.data_ptr() + 8 * off, n, mat.data_ptr() + off,
                                             dens.data_ptr() + 8 * off, None)
        N.check(rc)
        torch.cuda.synchronize()
        rm, rd = OP.ct_segment(table_dict(t), hu[off:off + n])
        np.testing.assert_array_equal(mat.cpu().numpy()[off:off + n], rm)
        np.testing.assert_array_equal(dens.cpu().numpy()[off:off + n], rd)


def organ_volume(shape, seed, n_labels=12):
    """Organ labels in blocks (long runs of one label) with a noisy border region."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    blocks = rng.integers(0, n_labels, size=(nz // 4 + 1, ny // 8 + 1, nx // 8 + 1))
    organ = np.kron(blocks, np.ones((4, 8, 8), dtype=np.int64))[:nz, :ny, :nx].astype(np.uint8)
    noisy = rng.random(shape) < 0.05
    organ[noisy] = rng.integers(0, n_labels + 3, size=int(noisy.sum()))  # some labels >= n_organs
    return organ


def test_organ_table_matches_oracle(gpu):
    from oracle import pipelines as OP

    shape = (40, 96, 128)
    rng = np.random.default_rng(3)
    organ = organ_volume(shape, 3)
    dose = rng.gamma(2.0, 1.5, shape)
    dens = rng.uniform(0.001, 1.9, shape)
    sp = (0.12, 0.12, 0.25)
    got = gpu.organ_dose_table(organ, dose, dens, sp, 12)
    ref = OP.organ_dose_table(organ, dose, dens, sp, 12)
    np.testing.assert_array_equal(got["n_voxels"], ref["n_voxels"])
    for k in ("volume_cm3", "mass_g", "dose"):
        np.testing.assert_allclose(got[k], ref[k], rtol=1e-12, atol=0)


@pytest.fixture(scope="module")
def dosed_world(gpu):
    ph = P.ellipsoid_phantom((48, 40, 32), (0.3, 0.3, 0.3), seed=11)
    w = gpu.GpuWorld(ph.dims, ph.spacing, ph.materials, 1)
    w.set_data(ph.density, ph.material)
    w.build()
    beam = P.dx_beam_params(kvp=90.0, field_cm=10.0, particles=30_000, exposures=10)
    return ph, w, beam


def test_world_organ_dose_matches_array_table(gpu, dosed_world):
    ph, w, beam = dosed_world
    w.clear()
    w.run(beam, gpu.run_options(seed=3))
    organ = organ_volume(ph.material.shape, 8, 10)
    d, _, _ = w.dose()
    rho, mat = w.packed_density()
    for air in (False, True):
        dd = np.where((mat == 0) & air, 0.0, d)
        got = w.organ_dose(organ, 10, delete_air_dose=air)
        ref = gpu.organ_dose_table(organ, dd, rho.astype(np.float64), ph.spacing, 10)
        np.testing.assert_array_equal(got["n_voxels"], ref["n_voxels"])
        for k in ("volume_cm3", "mass_g", "dose"):
            np.testing.assert_allclose(got[k], ref[k], rtol=1e-12, atol=0)
        assert got["dose"].max() > 0


@pytest.mark.parametrize("dap", [0.0, 1e7])
def test_postprocessed_readout_bit_exact(gpu, dosed_world, dap):
    """Both sides of the uGy switch: the raw beam (max dose < 1 mGy) and one
    calibrated to a large DAP (max dose > 1 mGy)."""
    from oracle import pipelines as OP

    ph, w, beam = dosed_world
    w.clear()
    b = dict(beam, dap_mgycm2=dap)
    w.run(b, gpu.run_options(seed=4, normalize=1 if dap else 0))
    d, v, c = w.dose()
    _, mat = w.packed_density()
    for air in (True, False):
        got = w.dose_postprocessed(delete_air_dose=air)
        ref = OP.dose_postprocess(d, v, c.astype(np.float64), mat, delete_air_dose=air)
        assert got[3] == ref[3]
        assert got[3] == (dap == 0.0)
        for g, r in zip(got[:3], ref[:3]):
            np.testing.assert_array_equal(g, r)
