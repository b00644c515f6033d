"""Dose calibration (dxmcg_run_options.normalize; the trailing `true` of
transport(world, beam, progress, true), simulationpipeline.cpp:165)."""
import numpy as np
import pytest

from opendxmc_gb300 import phantoms as P
import parity

pytestmark = pytest.mark.gpu

AIR = {7: 75.5, 8: 23.2, 18: 1.3}


def test_dap_calibration_factor_and_scaling(gpu, oracle):
    ph = parity.small_cylinder()
    gw = gpu.GpuWorld(ph.dims, ph.spacing, ph.materials)
    gw.set_data(ph.density, ph.material)
    gw.build()
    beam = dict(P.dx_beam_params(particles=50_000, exposures=4), dap_mgycm2=12.5)
    s0 = gw.run(beam, gpu.run_options(seed=3, normalize=0))
    e0, _, c0 = gw.tally()
    gw.clear()
    s1 = gw.run(beam, gpu.run_options(seed=3, normalize=1))
    e1, _, c1 = gw.tally()
    # F = DAP / (N sum_k p_k E_k (mu_tr/rho)_air), restated from the oracle's physics
    E, w = oracle.tube_spectrum(70.0, {13: 2.5})
    ph_, ic, _ = oracle.attenuation(AIR, E, 1)
    ftr = np.array([oracle.lib().or_kn_energy_transfer_fraction(x) for x in E])
    per = float(np.sum(w * E * (ph_ + ic * ftr))) * 1.602176634e-10
    F = 12.5 / (200_000 * per)
    assert s0["calibration"] == 1.0
    assert s1["calibration"] == pytest.approx(F, rel=1e-12)
    np.testing.assert_array_equal(c0, c1)
    m = e0 > 0
    np.testing.assert_allclose(e1[m] / e0[m], F, rtol=2e-6)


def _ctdi_phantom(diameter=32.0):
    """The phantom the library calibrates on: PMMA cylinder, 15 cm long, 1 mm x 5 mm
    voxels; chamber volumes 1.31 cm across, 10 cm long, centre and 1 cm deep."""
    R = diameter / 2
    sxy, sz = 0.1, 0.5
    nxy = 2 * int(np.ceil((R + 1.0) / sxy))
    nz = 30
    x = (np.arange(nxy) + 0.5) * sxy - 0.5 * nxy * sxy
    z = (np.arange(nz) + 0.5) * sz - 0.5 * nz * sz
    X, Y = np.meshgrid(x, x)
    inside = X ** 2 + Y ** 2 <= R * R
    mat = np.repeat(inside[None].astype(np.uint8), nz, axis=0)
    dens = np.where(mat == 1, 1.19, 0.0012)
    centres = [(0, 0), (0, R - 1), (R - 1, 0), (0, -(R - 1)), (-(R - 1), 0)]
    regions = []
    for cx, cy in centres:
        r2 = (X - cx) ** 2 + (Y - cy) ** 2 <= 0.655 ** 2
        regions.append(np.logical_and(r2[None] & inside[None], (np.abs(z) <= 5.0)[:, None, None]))
    pmma = {1: 8.054, 6: 59.985, 8: 31.961}
    return P.Phantom((nxy, nxy, nz), (sxy, sxy, sz), dens, mat, [AIR, pmma]), regions


def test_ctdi_calibration_reproduces_ctdiw(gpu):
    ph, regions = _ctdi_phantom(32.0)
    gw = gpu.GpuWorld(ph.dims, ph.spacing, ph.materials)
    gw.set_data(ph.density, ph.material)
    gw.build()
    T = 4.0
    beam = {"type": 2, "kvp": 120.0, "filters": {13: 6.0}, "particles_per_exposure": 120_000,
            "position": [0.0, 0.0, 0.0], "step_angle_deg": 5.0, "collimation_cm": T, "scan_fov_cm": 50.0,
            "sdd_cm": 119.0, "n_slices": 1, "bowtie": P.BODY_BOWTIE, "ctdi_w_mgy": 10.0,
            "ctdi_diameter_cm": 32.0}
    st = gw.run(beam, gpu.run_options(seed=21, stream=5, normalize=1))
    assert st["calibration"] > 0
    e, _, _ = gw.tally()
    e = e.reshape(ph.density.shape)
    vol = np.prod(ph.spacing)
    ctdi100 = []
    for r in regions:
        dose = e[r].sum() * 1.602176634e-10 / (ph.density[r].sum() * vol)
        ctdi100.append(dose * 10.0 / T)
    ctdiw = ctdi100[0] / 3 + 2 / 3 * np.mean(ctdi100[1:])
    assert ctdiw == pytest.approx(10.0, rel=0.03)
    assert ctdi100[1] > ctdi100[0]  # periphery above centre in a 32 cm body phantom


def test_ct_spiral_ctdivol_uses_pitch(gpu):
    ph = parity.small_torso()
    gw = gpu.GpuWorld(ph.dims, ph.spacing, ph.materials)
    gw.set_data(ph.density, ph.material)
    gw.build()
    b1 = dict(P.ct_spiral_params(particles=2000, pitch=1.0), ctdi_vol_mgy=10.0)
    b2 = dict(P.ct_spiral_params(particles=2000, pitch=2.0), ctdi_vol_mgy=5.0)
    f1 = gw.run(b1, gpu.run_options(seed=1, normalize=1))["calibration"]
    gw.clear()
    f2 = gw.run(b2, gpu.run_options(seed=1, normalize=1))["calibration"]
    # same CTDIw target (10 mGy x pitch), same photons per rotation: same factor up to calibration noise
    assert f2 == pytest.approx(f1, rel=0.03)
