"""CPU tests of the engine library: it builds, loads and exports every symbol
include/dxmcg.h declares; its host-side FP64 physics, spectra and beam geometry
agree with the oracle; it refuses bad input before touching a device."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from opendxmc_gb300 import phantoms as P

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    text = (ROOT / "include" / "dxmcg.h").read_text()
    return sorted(set(re.findall(r"DXMCG_API[^;]*?\b(dxmcg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(engine):
    from opendxmc_gb300 import native

    lib = native.lib()
    names = declared_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(native.EXPORTED) == names
    assert lib.dxmcg_version() == 1


def test_library_exports_nothing_else(engine):
    import subprocess

    from opendxmc_gb300 import native

    out = subprocess.run(["nm", "-D", "--defined-only", str(native.LIB_PATH)], capture_output=True, text=True).stdout
    ours = sorted({l.split()[-1] for l in out.splitlines() if " T dxmcg_" in l})
    assert ours == declared_functions()


@pytest.mark.parametrize("zw", [P.WATER, P.BONE, P.LUNG, P.AIR, P.ADIPOSE, {53: 1.0}, {74: 1.0}])
@pytest.mark.parametrize("correction", [0, 1, 2])
def test_host_attenuation_matches_oracle(engine, oracle, zw, correction):
    E = np.concatenate([oracle.energy_grid(), [1.3, 33.17, 69.6, 149.9]])
    a = oracle.attenuation(zw, E, correction)
    b = engine.attenuation(zw, E, correction)
    for x, y in zip(a, b):
        np.testing.assert_allclose(y, x, rtol=1e-13, atol=0)


@pytest.mark.parametrize("kvp,filters", [(70.0, {13: 2.5}), (120.0, {13: 6.0}), (140.0, {13: 3.0, 29: 0.1}),
                                         (80.0, {13: 9.0, 50: 0.4}), (150.0, {})])
def test_tube_matches_oracle(engine, oracle, kvp, filters):
    e1, w1 = oracle.tube_spectrum(kvp, filters)
    e2, w2 = engine.tube_spectrum(kvp, filters)
    np.testing.assert_array_equal(e1, e2)
    np.testing.assert_allclose(w2, w1, rtol=1e-13, atol=1e-300)
    assert engine.tube_mean_energy(kvp, filters) == pytest.approx(oracle.tube_mean_energy(kvp, filters), rel=1e-13)
    assert engine.tube_al_hvl(kvp, filters) == pytest.approx(oracle.tube_al_hvl_mm(kvp, filters), rel=1e-12)


BEAMS = {
    "dx": P.dx_beam_params(particles=10, exposures=4),
    "ct_spiral": P.ct_spiral_params(particles=10),
    "ct_spiral_aec": dict(P.ct_spiral_params(particles=10, pitch=0.8, collimation_cm=8.0),
                          aec=([0, 0, -10], [0, 0, 10], [1.0, 2.0, 0.5, 1.5])),
    "ct_sequential": {"type": 2, "kvp": 120.0, "filters": {13: 6.0}, "particles_per_exposure": 10,
                      "position": [0, 0, -3.0], "step_angle_deg": 10.0, "collimation_cm": 3.84, "scan_fov_cm": 50.0,
                      "sdd_cm": 119.0, "n_slices": 3, "slice_spacing_cm": 3.84},
    "cbct": {"type": 3, "kvp": 90.0, "filters": {13: 4.0}, "particles_per_exposure": 10, "position": [1.0, 0, 0],
             "rotation_axis": [0, 0, 1], "start_angle_deg": -90.0, "stop_angle_deg": 90.0, "step_angle_deg": 2.0,
             "sdd_cm": 120.0, "half_angles": [0.17, 0.17]},
    "pencil": {"type": 4, "energy_kev": 60.0, "particles_per_exposure": 10, "n_exposures": 2,
               "position": [0, 40, 0], "cosines": [[0, 0, 1], [-1, 0, 0]]},
    "dual_energy": dict(P.ct_spiral_params(particles=10), type=5, kvp_b=140.0, filters_b={13: 6.0, 50: 0.4},
                        tube_a_weight=0.4, fov_b_cm=33.0),
    "ct_spiral_organ_aec": dict(P.ct_spiral_params(particles=10), organ_aec=1, organ_aec_start_deg=300.0,
                                organ_aec_stop_deg=60.0, organ_aec_ramp_deg=20.0, organ_aec_low_weight=0.4,
                                organ_aec_compensate=1),
    "cbct_organ_aec": {"type": 3, "kvp": 90.0, "filters": {13: 4.0}, "particles_per_exposure": 10,
                       "position": [0, 0, 0], "rotation_axis": [0, 0, 1], "start_angle_deg": 0.0,
                       "stop_angle_deg": 358.0, "step_angle_deg": 2.0, "sdd_cm": 120.0, "half_angles": [0.17, 0.17],
                       "organ_aec": 1, "organ_aec_start_deg": 45.0, "organ_aec_stop_deg": 135.0,
                       "organ_aec_ramp_deg": 10.0, "organ_aec_low_weight": 0.2, "organ_aec_compensate": 0},
}


@pytest.mark.parametrize("name", sorted(BEAMS))
def test_exposures_match_oracle(engine, oracle, name):
    a = oracle.beam_exposures(BEAMS[name])
    b = engine.beam_exposures(BEAMS[name])
    assert len(a) == len(b) > 0
    for x, y in zip(a, b):
        for k in ("pos", "c0", "c1", "half"):
            np.testing.assert_allclose(y[k], x[k], rtol=0, atol=1e-12)
        assert y["weight"] == pytest.approx(x["weight"], rel=1e-13)
        assert y["tube"] == x["tube"]


def test_world_create_rejects_bad_input_on_host(engine):
    from opendxmc_gb300 import native as N

    lib = N.lib()
    dims = (C.c_int32 * 3)(4, 4, 4)
    sp = (C.c_double * 3)(0.1, 0.1, 0.1)
    good = (N.Material * 1)(N.Material.from_dict(P.WATER))
    h = C.c_void_p()
    bad_dims = (C.c_int32 * 3)(4, 0, 4)
    assert lib.dxmcg_world_create(bad_dims, sp, good, 1, 1, C.byref(h)) == -1
    bad = N.Material()
    bad.n = 1
    bad.Z[0] = 200
    bad.w[0] = 1.0
    assert lib.dxmcg_world_create(dims, sp, (N.Material * 1)(bad), 1, 1, C.byref(h)) == -1
    assert b"composition" in lib.dxmcg_last_error()
    assert lib.dxmcg_world_create(dims, sp, good, 0, 1, C.byref(h)) == -1
    assert lib.dxmcg_world_create(dims, sp, good, 1, 3, C.byref(h)) == -1


def test_no_device_is_an_error_not_a_fallback(engine):
    if engine.device_count() > 0:
        pytest.skip("a device is visible")
    with pytest.raises(Exception, match="NO_DEVICE"):
        engine.GpuWorld((4, 4, 4), (0.1, 0.1, 0.1), [P.WATER])


def test_batch_and_autotune_reject_bad_arguments_on_host(engine):
    from opendxmc_gb300 import native as N

    lib = N.lib()
    h = C.c_void_p()
    beams = (N.Beam * 1)()
    opts = (N.RunOptions * 1)()
    worlds = (C.c_void_p * 1)()
    assert lib.dxmcg_batch_create(0, worlds, beams, opts, C.byref(h)) == -1
    assert lib.dxmcg_batch_create(1, None, beams, opts, C.byref(h)) == -1
    assert lib.dxmcg_batch_create(1, worlds, beams, opts, None) == -1
    opts[0].tracking = 7
    assert lib.dxmcg_batch_create(1, worlds, beams, opts, C.byref(h)) == -1
    assert b"tracking" in lib.dxmcg_last_error()
    opts[0].tracking = 0
    assert lib.dxmcg_batch_create(1, worlds, beams, opts, C.byref(h)) == -3  # null world: not built
    assert lib.dxmcg_batch_run(None, None) == -1
    lib.dxmcg_batch_destroy(None)
    assert lib.dxmcg_batch_info(None, None, None, None) == -1
    assert lib.dxmcg_autotune(None, beams, opts, 0, None) == -3


def test_batched_job_generator_ranges():
    jobs = P.batched_jobs()
    assert len(jobs) == 64
    for j in jobs:
        assert all(64 <= d <= 320 for d in j["dims"])
        assert all(0.1 <= s <= 0.3 for s in j["spacing"])
        assert 60.0 <= j["kvp"] <= 140.0
        b = j["beam"]
        n_exp = b.get("n_exposures", 91)
        assert 0.9e6 <= b["particles_per_exposure"] * n_exp <= 1e8
    assert {j["beam"]["type"] for j in jobs} == {0, 3}
    from opendxmc_gb300 import engine as G

    assert len(G.beam_exposures(jobs[1]["beam"])) == 91
    ph = P.ellipsoid_phantom((40, 30, 20), (0.2, 0.3, 0.25), seed=4)
    assert ph.density.shape == (20, 30, 40) and ph.density.dtype == np.float32
    assert ph.material.max() <= 5 and (ph.material > 0).mean() > 0.2
    again = P.ellipsoid_phantom((40, 30, 20), (0.2, 0.3, 0.25), seed=4)
    np.testing.assert_array_equal(ph.material, again.material)
    np.testing.assert_array_equal(ph.density, again.density)


def _pencil(energy=55.0, kerma=3.5, particles=40_000, exposures=5):
    return {"type": 4, "energy_kev": energy, "particles_per_exposure": particles, "n_exposures": exposures,
            "position": [0.0, 40.0, 0.0], "cosines": [[0, 0, 1], [-1, 0, 0]], "air_kerma_mgy": kerma}


@pytest.mark.parametrize("beam", [
    _pencil(),
    _pencil(energy=20.0, kerma=0.25, particles=7, exposures=3),
    _pencil(energy=149.5, kerma=100.0),
    dict(P.dx_beam_params(particles=50_000, exposures=4), dap_mgycm2=12.5),
    {"type": 3, "kvp": 90.0, "anode_angle_deg": 12.0, "filters": {13: 4.0}, "particles_per_exposure": 1000,
     "position": [0.0, 0.0, 0.0], "rotation_axis": [0.0, 0.0, 1.0], "start_angle_deg": 0.0,
     "stop_angle_deg": 180.0, "step_angle_deg": 2.0, "sdd_cm": 120.0, "half_angles": [0.2, 0.1],
     "dap_mgycm2": 30.0},
], ids=["pencil55", "pencil20", "pencil149", "dx", "cbct"])
def test_analytic_calibration_factor_matches_oracle(engine, oracle, beam):
    """DX/CBCT (DAP) and pencil (air kerma, PencilBeam::setAirKerma,
    beamsettingsmodel.cpp:675) calibration factors: host arithmetic, no device."""
    n_hist = len(oracle.beam_exposures(beam)) * beam["particles_per_exposure"]
    F_or = oracle.calibration_factor(beam, n_hist)
    F = engine.beam_calibration(beam, 1, engine.run_options(normalize=1))
    assert F == pytest.approx(F_or, rel=1e-12)
    assert F != 1.0
    # normalize off, or no target: no scaling
    assert engine.beam_calibration(beam, 1, engine.run_options(normalize=0)) == 1.0
    key = "air_kerma_mgy" if beam["type"] == 4 else "dap_mgycm2"
    assert engine.beam_calibration(dict(beam, **{key: 0.0})) == 1.0


def test_pencil_calibration_is_kerma_per_history():
    """F = K / (N E (mu_tr/rho)_air(E)): doubling the target doubles F, doubling the
    histories halves it."""
    from opendxmc_gb300 import build

    build.build(verbose_ptxas=False)
    from opendxmc_gb300 import engine as G

    f1 = G.beam_calibration(_pencil(kerma=1.0))
    assert G.beam_calibration(_pencil(kerma=2.0)) == pytest.approx(2 * f1, rel=1e-14)
    assert G.beam_calibration(_pencil(kerma=1.0, particles=80_000)) == pytest.approx(f1 / 2, rel=1e-14)
