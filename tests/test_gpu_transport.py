"""GPU transport parity against the CPU oracle, through the C ABI.

Two kinds of comparison:
  * independent streams (different stream numbers): per-voxel energy
    imparted within 3 combined standard errors in >= 99 % of voxels above 5 % of
    the maximum; total energy within 4 standard errors of the difference (the
    spread of 32 replicate GPU runs of the beam), at history counts where that is
    at most 0.3 %;
  * shared streams (same seed and stream): the GPU (FP32 tracking) and the
    oracle (FP64) draw the same uniforms per history, so totals agree far more
    tightly; what is left is FP32 vs FP64 rounding flipping a few decisions.
"""
import threading
import time

import numpy as np
import pytest

from opendxmc_gb300 import phantoms as P
import parity

pytestmark = pytest.mark.gpu


def gpu_world(gpu, ph, correction=1):
    w = gpu.GpuWorld(ph.dims, ph.spacing, ph.materials, correction)
    w.set_data(ph.density, ph.material)
    w.build()
    return w


def oracle_world_on_packed(oracle, gw, ph, correction=1):
    """Oracle world fed the densities exactly as the device stores them."""
    d, m = gw.packed_density()
    np.testing.assert_array_equal(m, ph.material.ravel())
    ref = ph.density.ravel()
    pos = ref > 0
    assert np.all(d[~pos] == 0)
    assert np.max(np.abs(d[pos].astype(np.float64) / ref[pos] - 1), initial=0.0) <= 2.0 ** -16
    return oracle.World(ph.dims, ph.spacing, d.astype(np.float64), ph.material, ph.materials, correction)


def compare(gw, ow, n_hist):
    e1, q1, c1 = gw.tally()
    e2, q2, c2 = ow.tally()
    frac, nvox = parity.combined_sigma_agreement(e1, parity.tally_variance(e1, q1, n_hist), e2,
                                                 parity.tally_variance(e2, q2, n_hist))
    return frac, nvox, e1, e2


@pytest.fixture(scope="module")
def c1(gpu, oracle):
    """Water cylinder with bone insert, 128x128x64 at 1 x 1 x 2.5 mm, DX 70 kVp."""
    ph = P.water_cylinder_phantom()
    gw = gpu_world(gpu, ph)
    ow = oracle_world_on_packed(oracle, gw, ph)
    return ph, gw, ow


def test_c1_dx_independent_streams(c1, gpu):
    ph, gw, ow = c1
    gw.clear()
    ow.clear()
    beam = P.dx_beam_params(particles=1_000_000, exposures=10)  # 1e7 histories from seed 1
    sg = gw.run(beam, gpu.run_options(seed=1, stream=0))
    so = ow.run(beam, seed=1, stream=1)
    assert sg["n_histories"] == so["n_histories"] == 10_000_000
    assert sg["n_errors"] == 0
    frac, nvox, e1, e2 = compare(gw, ow, 10_000_000)
    assert nvox > 10000
    assert frac >= 0.99, frac
    tol = parity.total_tolerance(gw, beam, lambda r: gpu.run_options(seed=100 + r, stream=0))
    parity.assert_totals_agree(e1, e2, tol, "C1 DX")


def test_c1_dx_shared_streams(c1, gpu):
    ph, gw, ow = c1
    gw.clear()
    ow.clear()
    beam = P.dx_beam_params(particles=200_000, exposures=10)
    sg = gw.run(beam, gpu.run_options(seed=7, stream=2))
    so = ow.run(beam, seed=7, stream=2)
    for k in ("n_histories", "n_missed"):
        assert sg[k] == so[k]
    # decisions agree except where FP32 and FP64 round a comparison differently
    for k in ("n_photo", "n_compton", "n_rayleigh", "n_interacted"):
        assert sg[k] == pytest.approx(so[k], rel=2e-3), k
    e1, _, c1_ = gw.tally()
    e2, _, c2 = ow.tally()
    assert e1.sum() == pytest.approx(e2.sum(), rel=2e-3)
    assert np.mean(c1_ == c2) > 0.99


def test_level2_impulse_approximation_and_fluorescence(gpu, oracle):
    """Correction level 2 (Doppler-broadened Compton, K fluorescence) on the
    cylinder with its bone insert: shared streams give the oracle's totals and event
    counts; independent streams agree voxel by voxel; energy is conserved."""
    ph = parity.small_cylinder()
    gw = gpu_world(gpu, ph, correction=2)
    ow = oracle_world_on_packed(oracle, gw, ph, correction=2)
    beam = P.dx_beam_params(particles=100_000, exposures=10)
    sg = gw.run(beam, gpu.run_options(seed=5, stream=3))
    so = ow.run(beam, seed=5, stream=3)
    assert sg["n_errors"] == 0 and sg["n_histories"] == so["n_histories"] == 1_000_000
    assert sg["n_fluorescence"] > 0
    for k in ("n_photo", "n_compton", "n_rayleigh", "n_fluorescence"):
        assert sg[k] == pytest.approx(so[k], rel=5e-3), k
    e1, _, _ = gw.tally()
    e2, _, _ = ow.tally()
    assert e1.sum() == pytest.approx(e2.sum(), rel=2e-3)
    assert e1.sum() + sg["e_escaped"] == pytest.approx(sg["e_source"], rel=1e-5)
    # independent streams, 7e6 histories
    gw.clear()
    ow.clear()
    beam = P.dx_beam_params(particles=700_000, exposures=10)
    sg = gw.run(beam, gpu.run_options(seed=1, stream=0))
    ow.run(beam, seed=1, stream=1)
    frac, nvox, e1, e2 = compare(gw, ow, sg["n_histories"])
    assert nvox > 1000 and frac >= 0.99, frac
    tol = parity.total_tolerance(gw, beam, lambda r: gpu.run_options(seed=100 + r, stream=0))
    parity.assert_totals_agree(e1, e2, tol, "level 2")


@pytest.mark.parametrize("steps", [2, 5])
def test_woodcock_steps_per_phase_keep_every_history(c1, gpu, steps):
    """Several Woodcock steps per step phase change only when a lane's work runs,
    not what it draws: every history makes the same decisions, so the counts are
    equal and the per-voxel sums equal up to the order of the FP64 atomics."""
    ph, gw, _ = c1
    beam = P.dx_beam_params(particles=100_000, exposures=10)
    gw.clear()
    s1 = gw.run(beam, gpu.run_options(seed=3, stream=1, woodcock_steps=1))
    e1, q1, n1 = gw.tally()
    gw.clear()
    s2 = gw.run(beam, gpu.run_options(seed=3, stream=1, woodcock_steps=steps))
    e2, q2, n2 = gw.tally()
    for k in ("n_histories", "n_visits", "n_photo", "n_compton", "n_rayleigh", "n_cutoff", "n_interacted"):
        assert s1[k] == s2[k], k
    np.testing.assert_array_equal(n1, n2)
    np.testing.assert_allclose(e2, e1, rtol=1e-12, atol=0)
    np.testing.assert_allclose(q2, q1, rtol=1e-12, atol=0)


def test_gather_skip_keeps_every_history(gpu):
    """The Woodcock gather skip settles tentative collisions from the 8^3-voxel cell
    bound without reading the voxel, on the uniform the full test would use: every
    history makes the same decisions, so counts are equal and the per-voxel sums
    equal up to the order of the FP64 atomics, with far fewer voxel reads.  A cell
    holding a transparent voxel takes the full test."""
    ph = P.torso_phantom(dims=(96, 80, 64), spacing=(0.4, 0.4, 0.4), seed=6)
    ph.material[20:30, 30:40, 40:48] = 255  # transparent voxels in a few cells
    gw = gpu_world(gpu, ph)
    beam = P.ct_spiral_params(particles=3000, scan_cm=20.0)
    s_off = gw.run(beam, gpu.run_options(seed=9, stream=1, gather_skip=-1))
    e1, q1, n1 = gw.tally()
    gw.clear()
    s_on = gw.run(beam, gpu.run_options(seed=9, stream=1, gather_skip=1))
    e2, q2, n2 = gw.tally()
    for k in ("n_histories", "n_visits", "n_photo", "n_compton", "n_rayleigh", "n_cutoff", "n_interacted"):
        assert s_off[k] == s_on[k], k
    np.testing.assert_array_equal(n1, n2)
    np.testing.assert_allclose(e2, e1, rtol=1e-12, atol=0)
    np.testing.assert_allclose(q2, q1, rtol=1e-12, atol=0)
    assert s_off["n_voxel_reads"] == s_off["n_visits"] and s_off["n_cell_reads"] == 0
    # tentative collisions outside the two-region box read their voxel without a cell bound
    assert 0 < s_on["n_cell_reads"] <= s_on["n_visits"]
    # the default turns the skip on only for grids whose voxel words exceed 64 MiB
    gw.clear()
    assert gw.run(beam, gpu.run_options(seed=9, stream=1, hist_end=1000))["n_cell_reads"] == 0
    print(f"gather skip: {s_on['n_voxel_reads'] / s_on['n_visits']:.3f} of the tentative collisions read their voxel")
    assert s_on["n_voxel_reads"] < 0.7 * s_on["n_visits"]


def test_two_region_woodcock_matches_plain_woodcock(gpu):
    """Outside the box of non-air voxels, flights step against air's own majorant
    until they reach the box: the transport of plain Woodcock with fewer tentative
    collisions.  Per-voxel energy within 3 combined standard errors and totals of 16
    replicates within 4 standard errors of their difference, against the same kernel
    with one region (two_region = -1); fewer than half the visits."""
    ph = parity.small_torso(scale=2, seed=4)
    gw = gpu_world(gpu, ph)
    beam = P.ct_spiral_params(particles=4000, scan_cm=10.0)
    k = 16
    n = k * len(gpu.beam_exposures(beam)) * beam["particles_per_exposure"]
    one = parity.replicate_totals(gw, beam, lambda r: gpu.run_options(seed=2, stream=300 + r, two_region=-1), k)
    e1, q1, _ = gw.tally()
    v1 = gw.run(beam, gpu.run_options(seed=2, stream=1, two_region=-1, hist_end=200_000))["n_visits"]
    two = parity.replicate_totals(gw, beam, lambda r: gpu.run_options(seed=2, stream=400 + r, two_region=1), k)
    e2, q2, _ = gw.tally()
    v2 = gw.run(beam, gpu.run_options(seed=2, stream=1, two_region=1, hist_end=200_000))["n_visits"]
    frac, nvox = parity.combined_sigma_agreement(e1, parity.tally_variance(e1, q1, n), e2,
                                                 parity.tally_variance(e2, q2, n))
    sigma = np.hypot(parity.total_sigma(one), parity.total_sigma(two))
    print(f"two regions: {v2 / v1:.3f} of the visits, total difference {(two.sum() - one.sum()) / sigma:+.2f} sigma, "
          f"{frac:.4f} of {nvox} voxels within 3 sigma")
    assert nvox > 2000 and frac >= 0.99
    assert abs(two.sum() - one.sum()) <= 4.0 * sigma
    assert v2 < 0.5 * v1
    # the default: two regions, since the torso's box holds less than half the grid
    assert gw.run(beam, gpu.run_options(seed=2, stream=1, hist_end=200_000))["n_visits"] == v2


def test_launch_defaults_adapt_to_the_world(gpu):
    """Steps per phase: 8 on a fresh world, then 1.4 / p (clamped to 4..16) with p the
    stops (real collisions and escapes) per tentative collision of the world's previous
    Woodcock run; an explicit setting wins.  Two regions: on for the torso (its box holds
    less than half the grid), off for the cylinder that fills its grid."""
    ph = parity.small_torso(scale=2, seed=4)
    gw = gpu_world(gpu, ph)
    beam = P.ct_spiral_params(particles=2000, scan_cm=10.0)
    s1 = gw.run(beam, gpu.run_options(seed=3, hist_end=300_000))
    assert s1["woodcock_steps"] == 8 and s1["two_region"] == 1
    p = (s1["n_photo"] + s1["n_compton"] + s1["n_rayleigh"] + s1["n_histories"] - s1["n_missed"]) / s1["n_visits"]
    s2 = gw.run(beam, gpu.run_options(seed=3, hist_end=300_000))
    assert s2["woodcock_steps"] == int(np.clip(np.floor(1.4 / p + 0.5), 4, 16))
    assert gw.run(beam, gpu.run_options(seed=3, hist_end=1000, woodcock_steps=12))["woodcock_steps"] == 12
    assert gw.run(beam, gpu.run_options(seed=3, hist_end=1000, two_region=-1))["two_region"] == 0
    cyl = gpu_world(gpu, parity.small_cylinder())
    assert cyl.run(P.dx_beam_params(particles=1000, exposures=2))["two_region"] == 0


def test_two_region_woodcock_shared_streams_match_oracle(gpu, oracle):
    """Shared streams: the kernel's two-region Woodcock and the oracle's restatement
    (TRACK_WOODCOCK_BOX) draw the same uniforms per history, so counts, visits and the
    total agree closely; what differs is FP32 against FP64 rounding (the box entry,
    the reciprocals, voxel faces)."""
    ph = parity.small_torso(scale=2, seed=4)
    gw = gpu_world(gpu, ph)
    ow = oracle_world_on_packed(oracle, gw, ph)
    beam = P.ct_spiral_params(particles=2000, scan_cm=10.0)
    sg = gw.run(beam, gpu.run_options(seed=6, stream=3, two_region=1))
    so = ow.run(beam, seed=6, stream=3, tracking=oracle.TRACK_WOODCOCK_BOX)
    assert sg["n_errors"] == 0 and sg["n_histories"] == so["n_histories"]
    for k in ("n_visits", "n_photo", "n_compton", "n_rayleigh", "n_interacted"):
        assert sg[k] == pytest.approx(so[k], rel=2e-3), k
    e1, _, c1_ = gw.tally()
    e2, _, c2 = ow.tally()
    assert e1.sum() == pytest.approx(e2.sum(), rel=2e-3)
    assert np.mean(c1_ == c2) > 0.99


def test_energy_conservation(c1, gpu):
    ph, gw, ow = c1
    gw.clear()
    st = gw.run(P.dx_beam_params(particles=100_000, exposures=10), gpu.run_options(seed=3))
    e, _, _ = gw.tally()
    assert st["e_deposited"] == pytest.approx(e.sum(), rel=1e-9)
    assert e.sum() + st["e_escaped"] == pytest.approx(st["e_source"], rel=1e-5)


def test_counts_deterministic_and_shardable(c1, gpu):
    """Event counts are integers: identical across runs, launch shapes, chunking
    and history-range splits (the basis of multi-GPU replicas)."""
    ph, gw, ow = c1
    beam = P.dx_beam_params(particles=50_000, exposures=4)
    gw.clear()
    gw.run(beam, gpu.run_options(seed=5))
    e_a, _, c_a = gw.tally()
    gw.clear()
    gw.run(beam, gpu.run_options(seed=5, block_size=128, blocks_per_sm=3, chunk_log2=14))
    e_b, _, c_b = gw.tally()
    gw.clear()
    gw.run(beam, gpu.run_options(seed=5, hist_begin=0, hist_end=77_777))
    gw.run(beam, gpu.run_options(seed=5, hist_begin=77_777, hist_end=0))
    e_c, _, c_c = gw.tally()
    np.testing.assert_array_equal(c_a, c_b)
    np.testing.assert_array_equal(c_a, c_c)
    np.testing.assert_allclose(e_b, e_a, rtol=1e-9)
    np.testing.assert_allclose(e_c, e_a, rtol=1e-9)


def test_c2_spiral_ct_torso_independent_streams(gpu, oracle):
    ph = P.torso_phantom(seed=1)
    gw = gpu_world(gpu, ph)
    ow = oracle_world_on_packed(oracle, gw, ph)
    beam = P.ct_spiral_params(particles=54_000)  # 360 exposures -> 1.94e7 histories
    sg = gw.run(beam, gpu.run_options(seed=11, stream=0))
    so = ow.run(beam, seed=11, stream=1)
    n = sg["n_histories"]
    assert n == so["n_histories"] == 360 * 54_000
    frac, nvox, e1, e2 = compare(gw, ow, n)
    assert nvox > 2000
    assert frac >= 0.99, frac
    tol = parity.total_tolerance(gw, beam, lambda r: gpu.run_options(seed=100 + r, stream=0))
    parity.assert_totals_agree(e1, e2, tol, "C2 torso")


def test_c5_torso_full_size_conservation(gpu):
    """The 512 x 512 x 400 torso (the voxels and tallies exceed L2): no device error,
    energy conserved, the tally sum equal to the deposited-energy counter, and the
    dose readout finite and non-negative."""
    dims, spacing = (512, 512, 400), (0.08, 0.08, 0.1)
    ph = P.torso_phantom(dims=dims, spacing=spacing, seed=7)
    gw = gpu_world(gpu, ph)
    beam = P.ct_spiral_params(pitch=0.8, collimation_cm=8.0, particles=20_000)
    st = gw.run(beam, gpu.run_options(seed=9))
    assert st["n_errors"] == 0 and st["n_histories"] > 1_000_000
    e, _, _ = gw.tally()
    assert st["e_deposited"] == pytest.approx(e.sum(), rel=1e-9)
    assert e.sum() + st["e_escaped"] == pytest.approx(st["e_source"], rel=1e-5)
    dose, var, cnt = gw.dose()
    assert np.isfinite(dose).all() and (dose >= 0).all() and (var >= 0).all()
    assert cnt.sum() > 0


@pytest.mark.parametrize("cell", [8, 16])
def test_macro_tracking_matches_oracle(c1, gpu, cell):
    """Macro-cell majorants: shared streams follow the oracle's histories; the
    independent-stream estimate agrees within 3 combined standard errors."""
    ph, gw, ow = c1
    ow.set_macro(cell)
    beam = P.dx_beam_params(particles=200_000, exposures=5)
    gw.clear()
    ow.clear()
    sg = gw.run(beam, gpu.run_options(seed=13, stream=6, tracking=2, macro_cell=cell))
    so = ow.run(beam, seed=13, stream=6, tracking=oracle_macro())
    assert sg["n_errors"] == 0 and sg["n_crossings"] > 0
    assert sg["n_visits"] == pytest.approx(so["n_visits"], rel=2e-3)
    assert sg["n_crossings"] == pytest.approx(so["n_crossings"], rel=2e-3)
    for k in ("n_photo", "n_compton", "n_rayleigh", "n_interacted"):
        assert sg[k] == pytest.approx(so[k], rel=2e-3), k
    e1, _, _ = gw.tally()
    e2, _, _ = ow.tally()
    assert e1.sum() == pytest.approx(e2.sum(), rel=2e-3)
    gw.clear()
    ow.clear()
    beam = P.dx_beam_params(particles=800_000, exposures=5)
    sg = gw.run(beam, gpu.run_options(seed=14, stream=0, tracking=2, macro_cell=cell))
    ow.run(beam, seed=14, stream=1, tracking=0)
    frac, nvox, e1, e2 = compare(gw, ow, sg["n_histories"])
    assert nvox > 5000 and frac >= 0.99
    tol = parity.total_tolerance(gw, beam, lambda r: gpu.run_options(seed=100 + r, tracking=2, macro_cell=cell))
    parity.assert_totals_agree(e1, e2, tol, f"macro cells {cell}")


def oracle_macro():
    from oracle import oracle as O

    return O.TRACK_MACRO


def test_macro_tracking_c2_torso(gpu, oracle):
    ph = P.torso_phantom(seed=2)
    gw = gpu_world(gpu, ph)
    ow = oracle_world_on_packed(oracle, gw, ph)
    beam = P.ct_spiral_params(particles=67_000)  # 2.4e7 histories
    sg = gw.run(beam, gpu.run_options(seed=3, stream=0, tracking=2))
    ow.run(beam, seed=3, stream=1)
    assert sg["n_visits"] < 0.4 * 20.5 * sg["n_histories"]  # far fewer voxel lookups than global Woodcock
    frac, nvox, e1, e2 = compare(gw, ow, sg["n_histories"])
    assert nvox > 2000 and frac >= 0.99
    tol = parity.total_tolerance(gw, beam, lambda r: gpu.run_options(seed=100 + r, tracking=2))
    parity.assert_totals_agree(e1, e2, tol, "macro cells, C2 torso")


def test_siddon_tracking_matches_woodcock(gpu):
    """Regular tracking with exact path lengths and Woodcock tracking sample the same
    transport: per-voxel energy within 3 combined standard errors, and total energy
    within 4 standard errors of the difference, estimated from eight independent
    replicates of the beam with each method (at a few 1e5 histories a total scatters
    by a few 0.1 %, so a fixed relative tolerance would be a coin toss)."""
    ph = parity.small_torso(scale=2)
    gw = gpu_world(gpu, ph)
    beam = P.ct_spiral_params(particles=2000, scan_cm=10.0)
    k = 8
    n = k * len(gpu.beam_exposures(beam)) * beam["particles_per_exposure"]
    tw = parity.replicate_totals(gw, beam, lambda r: gpu.run_options(seed=1, stream=100 + r, tracking=0), k)
    e1, q1, _ = gw.tally()
    ts = parity.replicate_totals(gw, beam, lambda r: gpu.run_options(seed=1, stream=200 + r, tracking=1), k)
    e2, q2, _ = gw.tally()
    frac, nvox = parity.combined_sigma_agreement(e1, parity.tally_variance(e1, q1, n), e2,
                                                 parity.tally_variance(e2, q2, n))
    assert nvox > 500 and frac >= 0.99
    sigma = np.hypot(parity.total_sigma(tw), parity.total_sigma(ts))
    print(f"Woodcock - Siddon total: {tw.sum() - ts.sum():+.4g} keV, {(tw.sum() - ts.sum()) / sigma:+.2f} sigma "
          f"({sigma / ts.sum():.2e} relative)")
    assert abs(tw.sum() - ts.sum()) <= 4.0 * sigma
    gw.clear()
    s1 = gw.run(beam, gpu.run_options(seed=1, tracking=0, hist_end=100_000))
    s2 = gw.run(beam, gpu.run_options(seed=1, stream=9, tracking=1, hist_end=100_000))
    assert s2["n_visits"] > s1["n_visits"]  # exact stepping visits every voxel on the path


def test_siddon_tracking_matches_oracle(gpu, oracle):
    ph = parity.small_cylinder()
    gw = gpu_world(gpu, ph)
    ow = oracle_world_on_packed(oracle, gw, ph)
    beam = P.dx_beam_params(particles=850_000, exposures=4)
    sg = gw.run(beam, gpu.run_options(seed=2, stream=0, tracking=1))
    ow.run(beam, seed=2, stream=1, tracking=oracle.TRACK_SIDDON)
    frac, nvox, e1, e2 = compare(gw, ow, sg["n_histories"])
    assert nvox > 500 and frac >= 0.99
    tol = parity.total_tolerance(gw, beam, lambda r: gpu.run_options(seed=100 + r, tracking=1))
    parity.assert_totals_agree(e1, e2, tol, "Siddon")


def test_beer_lambert_transmission(gpu, oracle):
    dims = (4, 40, 4)
    ph = P.Phantom(dims, (0.25, 0.25, 0.25), np.ones(dims[::-1]), np.zeros(dims[::-1], np.uint8), [P.WATER])
    gw = gpu_world(gpu, ph)
    n = 1_000_000
    beam = {"type": 4, "energy_kev": 60.0, "particles_per_exposure": n, "n_exposures": 1,
            "position": [0.0, 50.0, 0.0], "cosines": [[0, 0, 1], [-1, 0, 0]]}
    st = gw.run(beam)
    xs, _ = gw.tables(0)
    mu = float(xs[(60 - 1) * 2, 3])  # 60 keV is a grid node
    trans = np.exp(-mu * 10.0)
    measured = 1.0 - st["n_interacted"] / n
    assert measured == pytest.approx(trans, abs=5 * np.sqrt(trans * (1 - trans) / n))


def test_device_tables_match_oracle(gpu, oracle):
    ph = parity.small_torso()
    gw = gpu_world(gpu, ph)
    ow = oracle_world_on_packed(oracle, gw, ph)
    for m in range(len(ph.materials)):
        xs, maj = gw.tables(m)
        p, ic, co = ow.table(m)
        np.testing.assert_allclose(xs[:, 0], p, rtol=1e-6)
        np.testing.assert_allclose(xs[:, 1], ic, rtol=1e-6)
        np.testing.assert_allclose(xs[:, 2], co, rtol=1e-6)
    np.testing.assert_allclose(maj, ow.majorant(), rtol=1e-6)


def test_dose_readout(c1, gpu):
    ph, gw, ow = c1
    gw.clear()
    st = gw.run(P.dx_beam_params(particles=20_000, exposures=5))
    e, e2, c = gw.tally()
    d, v, c2 = gw.dose()
    np.testing.assert_array_equal(c, c2)
    rho, _ = gw.packed_density()
    vol = np.prod(ph.spacing)
    scale = st["dose_scale"]
    assert scale == pytest.approx(1.602176634e-10 / vol)
    np.testing.assert_allclose(d, e * scale / rho.astype(np.float64), rtol=1e-12)
    var = np.maximum(e2 - e * e / st["n_histories"], 0) * (scale / rho.astype(np.float64)) ** 2
    np.testing.assert_allclose(v, var, rtol=1e-9, atol=1e-300)
    # pinned host arrays take the direct path (the kernel writes them over the host
    # link), device arrays too; both give the staged result exactly
    import torch

    pinned = (torch.zeros(gw.N, dtype=torch.float64, pin_memory=True).numpy(),
              torch.zeros(gw.N, dtype=torch.float64, pin_memory=True).numpy(),
              torch.zeros(gw.N, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64))
    dp, vp, cp = gw.dose(out=pinned)
    np.testing.assert_array_equal(dp, d)
    np.testing.assert_array_equal(vp, v)
    np.testing.assert_array_equal(cp, c2)
    dev = [torch.zeros(gw.N, dtype=torch.float64, device="cuda:0") for _ in range(2)]
    devc = torch.zeros(gw.N, dtype=torch.int64, device="cuda:0")
    from opendxmc_gb300 import native as N
    import ctypes as C

    N.check(N.lib().dxmcg_world_read_dose(gw._h, C.cast(dev[0].data_ptr(), C.POINTER(C.c_double)),
                                          C.cast(dev[1].data_ptr(), C.POINTER(C.c_double)),
                                          C.cast(devc.data_ptr(), C.POINTER(C.c_uint64))))
    np.testing.assert_array_equal(dev[0].cpu().numpy(), d)
    np.testing.assert_array_equal(dev[1].cpu().numpy(), v)
    np.testing.assert_array_equal(devc.cpu().numpy().view(np.uint64), c2)


def test_invalid_material_index_rejected(gpu):
    ph = parity.small_cylinder()
    mat = ph.material.copy()
    mat[3, 3, 3] = 7  # only 3 materials
    w = gpu.GpuWorld(ph.dims, ph.spacing, ph.materials)
    w.set_data(ph.density, mat)
    with pytest.raises(Exception, match="material index"):
        w.build()


def test_invalid_density_rejected(gpu):
    ph = parity.small_cylinder()
    dens = ph.density.copy()
    dens[1, 2, 3] = np.nan
    w = gpu.GpuWorld(ph.dims, ph.spacing, ph.materials)
    w.set_data(dens, ph.material)
    with pytest.raises(Exception, match="density"):
        w.build()


def test_transparent_material_is_skipped(gpu):
    ph = parity.small_cylinder()
    mat = np.full_like(ph.material, 255)
    gw = gpu_world(gpu, P.Phantom(ph.dims, ph.spacing, ph.density, mat, ph.materials))
    st = gw.run(P.dx_beam_params(particles=10_000, exposures=2))
    e, _, _ = gw.tally()
    assert e.sum() == 0 and st["n_interacted"] == 0
    assert st["e_escaped"] == pytest.approx(st["e_source"], rel=1e-6)


@pytest.mark.parametrize("dims,spacing", [((1, 1, 1), (12.0, 12.0, 12.0)), ((7, 5, 3), (1.3, 2.1, 3.7))])
def test_degenerate_and_odd_grids_match_oracle(gpu, oracle, dims, spacing):
    """A single voxel, and an odd-sized grid with anisotropic voxels and zero-density
    voxels, both under a DX beam: shared streams give the oracle's counts and energy."""
    rng = np.random.default_rng(sum(dims))
    nx, ny, nz = dims
    mat = rng.integers(0, 3, (nz, ny, nx)).astype(np.uint8)
    dens = np.array([0.0012, 1.0, 1.92])[mat] * rng.uniform(0.9, 1.1, mat.shape)
    if mat.size > 1:
        dens.ravel()[::4] = 0.0  # empty voxels
    ph = P.Phantom(dims, spacing, dens, mat, [P.AIR, P.WATER, P.BONE])
    gw = gpu_world(gpu, ph)
    ow = oracle_world_on_packed(oracle, gw, ph)
    beam = P.dx_beam_params(particles=50_000, exposures=4, field_cm=30.0)
    sg = gw.run(beam, gpu.run_options(seed=2, stream=5))
    so = ow.run(beam, seed=2, stream=5)
    assert sg["n_errors"] == 0
    for k in ("n_histories", "n_missed"):
        assert sg[k] == so[k], k
    assert sg["n_photo"] + sg["n_compton"] > 0
    for k in ("n_photo", "n_compton", "n_rayleigh", "n_interacted"):
        assert sg[k] == pytest.approx(so[k], rel=5e-3, abs=3), k
    e1, _, _ = gw.tally()
    e2, _, _ = ow.tally()
    assert e1.sum() == pytest.approx(e2.sum(), rel=5e-3)
    assert e1.sum() + sg["e_escaped"] == pytest.approx(sg["e_source"], rel=1e-5)


def test_beam_that_misses_the_grid(gpu):
    """A pencil beam passing beside the grid: every history is missed, nothing is
    deposited and all source energy escapes."""
    ph = parity.small_cylinder()
    gw = gpu_world(gpu, ph)
    beam = {"type": 4, "energy_kev": 60.0, "particles_per_exposure": 10_000, "n_exposures": 1,
            "position": [100.0, 100.0, 0.0], "cosines": [[0, 0, 1], [-1, 0, 0]]}
    st = gw.run(beam, gpu.run_options(seed=1))
    e, _, c = gw.tally()
    assert st["n_histories"] == st["n_missed"] == 10_000
    assert e.sum() == 0 and c.sum() == 0
    assert st["e_escaped"] == pytest.approx(st["e_source"], rel=1e-6)


def test_zero_histories_rejected(gpu):
    from opendxmc_gb300 import native as N

    ph = parity.small_cylinder()
    gw = gpu_world(gpu, ph)
    with pytest.raises(N.DxmcgError, match="particles_per_exposure"):
        gw.run(P.dx_beam_params(particles=0, exposures=2))


def test_cancel_stops_between_launches(gpu):
    ph = parity.small_cylinder()
    gw = gpu_world(gpu, ph)
    prog = gpu.Progress()
    prog.setStopSimulation()
    rc, st = gw.run_status(P.dx_beam_params(particles=100_000, exposures=10), gpu.run_options(chunk_log2=14),
                           prog)
    assert rc == -4 and st["n_histories"] == 0
    assert not prog.continueSimulation()
    # stop from another thread while the run is in flight
    prog2 = gpu.Progress()
    res = {}

    def work():
        res["rc"], res["st"] = gw.run_status(P.dx_beam_params(particles=10_000_000, exposures=10),
                                             gpu.run_options(chunk_log2=16), prog2)

    t = threading.Thread(target=work)
    t.start()
    for _ in range(2000):
        done, total = prog2.progress()
        if done > 0:
            break
        time.sleep(0.005)
    prog2.setStopSimulation()
    t.join(timeout=120)
    assert not t.is_alive()
    assert res["rc"] in (-4, 0)
    if res["rc"] == -4:
        assert res["st"]["n_histories"] < 100_000_000
        assert prog2.message() == "Cancelled"


def test_progress_reports_histories(gpu):
    ph = parity.small_cylinder()
    gw = gpu_world(gpu, ph)
    prog = gpu.Progress()
    gw.run(P.dx_beam_params(particles=100_000, exposures=3), gpu.run_options(chunk_log2=15), prog)
    assert prog.progress() == (300_000, 300_000)
    assert prog.message() == "Done"
