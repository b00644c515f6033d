"""CPU tests of the oracle: pinned to the reference's own data files (golden
fixtures) and to analytic known answers.  No GPU needed."""
import json
from pathlib import Path

import numpy as np
import pytest

from opendxmc_gb300 import phantoms as P
import parity

GOLDEN = json.loads((Path(__file__).parent / "golden" / "reference_data.json").read_text())
SIGMA_THOMSON = 8.0 * np.pi / 3.0 * 0.0794077878  # barn


def as_zw(comp: dict) -> dict:
    return {int(z): float(w) for z, w in comp.items()}


@pytest.mark.parametrize("row,const", [("2", P.BONE), ("29", P.MUSCLE), ("45", P.SOFT_TISSUE),
                                       ("49", P.ADIPOSE), ("50", P.LUNG), ("53", P.AIR)])
def test_compositions_match_reference_media_table(row, const):
    assert as_zw(GOLDEN["AM_media"][row]["composition"]) == {int(z): float(w) for z, w in const.items()}


def test_water_and_bowtie_match_reference_files():
    assert as_zw(GOLDEN["other_media"]["53"]["composition"]) == P.WATER
    assert GOLDEN["other_media"]["53"]["name"] == "Water"
    tpl = GOLDEN["bowtie_template"]["Siemens Definition Flash Body W3 120kV"]
    assert [tuple(x) for x in tpl] == P.BODY_BOWTIE
    assert "Siemens Definition Flash W1 120kV" in GOLDEN["bowtiefilters"]  # default key, beamsettingsmodel.cpp:1303
    assert len(GOLDEN["bowtiefilters"]) == 41


def test_klein_nishina_limits(oracle):
    L = oracle.lib()
    assert L.or_sigma_kn(0.01) == pytest.approx(SIGMA_THOMSON, rel=1e-4)
    assert L.or_sigma_kn(100.0) < L.or_sigma_kn(10.0) < SIGMA_THOMSON
    # level 0 is free-electron KN; binding (S < Z) only lowers it
    for Z in (1, 8, 20):
        for E in (5.0, 30.0, 100.0):
            assert L.or_sigma_incoh(E, Z, 0) == pytest.approx(Z * L.or_sigma_kn(E), rel=1e-12)
            assert L.or_sigma_incoh(E, Z, 1) < L.or_sigma_incoh(E, Z, 0)
    # S saturates for hydrogen at high energy
    assert L.or_sigma_incoh(150.0, 1, 1) / L.or_sigma_kn(150.0) > 0.99


def test_rayleigh_low_energy_limit(oracle):
    # F -> Z as x -> 0: sigma_coh -> Z^2 sigma_Thomson
    L = oracle.lib()
    for Z in (1, 8, 20):
        assert L.or_sigma_coh(1e-3, Z) == pytest.approx(Z * Z * SIGMA_THOMSON, rel=1e-3)


def test_water_attenuation_plausible(oracle):
    p, ic, co = oracle.attenuation(P.WATER, [30.0, 60.0, 100.0])
    tot = p + ic + co
    # project model within 10 % of the textbook values 0.376 / 0.206 / 0.171 cm2/g
    assert tot == pytest.approx([0.376, 0.206, 0.171], rel=0.10)
    assert p[0] == pytest.approx(ic[0], rel=0.3)  # photo/Compton crossover near 30 keV


def _chi2_p(hist, expected):
    from scipy import stats

    m = expected > 5
    chi2 = float((((hist - expected) ** 2) / expected)[m].sum())
    return stats.chi2.sf(chi2, m.sum() - 1)


@pytest.mark.parametrize("E", [20.0, 80.0, 150.0])
def test_compton_sampler_matches_klein_nishina(oracle, E):
    rng = np.random.default_rng(7)
    n = 20000
    mus = np.array([oracle.sample_compton(E, {8: 1.0}, 0, rng.random(64))[1] for _ in range(n)])
    k = E / 510.99895
    edges = np.linspace(-1, 1, 41)
    x = np.linspace(-1, 1, 4001)
    eps = 1 / (1 + k * (1 - x))
    pdf = eps ** 2 * (eps + 1 / eps - (1 - x * x))
    cdf = np.concatenate([[0], np.cumsum(0.5 * (pdf[1:] + pdf[:-1]) * np.diff(x))])
    cdf /= cdf[-1]
    expected = np.diff(np.interp(edges, x, cdf)) * n
    hist, _ = np.histogram(mus, edges)
    assert _chi2_p(hist, expected) > 1e-4


def test_compton_with_incoherent_function_suppresses_forward(oracle):
    rng = np.random.default_rng(9)
    E = 20.0
    mu0 = np.array([oracle.sample_compton(E, P.WATER, 0, rng.random(256))[1] for _ in range(5000)])
    mu1 = np.array([oracle.sample_compton(E, P.WATER, 1, rng.random(256))[1] for _ in range(5000)])
    assert (mu1 > 0.95).mean() < 0.5 * (mu0 > 0.95).mean()


def test_rayleigh_sampler_matches_form_factor(oracle):
    rng = np.random.default_rng(11)
    E, Z = 40.0, 8
    n = 20000
    mus = np.array([oracle.sample_rayleigh(E, {Z: 1.0}, rng.random(128))[0] for _ in range(n)])
    a = (Z ** (1 / 3) / (2 * np.pi * 0.529177210903)) ** 2
    q = E / 12.398419843
    x = np.linspace(-1, 1, 20001)
    t = q * q * (1 - x) / 2
    pdf = (1 + x * x) / (1 + t / a) ** 4
    cdf = np.concatenate([[0], np.cumsum(0.5 * (pdf[1:] + pdf[:-1]) * np.diff(x))])
    cdf /= cdf[-1]
    edges = np.concatenate([np.linspace(-1, 0.9, 20), np.linspace(0.91, 1, 10)])
    expected = np.diff(np.interp(edges, x, cdf)) * n
    hist, _ = np.histogram(mus, edges)
    assert _chi2_p(hist, expected) > 1e-4


def test_stream_uniforms(oracle):
    from scipy import stats

    raw = oracle.history_stream(1, 5, 0, 2500, 2).ravel()
    u = np.array([oracle.lib().or_uniform_from_u32(int(x)) for x in raw])
    assert u.min() > 0 and u.max() < 1
    assert stats.kstest(u, "uniform").pvalue > 1e-3
    assert oracle.lib().or_uniform_from_u32(0) == 2.0 ** -24
    assert oracle.lib().or_uniform_from_u32(0xFFFFFFFF) == 1.0 - 2.0 ** -24


def _xoshiro128p(state, n):
    """Plain-Python xoshiro128+ (Blackman & Vigna 2018) for checking the oracle."""
    s = [int(x) for x in state]
    M = 0xFFFFFFFF
    rotl = lambda x, k: ((x << k) | (x >> (32 - k))) & M
    out = []
    for _ in range(n):
        out.append((s[0] + s[3]) & M)
        t = (s[1] << 9) & M
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = rotl(s[3], 11)
    return out


def _splitmix64(z):
    """Plain-Python SplitMix64 output function (Steele, Lea & Flood 2014)."""
    M = (1 << 64) - 1
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
    return z ^ (z >> 31)


def test_history_streams_are_splitmix_seeded_xoshiro(oracle):
    M, G = (1 << 64) - 1, 0x9E3779B97F4A7C15
    seed, stream = 0x1234567890ABCDEF, 3
    key = _splitmix64(seed ^ _splitmix64((stream + G) & M))
    got = oracle.history_stream(seed, stream, 2 ** 33 - 2, 4, 12)
    for i in range(4):
        h = 2 ** 33 - 2 + i
        x = (key + (2 * h + 1) * G) & M
        a, b = _splitmix64(x), _splitmix64((x + G) & M)
        state = [a & 0xFFFFFFFF, a >> 32, b & 0xFFFFFFFF, b >> 32]
        assert list(got[i]) == _xoshiro128p(state, 12)
    # streams of neighbouring histories and stream words differ
    a = oracle.history_stream(1, 0, 0, 2, 8)
    b = oracle.history_stream(1, 1, 0, 1, 8)
    assert not np.array_equal(a[0], a[1]) and not np.array_equal(a[0], b[0])


def test_tube_spectrum_properties(oracle):
    E, w = oracle.tube_spectrum(120.0, {13: 6.0})
    assert E[0] == 1.0 and E[-1] == 120.0 and len(E) == 120
    assert w.sum() == pytest.approx(1.0, abs=1e-12)
    assert w[57] > w[55] and w[58] > w[60]  # tungsten K lines at 58 and 59 keV
    assert oracle.tube_mean_energy(120, {13: 9.0}) > oracle.tube_mean_energy(120, {13: 6.0})
    assert oracle.tube_al_hvl_mm(120, {13: 9.0}) > oracle.tube_al_hvl_mm(120, {13: 6.0})
    assert 4.0 < oracle.tube_al_hvl_mm(120, {13: 6.0}) < 9.0


def test_ct_spiral_exposure_geometry(oracle):
    cp = P.ct_spiral_params(particles=1)
    ex = oracle.beam_exposures(cp)
    assert len(ex) == 360  # 20 cm / (4 cm x pitch 1) x 72 views
    sid = 119.0 / 2
    for i, e in enumerate(ex[:80]):
        pos, c0, c1 = map(np.array, (e["pos"], e["c0"], e["c1"]))
        iso = np.array([0.0, 0.0, -10.0 + i * 4.0 / 72])
        assert np.linalg.norm((pos - iso)[:2]) == pytest.approx(sid)
        assert pos[2] == pytest.approx(iso[2])
        n = np.cross(c0, c1)
        assert np.dot(n, (iso - pos) / sid) == pytest.approx(1.0)
        assert np.dot(c0, c1) == pytest.approx(0.0, abs=1e-12)
    assert ex[0]["half"][0] == pytest.approx(np.arctan(25.0 / sid))
    assert ex[0]["half"][1] == pytest.approx(np.arctan(2.0 / sid))


def test_dx_pose_matches_reference_dxbeam(oracle):
    # DXBeam at 0/0 deg: source at rotation centre + SPD * (0, 1, 0), beam along -y
    ex = oracle.beam_exposures(P.dx_beam_params(particles=1, exposures=3))
    assert len(ex) == 3
    n = np.cross(ex[0]["c0"], ex[0]["c1"])
    assert np.allclose(n, [0, -1, 0]) and np.allclose(ex[0]["pos"], [0, 100, 0])


def test_aec_weights_are_relative(oracle):
    cp = P.ct_spiral_params(particles=1)
    cp["aec"] = ([0, 0, -10], [0, 0, 10], [1.0, 3.0])
    w = np.array([e["weight"] for e in oracle.beam_exposures(cp)])
    assert w.mean() == pytest.approx(1.0)
    assert w[-1] / w[0] == pytest.approx(3.0, rel=0.02)


@pytest.mark.parametrize("compensate", [0, 1])
def test_organ_aec_weights(oracle, compensate):
    cp = dict(P.ct_spiral_params(particles=1, scan_cm=8.0), organ_aec=1, organ_aec_start_deg=332.5,
              organ_aec_stop_deg=27.5, organ_aec_ramp_deg=12.0, organ_aec_low_weight=0.3,
              organ_aec_compensate=compensate)
    ex = oracle.beam_exposures(cp)
    w = np.array([e["weight"] for e in ex])
    ang = (np.arange(len(ex)) * 5.0) % 360.0
    inside = (ang >= 332.5) | (ang <= 27.5)
    ramp = ((ang > 27.5) & (ang < 39.5)) | ((ang > 320.5) & (ang < 332.5))
    assert np.allclose(w[inside], 0.3)
    assert np.all((w[ramp] > 0.3) & (w[ramp] < 1.0))
    out = ~(inside | ramp)
    if compensate:
        assert w.mean() == pytest.approx(1.0)
        assert np.allclose(w[out], w[out][0]) and w[out][0] > 1.0
    else:
        assert np.allclose(w[out], 1.0) and w.mean() < 1.0


def test_oracle_energy_conservation(oracle):
    ph = parity.small_cylinder()
    w = oracle.World(ph.dims, ph.spacing, ph.density, ph.material, ph.materials)
    st = w.run(P.dx_beam_params(particles=2000, exposures=5), threads=4)
    e, _, _ = w.tally()
    assert st["n_histories"] == 10000 and st["n_errors"] == 0
    assert e.sum() + st["e_escaped"] == pytest.approx(st["e_source"], rel=1e-12)
    assert e.sum() == pytest.approx(st["e_deposited"], rel=1e-12)


def test_oracle_beer_lambert_transmission(oracle):
    # 60 keV pencil beam through 10 cm of water: P(no interaction) = exp(-mu L)
    dims = (4, 40, 4)
    dens = np.ones(dims[::-1])
    mat = np.zeros(dims[::-1], dtype=np.uint8)
    w = oracle.World(dims, (0.25, 0.25, 0.25), dens, mat, [P.WATER])
    n = 40000
    beam = {"type": oracle.BEAM_PENCIL, "energy_kev": 60.0, "particles_per_exposure": n, "n_exposures": 1,
            "position": [0.0, 50.0, 0.0], "cosines": [[0, 0, 1], [-1, 0, 0]]}
    st = w.run(beam, threads=4)
    p, ic, co = oracle.attenuation(P.WATER, [60.0])
    trans = np.exp(-(p + ic + co)[0] * 1.0 * 10.0)
    measured = 1.0 - st["n_interacted"] / n
    assert measured == pytest.approx(trans, abs=4 * np.sqrt(trans * (1 - trans) / n))


def test_oracle_woodcock_and_siddon_tracking_agree(oracle):
    ph = parity.small_cylinder()
    w = oracle.World(ph.dims, ph.spacing, ph.density, ph.material, ph.materials)
    beam = P.dx_beam_params(particles=20000, exposures=5)
    s1 = w.run(beam, tracking=oracle.TRACK_WOODCOCK, threads=8)
    e1, q1, _ = w.tally()
    w.clear()
    s2 = w.run(beam, tracking=oracle.TRACK_SIDDON, threads=8, stream=1)
    e2, q2, _ = w.tally()
    n = s1["n_histories"]
    frac, nvox = parity.combined_sigma_agreement(e1, parity.tally_variance(e1, q1, n), e2,
                                                 parity.tally_variance(e2, q2, n))
    assert nvox > 100 and frac >= 0.99
    assert e1.sum() == pytest.approx(e2.sum(), rel=0.01)


def test_oracle_default_tracking_follows_the_box_fraction(oracle):
    """The oracle's default Woodcock mirrors the transport kernel's: two regions when
    the box of the voxels whose material is neither 0 nor transparent holds less than
    half the grid's voxels."""
    for ph, two in ((parity.small_torso(scale=4, seed=3), True), (parity.small_cylinder(), False)):
        w = oracle.World(ph.dims, ph.spacing, ph.density, ph.material, ph.materials)
        fg = (ph.material != 0) & (ph.material != 255)
        idx = np.argwhere(fg)
        frac = float(np.prod((idx.max(0) - idx.min(0) + 1) / np.array(ph.material.shape)))
        assert w.box_fraction == pytest.approx(frac, abs=1e-12)
        assert (w.box_fraction < oracle.TWO_REGION_BOX_FRACTION) == two


def test_oracle_two_region_woodcock_equals_plain_woodcock(oracle):
    """Two-region Woodcock (material 0's own majorant outside the box of the other
    voxels) samples the plain Woodcock transport with fewer tentative collisions:
    per-voxel energy within 3 combined standard errors, totals of 16 replicates each
    within 4 standard errors of their difference, and a third of the visits.  The box
    is empty on a grid without background voxels, where the mode is plain Woodcock."""
    ph = parity.small_torso(scale=4, seed=3)
    w = oracle.World(ph.dims, ph.spacing, ph.density, ph.material, ph.materials)
    beam = P.ct_spiral_params(particles=400, scan_cm=10.0)
    tot, tally, visits = {}, {}, {}
    for trk in (oracle.TRACK_WOODCOCK, oracle.TRACK_WOODCOCK_BOX):
        w.clear()
        runs = [w.run(beam, stream=100 * trk + r, tracking=trk, threads=8) for r in range(16)]
        tot[trk] = np.array([s["e_deposited"] for s in runs])
        visits[trk] = sum(s["n_visits"] for s in runs) / sum(s["n_histories"] for s in runs)
        tally[trk] = w.tally()
        assert sum(s["n_errors"] for s in runs) == 0
    n = 16 * runs[0]["n_histories"]
    (e1, q1, _), (e2, q2, _) = tally[oracle.TRACK_WOODCOCK], tally[oracle.TRACK_WOODCOCK_BOX]
    frac, nvox = parity.combined_sigma_agreement(e1, parity.tally_variance(e1, q1, n), e2,
                                                 parity.tally_variance(e2, q2, n))
    assert nvox > 200 and frac >= 0.99
    a, b = tot[oracle.TRACK_WOODCOCK], tot[oracle.TRACK_WOODCOCK_BOX]
    assert abs(a.sum() - b.sum()) <= 4.0 * np.hypot(parity.total_sigma(a), parity.total_sigma(b))
    assert visits[oracle.TRACK_WOODCOCK_BOX] < 0.5 * visits[oracle.TRACK_WOODCOCK]
    # no background voxel: one region, the same histories as plain Woodcock
    full = oracle.World(ph.dims, ph.spacing, ph.density, np.ones_like(ph.material), ph.materials)
    s1 = full.run(beam, stream=5, tracking=oracle.TRACK_WOODCOCK, hist_end=20000)
    e1, _, _ = full.tally()
    full.clear()
    s2 = full.run(beam, stream=5, tracking=oracle.TRACK_WOODCOCK_BOX, hist_end=20000)
    e2, _, _ = full.tally()
    assert s1["n_visits"] == s2["n_visits"]
    np.testing.assert_allclose(e2, e1, rtol=1e-12, atol=0)


# ---- correction level 2 (impulse approximation, fluorescence)
ME = 510.99895


def test_doppler_energy_solves_the_impulse_relation(oracle):
    rng = np.random.default_rng(3)
    for _ in range(2000):
        E = rng.uniform(5.0, 150.0)
        c = rng.uniform(-1.0, 1.0)
        rho = rng.uniform(-0.3, 0.3)
        omu = 1.0 - c
        A = 1.0 + E / ME * omu
        x = oracle.doppler_energy(E, A, omu, rho)
        assert x > 0.0
        q = np.sqrt(E * E + x * x - 2.0 * E * x * c)
        back = (E * x * omu / ME - (E - x)) / q
        assert back == pytest.approx(rho, rel=1e-9, abs=1e-12)
    # no electron momentum: the Compton line
    assert oracle.doppler_energy(60.0, 1.0 + 60.0 / ME, 1.0, 0.0) == pytest.approx(60.0 / (1.0 + 60.0 / ME))


def test_level2_shells_and_yields(oracle):
    for Z in (1, 6, 8, 15, 20, 53, 74):
        e, b, m = oracle.compton_shells(Z)
        assert e.sum() == pytest.approx(Z)
        assert np.all(np.diff(b) < 0)  # inner shells bound more tightly
        assert b[0] == pytest.approx(oracle.lib().or_k_edge(Z) if Z > 1 else 13.605693122994e-3)
        assert np.allclose(m, np.sqrt(b / 13.605693122994e-3) / 137.035999084, rtol=1e-9)
    # K fluorescence yields of the Bambynek fit: calcium ~0.16, tungsten ~0.96
    assert oracle.lib().or_fluorescence_yield_k(20) == pytest.approx(0.163, abs=0.005)
    assert oracle.lib().or_fluorescence_yield_k(74) == pytest.approx(0.957, abs=0.005)


@pytest.mark.parametrize("E", [20.0, 60.0, 140.0])
def test_level2_compton_is_doppler_broadened(oracle, E):
    rng = np.random.default_rng(int(E))
    n = 20000
    U = parity.uniforms_f32_exact(rng, (n, 1024))
    d_rel = []
    for i in range(n):
        Ep, cost, used = oracle.sample_compton(E, P.WATER, 2, U[i])
        Ec = E / (1.0 + E / ME * (1.0 - cost))
        assert used < 1024
        assert 0.0 < Ep < E
        d_rel.append((Ep - Ec) / Ec)
    d_rel = np.asarray(d_rel)
    # broadened around the Compton line: centred, with a spread of a few per cent or less
    assert abs(np.median(d_rel)) < 2e-3
    assert 1e-4 < np.std(d_rel) < 0.05
    # level 1 returns the Compton line exactly
    Ep, cost, _ = oracle.sample_compton(E, P.WATER, 1, U[0])
    assert Ep == pytest.approx(E / (1.0 + E / ME * (1.0 - cost)), rel=1e-12)


def test_level2_photoelectric_fluorescence(oracle):
    calcium = {20: 1.0}
    rng = np.random.default_rng(9)
    n = 40000
    U = parity.uniforms_f32_exact(rng, (n, 8))
    ka = oracle.lib().or_k_alpha(20)
    out = np.array([oracle.sample_photoelectric(60.0, calcium, U[i])[:2] for i in range(n)])
    emitted = out[:, 0] > 0
    assert np.all(out[emitted, 0] == ka)
    p = (1.0 - 1.0 / 7.0) * oracle.lib().or_fluorescence_yield_k(20)
    assert emitted.mean() == pytest.approx(p, abs=5 * np.sqrt(p * (1 - p) / n))
    # isotropic: dz uniform in [-1, 1]
    assert abs(out[emitted, 1].mean()) < 0.03 and out[emitted, 1].var() == pytest.approx(1 / 3, abs=0.02)
    # below the K edge, and for water (oxygen's K-alpha is under the 1 keV cutoff): no photon
    assert all(oracle.sample_photoelectric(3.0, calcium, U[i])[0] == 0.0 for i in range(200))
    assert all(oracle.sample_photoelectric(60.0, P.WATER, U[i])[0] == 0.0 for i in range(200))


def test_oracle_level2_transport_conserves_energy(oracle):
    ph = parity.small_cylinder()
    w = oracle.World(ph.dims, ph.spacing, ph.density, ph.material, ph.materials, 2)
    st = w.run(P.dx_beam_params(particles=4000, exposures=5), threads=4)
    e, _, _ = w.tally()
    assert st["n_histories"] == 20000 and st["n_errors"] == 0
    assert st["n_fluorescence"] > 0  # the bone insert holds calcium
    assert e.sum() + st["e_escaped"] == pytest.approx(st["e_source"], rel=1e-12)


@pytest.mark.parametrize("correction", [0, 1])
@pytest.mark.parametrize("index", [8, 118, 298])  # 5, 60 and 150 keV
def test_compton_angle_table_matches_klein_nishina_times_s(oracle, correction, index):
    """The Compton angle table against the distribution it stands for: KN(mu) S(x)/Z
    for water (S = 1 at correction 0), integrated here on 4e5 steps.  Sampling the
    table inverts it linearly between its probabilities u_j = (1 - cos(pi j/255))/2, so
    the sampled distribution's CDF is the table's points joined linearly; its largest
    distance from the exact CDF (Kolmogorov distance) must stay below 5e-5."""
    E = oracle.EMIN + index * oracle.DE
    omu = oracle.compton_quantiles(P.WATER, correction, index)
    assert omu[0] == 2.0 and omu[-1] == 0.0 and np.all(np.diff(omu) <= 0)
    u = 0.5 * (1.0 - np.cos(np.pi * np.arange(256) / 255.0))
    mu_tab = 1.0 - omu
    k = E / 510.99895
    mu = np.linspace(-1.0, 1.0, 400_001)
    p = 1.0 / (1.0 + k * (1.0 - mu))
    pdf = p * p * (p + 1.0 / p - 1.0 + mu * mu)
    if correction:
        t = (E / 12.398419843) ** 2 * 0.5 * (1.0 - mu)
        S = np.zeros_like(mu)
        zsum = 0.0
        for z, w in P.WATER.items():
            n = w / {1: 1.008, 8: 15.999}[z]
            a = (z ** (1 / 3) / (2 * np.pi * 0.529177210903)) ** 2
            S += n * z * (1.0 - (1.0 + t / a) ** -4)
            zsum += n * z
        pdf = pdf * S / zsum
    cdf = np.concatenate([[0.0], np.cumsum(0.5 * (pdf[1:] + pdf[:-1]) * np.diff(mu))])
    cdf /= cdf[-1]
    implied = np.interp(mu, mu_tab, u)
    assert np.abs(implied - cdf).max() < 5e-5


@pytest.mark.parametrize("index", [8, 38, 118, 298])  # 5, 20, 60 and 150 keV
def test_rayleigh_angle_table_matches_form_factor(oracle, index):
    """The Rayleigh angle table against (1 + mu^2)/2 sum_i n_i Z_i^2 (1 + t/a_i)^-4 for
    water (t = x^2), integrated here on 2e6 steps of w = sqrt((1 - mu)/2) squared: the
    sampled distribution (the table's points joined linearly in probability) is within
    a Kolmogorov distance of 5e-5 of it."""
    E = oracle.EMIN + index * oracle.DE
    omu = oracle.rayleigh_quantiles(P.WATER, index)
    assert omu[0] == 2.0 and omu[-1] == 0.0 and np.all(np.diff(omu) <= 0)
    u = 0.5 * (1.0 - np.cos(np.pi * np.arange(256) / 255.0))
    s = np.linspace(0.0, 1.0, 2_000_001)
    w = s * s
    om = 2.0 * w * w
    mu = 1.0 - om
    t = (E / 12.398419843) ** 2 * 0.5 * om
    F2 = np.zeros_like(s)
    for z, wt in P.WATER.items():
        n = wt / {1: 1.008, 8: 15.999}[z]
        a = (z ** (1 / 3) / (2 * np.pi * 0.529177210903)) ** 2
        F2 += n * z * z / (1.0 + t / a) ** 4
    f = 0.5 * (1.0 + mu * mu) * F2 * 4.0 * w * 2.0 * s  # density in s
    mass = np.concatenate([[0.0], np.cumsum(0.5 * (f[1:] + f[:-1]) * np.diff(s))])
    mass /= mass[-1]  # probability of 1 - cos theta below om
    implied = 1.0 - np.interp(om[::-1], omu[::-1], u[::-1])[::-1]  # table's P(1 - cos < om)
    assert np.abs(implied - mass).max() < 5e-5
