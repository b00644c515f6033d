"""Batched jobs in one persistent launch (dxmcg_batch_*) and the launch-shape
autotuner (dxmcg_autotune), through the C ABI.

A history's random stream depends only on (seed, stream, history index), so a
job run inside a batch, or under another launch shape, follows the same
histories as the job run alone: tallies agree up to the order of the FP64
atomic additions, and up to the rare decision that the multi-job kernel
instance rounds differently from the single-job one.
"""
import numpy as np
import pytest

from opendxmc_gb300 import native as N
from opendxmc_gb300 import phantoms as P

pytestmark = pytest.mark.gpu

TRACKINGS = {"woodcock": N.TRACK_WOODCOCK, "siddon": N.TRACK_SIDDON, "macro": N.TRACK_MACRO,
             "woodcock_two_region": N.TRACK_WOODCOCK}


def make_world(gpu, ph):
    w = gpu.GpuWorld(ph.dims, ph.spacing, ph.materials, 1)
    w.set_data(ph.density, ph.material)
    w.build()
    return w


@pytest.fixture(scope="module")
def jobs():
    """Three small phantoms of uneven size; phantom 0 carries two jobs (DX + CBCT)."""
    specs = P.batched_jobs(n_jobs=4, seed=7, dim_range=(24, 56), spacing_cm=(0.2, 0.4), hist_range=(4e4, 4e5))
    phantoms = [P.ellipsoid_phantom(s["dims"], s["spacing"], s["seed"]) for s in specs[:3]]
    plan = [(0, specs[0]["beam"]), (1, specs[1]["beam"]), (2, specs[2]["beam"]), (0, specs[3]["beam"])]
    return phantoms, plan


def assert_tallies_match(a, b):
    e1, q1, c1 = a
    e2, q2, c2 = b
    assert e1.sum() > 0
    # integer event counts: identical but for a rare rounding-flipped decision
    assert np.mean(c1 == c2) >= 0.999, f"count mismatch in {np.sum(c1 != c2)} voxels"
    assert abs(e1.sum() / e2.sum() - 1) < 1e-5
    hot = e2 > 0.05 * e2.max()
    np.testing.assert_allclose(e1[hot], e2[hot], rtol=1e-3)


@pytest.mark.parametrize("tracking", sorted(TRACKINGS))
def test_batch_matches_single_runs(gpu, jobs, tracking):
    phantoms, plan = jobs
    trk = TRACKINGS[tracking]
    two = 1 if tracking == "woodcock_two_region" else 0
    opts = [gpu.run_options(seed=11 + k, stream=3 * k, tracking=trk, two_region=two) for k in range(len(plan))]

    worlds = [make_world(gpu, ph) for ph in phantoms]
    batch = gpu.Batch([(worlds[i], beam, o) for (i, beam), o in zip(plan, opts)])
    hist, cal = batch.info()
    np.testing.assert_array_equal(cal, 1.0)
    sb = batch.run()
    assert sb["n_histories"] == int(hist.sum())
    assert sb["n_errors"] == 0

    alone = [make_world(gpu, ph) for ph in phantoms]
    totals = {"n_histories": 0, "n_missed": 0, "n_photo": 0, "n_compton": 0}
    for ((i, beam), o), n in zip(zip(plan, opts), hist):
        s = alone[i].run(beam, o)
        assert s["n_histories"] == int(n)
        for k in totals:
            totals[k] += s[k]
    assert sb["n_histories"] == totals["n_histories"]
    assert sb["n_missed"] == totals["n_missed"]  # source sampling: the same code on both paths
    for k in ("n_photo", "n_compton"):
        assert abs(sb[k] / totals[k] - 1) < 1e-4
    for wb, wa in zip(worlds, alone):
        assert_tallies_match(wb.tally(), wa.tally())
        db, _, _ = wb.dose()
        da, _, _ = wa.dose()
        assert abs(db.sum() / da.sum() - 1) < 1e-5
    batch.close()


def test_batch_graph_replay(gpu, jobs):
    """Every run replays the captured graph: the same histories again, so counts
    and the dose (which accumulates over runs, as DXMClib's does) double."""
    phantoms, plan = jobs
    worlds = [make_world(gpu, ph) for ph in phantoms]
    batch = gpu.Batch([(worlds[i], beam, gpu.run_options(seed=5, stream=k)) for k, (i, beam) in enumerate(plan)])
    s1 = batch.run()
    one = [w.tally() for w in worlds]
    d1 = [w.dose()[0] for w in worlds]
    s2 = batch.run()
    assert s1["n_histories"] == s2["n_histories"]
    assert s1["n_photo"] == s2["n_photo"] and s1["n_compton"] == s2["n_compton"]
    for w, (e, _, c), d in zip(worlds, one, d1):
        e2, _, c2 = w.tally()
        np.testing.assert_array_equal(c2, 2 * c)
        np.testing.assert_allclose(e2, 2 * e, rtol=1e-9, atol=1e-9)
        np.testing.assert_allclose(w.dose()[0], 2 * d, rtol=1e-9, atol=1e-30)
    batch.close()


def test_per_job_batch_matches_single_runs_and_replays(gpu):
    """Jobs of 2.1e6 histories or more on average run as one single-job launch each,
    on several streams of the captured graph: the same kernel and streams as
    dxmcg_transport_run, so counts equal the single runs exactly and energies up to the
    order of FP64 atomics.  Two jobs share one world; a replay doubles the tallies."""
    phs = [P.ellipsoid_phantom((40, 36, 30), (0.3, 0.3, 0.3), seed=s) for s in (1, 2)]
    beams = [P.dx_beam_params(kvp=80.0, field_cm=10.0, particles=400_000, exposures=6),
             P.cbct_params(particles=30_000, kvp=90.0),
             P.dx_beam_params(kvp=70.0, field_cm=8.0, particles=300_000, exposures=8)]
    plan = [(0, 0), (1, 1), (0, 2)]
    worlds = [make_world(gpu, ph) for ph in phs]
    opts = [gpu.run_options(seed=21 + k, stream=k) for k in range(len(plan))]
    batch = gpu.Batch([(worlds[i], beams[b], o) for (i, b), o in zip(plan, opts)])
    hist, _ = batch.info()
    assert hist.sum() >= (1 << 21) * len(plan)  # the per-job path
    sb = batch.run()
    assert sb["n_errors"] == 0 and sb["n_histories"] == int(hist.sum())
    alone = [make_world(gpu, ph) for ph in phs]
    tot = {"n_histories": 0, "n_photo": 0, "n_compton": 0, "n_rayleigh": 0, "n_visits": 0}
    for (i, b), o in zip(plan, opts):
        s = alone[i].run(beams[b], o)
        for k in tot:
            tot[k] += s[k]
    for k in tot:
        assert sb[k] == tot[k], k
    for wb, wa in zip(worlds, alone):
        e1, _, c1 = wb.tally()
        e2, _, c2 = wa.tally()
        np.testing.assert_array_equal(c1, c2)
        np.testing.assert_allclose(e1, e2, rtol=1e-9, atol=1e-9)
    batch.run()
    for wb, wa in zip(worlds, alone):
        np.testing.assert_array_equal(wb.tally()[2], 2 * wa.tally()[2])
    batch.close()


def test_batch_rejects_bad_jobs(gpu, jobs):
    phantoms, plan = jobs
    w = make_world(gpu, phantoms[0])
    beam = plan[0][1]
    with pytest.raises(N.DxmcgError, match="tracking"):
        gpu.Batch([(w, beam, gpu.run_options(tracking=N.TRACK_WOODCOCK)),
                   (w, beam, gpu.run_options(tracking=N.TRACK_SIDDON))])
    with pytest.raises(N.DxmcgError, match="hist_begin"):
        gpu.Batch([(w, beam, gpu.run_options(hist_end=100))])
    with pytest.raises(N.DxmcgError, match="macro_cell"):
        gpu.Batch([(w, beam, gpu.run_options(tracking=N.TRACK_MACRO, macro_cell=8)),
                   (w, beam, gpu.run_options(tracking=N.TRACK_MACRO, macro_cell=16))])
    unbuilt = gpu.GpuWorld(phantoms[1].dims, phantoms[1].spacing, phantoms[1].materials, 1)
    with pytest.raises(N.DxmcgError, match="not built"):
        gpu.Batch([(unbuilt, beam, None)])


def test_autotune_leaves_dose_and_histories_unchanged(gpu):
    ph = P.ellipsoid_phantom((64, 64, 48), (0.3, 0.3, 0.3), seed=3)
    beam = P.dx_beam_params(kvp=80.0, field_cm=12.0, particles=40_000, exposures=10)
    w = make_world(gpu, ph)
    tuned, rate = w.autotune(beam, gpu.run_options(seed=2), sample_histories=1 << 20)
    assert rate > 0
    assert tuned.block_size in (128, 256)
    assert tuned.interact_batch in (8, 12, 16, 24)
    assert tuned.refill_batch in (4, 8, 16)
    e, _, c = w.tally()
    assert e.sum() == 0 and c.sum() == 0  # trials used a scratch tally
    st = w.run(beam, tuned)
    ref = make_world(gpu, ph)
    sr = ref.run(beam, gpu.run_options(seed=2))
    assert st["n_histories"] == sr["n_histories"]
    # the launch shape does not change which histories run: same tallies up to FP order
    e1, _, c1 = w.tally()
    e2, _, c2 = ref.tally()
    np.testing.assert_array_equal(c1, c2)
    assert abs(e1.sum() / e2.sum() - 1) < 1e-9
