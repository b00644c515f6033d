"""A loaded physics table drives the GPU transport: the model written as a table
leaves every device table bit for bit as the model builds it, and a different table
changes the dose while the GPU still matches the oracle reading the same file."""
import numpy as np
import pytest

from opendxmc_gb300 import phantoms as P
import parity
from test_cpu_physics_tables import MODEL_TABLE, modified_table

pytestmark = pytest.mark.gpu


@pytest.fixture
def tables(gpu, oracle):
    yield gpu, oracle
    gpu.physics_reset()
    oracle.physics_reset()


def world(gpu, ph, correction=1):
    w = gpu.GpuWorld(ph.dims, ph.spacing, ph.materials, correction)
    w.set_data(ph.density, ph.material)
    w.build()
    return w


def test_model_table_gives_identical_device_tables(tables, tmp_path):
    gpu, _ = tables
    ph = parity.small_torso()
    ref = [world(gpu, ph).tables(m) for m in range(len(ph.materials))]
    path = tmp_path / "model.txt"
    gpu.physics_write(path, sorted({z for m in ph.materials for z in m}))
    gpu.physics_load(path)
    w = world(gpu, ph)
    for m, (xs, maj) in enumerate(ref):
        xs2, maj2 = w.tables(m)
        np.testing.assert_array_equal(xs2, xs)
        np.testing.assert_array_equal(maj2, maj)


def test_modified_table_transport_matches_oracle(tables, tmp_path):
    gpu, oracle = tables
    ph = parity.small_cylinder()
    beam = P.dx_beam_params(particles=300_000, exposures=10)
    base = world(gpu, ph)
    base.run(beam, gpu.run_options(seed=6, stream=0))
    e0, _, _ = base.tally()
    path = tmp_path / "modified.txt"
    modified_table(MODEL_TABLE, path)
    gpu.physics_load(path)
    oracle.physics_load(path)
    gw = world(gpu, ph)
    d, _ = gw.packed_density()
    ow = oracle.World(ph.dims, ph.spacing, d.astype(np.float64), ph.material, ph.materials)
    sg = gw.run(beam, gpu.run_options(seed=6, stream=0))
    ow.run(beam, seed=6, stream=1)
    n = sg["n_histories"]
    e1, q1, _ = gw.tally()
    e2, q2, _ = ow.tally()
    frac, nvox = parity.combined_sigma_agreement(e1, parity.tally_variance(e1, q1, n), e2,
                                                 parity.tally_variance(e2, q2, n))
    print(f"modified table: {frac:.4f} of {nvox} voxels within 3 sigma, "
          f"model/modified energy {e0.sum() / e1.sum():.4f}")
    assert nvox > 2000 and frac >= 0.99
    tol = parity.total_tolerance(gw, beam, lambda r: gpu.run_options(seed=100 + r, stream=0))
    parity.assert_totals_agree(e1, e2, tol, "modified table")
    assert abs(e0.sum() / e1.sum() - 1) > 0.01  # oxygen's photoelectric x 1.5 shows in the dose
