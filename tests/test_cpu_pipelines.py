"""CPU tests of the passes around the transport: the library's host-side CT-number
table against the oracle restatement, and the restatement's own edge cases
(ctsegmentationpipeline.cpp:59-160, dosetablepipeline.cpp:55-85,
simulationpipeline.cpp:173-231)."""
import numpy as np
import pytest

from opendxmc_gb300 import phantoms as P

MATS = [(c, d) for _, c, d in P.SEGMENTATION_MATERIALS]


@pytest.mark.parametrize("kvp,al,sn", [(120.0, 0.0, 0.0), (80.0, 2.5, 0.0), (140.0, 6.0, 0.4)])
def test_segmentation_table_matches_oracle(engine, kvp, al, sn):
    from oracle import pipelines as OP

    t = engine.ct_segmentation_table(kvp, al, sn)
    ref = OP.ct_segmentation_table(kvp, al, sn, MATS)
    n = len(MATS)
    assert t.n_materials == n
    np.testing.assert_allclose(list(t.hu)[:n], ref["hu"], rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(list(t.attenuation)[:n], ref["attenuation"], rtol=1e-12)
    np.testing.assert_allclose(list(t.separator)[:n - 1], ref["separator"], rtol=1e-12, atol=1e-9)
    assert abs(t.water_attenuation / ref["water_attenuation"] - 1) < 1e-12
    assert abs(t.air_attenuation / ref["air_attenuation"] - 1) < 1e-12
    # the pipeline's five materials come out in ascending CT number, air near -1000
    hu = list(t.hu)[:n]
    assert all(a < b for a, b in zip(hu, hu[1:]))
    assert -1001.0 < hu[0] < -990.0


def test_segmentation_table_rejects_bad_input(engine):
    from opendxmc_gb300 import native as N

    with pytest.raises(N.DxmcgError):
        engine.ct_segmentation_table(0.5)
    with pytest.raises(N.DxmcgError):
        engine.ct_segmentation_table(120.0, materials=[({1: 1.0}, -1.0)])
    with pytest.raises(N.DxmcgError):
        engine.ct_segmentation_table(120.0, materials=[({1: 1.0}, 1.0)] * 65)


def test_oracle_segment_edges():
    from oracle import pipelines as OP

    table = OP.ct_segmentation_table(120.0, 0.0, 0.0, MATS)
    sep = table["separator"]
    hu = np.array([-2000.0, sep[0], np.nextafter(sep[0], -np.inf), sep[-1], 5000.0, np.nan])
    m, d = OP.ct_segment(table, hu)
    assert list(m) == [0, 1, 0, 4, 4, 4]  # hu == separator goes up; NaN falls through to the last
    assert d[0] == 0.0  # clamped
    assert np.isnan(d[-1])


def test_oracle_organ_table_and_postprocess():
    from oracle import pipelines as OP

    organ = np.array([0, 0, 1, 1, 1, 3, 9], dtype=np.uint8)
    dose = np.array([1.0, 2.0, 3.0, 3.0, 3.0, 0.5, 7.0])
    dens = np.array([0.001, 0.001, 1.0, 2.0, 1.0, 1.5, 1.0])
    t = OP.organ_dose_table(organ, dose, dens, (0.1, 0.2, 0.5), 4)
    assert list(t["n_voxels"]) == [2, 3, 0, 1]  # label 9 >= n_organs: ignored
    assert t["dose"][1] == pytest.approx(3.0)
    assert t["mass_g"][1] == pytest.approx(0.01 * 4.0)
    assert t["dose"][2] == 0.0
    d, v, c, micro = OP.dose_postprocess([0.1, 0.5], [1e-4, 2e-4], [3, 4], [0, 1])
    assert micro and list(d) == [0.0, 500.0] and list(c) == [0.0, 4.0]
    assert v[1] == pytest.approx(200.0)
