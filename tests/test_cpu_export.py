"""Study export in OpenDXMC's HDF5 layout (opendxmc_gb300/export.py): dataset names,
beam groups, attribute names and element types equal those the reference writes
(hdf5wrapper.cpp, extracted into tests/golden/reference_data.json by
tests/golden/make_golden.py); values round-trip through the archive.  No GPU."""
import json
from pathlib import Path

import numpy as np
import pytest

from opendxmc_gb300 import export as X
from opendxmc_gb300 import phantoms as P

LAYOUT = json.loads((Path(__file__).parent / "golden" / "reference_data.json").read_text())["hdf5_layout"]

FULL_BEAMS = {
    "DXBeams": dict(P.dx_beam_params(), rotation_center=[0.0, 0.0, 0.0], source_center_distance=100.0,
                    primary_angle=0.0, secondary_angle=0.0, sdd_cm=110.0, dap_mgycm2=1500.0),
    "CTSpiralBeams": dict(P.ct_spiral_params(), organ_aec=1, organ_aec_start_deg=30.0, organ_aec_stop_deg=150.0,
                          organ_aec_ramp_deg=20.0, organ_aec_low_weight=0.6, ctdi_vol_mgy=10.0),
    "CTSequentialBeams": {"type": 2, "kvp": 120.0, "filters": {13: 6.0, 50: 0.4}, "particles_per_exposure": 1000,
                          "start": [0, 0, -2], "rotation_axis": [0, 0, 1], "scan_fov_cm": 50.0, "sdd_cm": 119.0,
                          "collimation_cm": 4.0, "start_angle_deg": 0.0, "step_angle_deg": 5.0, "n_slices": 3,
                          "slice_spacing_cm": 4.0, "ctdi_w_mgy": 12.0, "ctdi_diameter_cm": 32.0},
    "CBCTBeams": {"type": 3, "kvp": 90.0, "filters": {13: 3.0}, "particles_per_exposure": 1000,
                  "position": [0, 0, 0], "sdd_cm": 120.0, "start_angle_deg": -90.0, "stop_angle_deg": 90.0,
                  "step_angle_deg": 1.0, "half_angles": [0.1, 0.08], "dap_mgycm2": 800.0},
    "CTSpiralDualEnergyBeams": dict(P.ct_spiral_params(), type=5, kvp_b=140.0, filters_b={13: 6.0, 50: 0.4},
                                    fov_b_cm=33.0, tube_a_weight=0.4, ctdi_vol_mgy=8.0),
}


@pytest.mark.parametrize("kind", sorted(FULL_BEAMS))
def test_beam_groups_match_reference_attributes(kind):
    got_kind, attrs = X.beam_attributes(FULL_BEAMS[kind])
    assert got_kind == kind
    ref = LAYOUT["beams"][kind]
    assert set(attrs) == set(ref)
    for name, value in attrs.items():
        kind_of = "uint64" if np.asarray(value).dtype == np.uint64 else "double"
        assert kind_of == ref[name], name


def test_dx_beam_without_pose_angles_leaves_them_out():
    _, attrs = X.beam_attributes(P.dx_beam_params())
    missing = set(LAYOUT["beams"]["DXBeams"]) - set(attrs)
    assert missing == {"rotation_center", "source_center_distance", "primary_angle", "secondary_angle"}


def test_study_datasets_match_reference_and_round_trip(tmp_path):
    ph = P.water_cylinder_phantom(dims=(12, 10, 6), spacing=(0.5, 0.5, 1.0))
    n = ph.n_voxels
    rng = np.random.default_rng(1)
    dose, var, cnt = rng.random(n), rng.random(n) * 1e-3, rng.integers(0, 9, n).astype(float)
    organ = rng.integers(0, 3, n)
    entries = X.study_entries(ph.dims, ph.spacing, density=ph.density, ct=rng.normal(0, 100, n),
                              material=ph.material, organ=organ, organ_names=["a", "b", "c"],
                              materials=ph.materials, material_names=ph.names, dose=dose, variance=var, count=cnt,
                              aec=([1.0, 0.8, 1.2], [0, 0, -5], [0, 0, 5]),
                              beams=[FULL_BEAMS["CTSpiralBeams"], FULL_BEAMS["CTSpiralBeams"], FULL_BEAMS["DXBeams"]])
    datasets = {k for k in entries if not k.startswith("beams/")}
    assert datasets == set(LAYOUT["datasets"])
    assert "beams/CTSpiralBeams/2/pitch" in entries and "beams/DXBeams/1/DAPvalue" in entries
    # volume arrays are flat, x fastest (index = x + nx (y + ny z)), as OpenDXMC stores them
    np.testing.assert_array_equal(entries["materialarray"], ph.material.reshape(-1))
    assert entries["dimensions"].tolist() == list(ph.dims)
    path = tmp_path / "study.npz"
    X.save_npz(path, entries)
    back = X.load_npz(path)
    assert set(back) == set(entries)
    for k, v in entries.items():
        if np.asarray(v).dtype == object:
            assert list(back[k]) == list(v)
        else:
            np.testing.assert_array_equal(back[k], np.asarray(v))


def test_material_composition_strings():
    assert X.composition_string({8: 88.81, 1: 11.19}) == "H11.190000O88.810000"
    assert X.composition_string({"20": 21.3, "6": 15.9}) == "C15.900000Ca21.300000"


def test_volume_size_checked():
    with pytest.raises(ValueError, match="voxels"):
        X.study_entries((2, 2, 2), (1, 1, 1), dose=np.zeros(7))


def test_hdf5_file_where_h5py_exists(tmp_path):
    h5py = pytest.importorskip("h5py")
    entries = X.study_entries((3, 2, 2), (0.1, 0.1, 0.2), dose=np.arange(12.0), beams=[FULL_BEAMS["CBCTBeams"]])
    X.save_hdf5(tmp_path / "s.h5", entries)
    with h5py.File(tmp_path / "s.h5") as f:
        assert f["dosearray"].shape == (3, 2, 2)
        np.testing.assert_array_equal(f["dosearray"][...].reshape(-1), np.arange(12.0))
        assert f["beams/CBCTBeams/1"].attrs["DAPvalue"] == 800.0


def test_study_round_trip_through_the_archive(engine, tmp_path):
    """A study written with save_npz and read with load_study gives back the arrays,
    the material compositions and beams that expand to the same exposures (the loader
    is HDF5Wrapper::load's counterpart, hdf5wrapper.cpp:1070-1207)."""
    ph = P.water_cylinder_phantom(dims=(16, 12, 8), spacing=(0.5, 0.6, 0.7))
    rng = np.random.default_rng(2)
    dose = rng.uniform(0, 1, ph.material.shape)
    beams = [
        dict(P.dx_beam_params(particles=10, exposures=3), rotation_center=[0.0, 0.0, 0.0],
             source_center_distance=100.0, primary_angle=0.0, secondary_angle=0.0, sdd_cm=110.0, dap_mgycm2=5.0),
        dict(P.dx_beam_params(particles=20, exposures=2), rotation_center=[1.0, -2.0, 3.0],
             source_center_distance=80.0, primary_angle=30.0, secondary_angle=-20.0, sdd_cm=100.0),
        P.ct_spiral_params(particles=7, scan_cm=6.0),
        dict(P.ct_spiral_params(particles=7, scan_cm=6.0), organ_aec=1, organ_aec_start_deg=30.0,
             organ_aec_stop_deg=150.0, organ_aec_ramp_deg=20.0, organ_aec_low_weight=0.6),
        P.ct_sequential_params(particles=5),
        P.cbct_params(particles=9),
        P.ct_dual_energy_params(particles=3, scan_cm=4.0, tube_a_weight=0.3),
    ]
    # the DX poses as a caller's DXBeam would have them
    for b in beams[:2]:
        b["position"], b["cosines"] = X._dx_pose(b["rotation_center"], b["source_center_distance"],
                                                 b["primary_angle"], b["secondary_angle"])
    tree = X.study_entries(ph.dims, ph.spacing, density=ph.density, material=ph.material, materials=ph.materials,
                           material_names=ph.names, dose=dose, variance=dose * 0.1, count=np.round(dose * 100),
                           beams=beams)
    X.save_npz(tmp_path / "study.npz", tree)
    st = X.load_study(tmp_path / "study.npz")
    assert st["dims"] == tuple(ph.dims) and st["spacing"] == pytest.approx(ph.spacing)
    np.testing.assert_array_equal(st["density"], ph.density)
    np.testing.assert_array_equal(st["material"], ph.material)
    np.testing.assert_array_equal(st["dose"], dose)
    assert st["material_names"] == ph.names
    for got, want in zip(st["materials"], ph.materials):
        assert set(got) == set(want)
        s_got, s_want = sum(got.values()), sum(want.values())
        for z in want:
            assert got[z] / s_got == pytest.approx(want[z] / s_want, abs=1e-6)
    assert len(st["beams"]) == len(beams)
    # group order is DX, spiral, sequential, CBCT, dual energy; beams are listed that way
    for got, want in zip(st["beams"], beams):
        assert got["type"] == want["type"]
        pose = ("rotation_center", "source_center_distance", "primary_angle", "secondary_angle")
        e1 = engine.beam_exposures({k: v for k, v in want.items() if k not in pose})
        e2 = engine.beam_exposures({k: v for k, v in got.items() if k not in pose})
        assert len(e1) == len(e2)
        for a, b in zip(e1, e2):
            for k in ("pos", "c0", "c1", "half"):
                np.testing.assert_allclose(b[k], a[k], rtol=1e-9, atol=1e-9, err_msg=k)
            assert b["weight"] == pytest.approx(a["weight"], rel=1e-9)
            assert b["tube"] == a["tube"]
        assert got["particles_per_exposure"] == want["particles_per_exposure"]
        for k in ("kvp", "kvp_b", "pitch", "collimation_cm", "sdd_cm", "tube_a_weight"):
            if k in want:
                assert got[k] == pytest.approx(want[k]), k
        assert got["filters"] == {int(z): float(v) for z, v in want["filters"].items()}
