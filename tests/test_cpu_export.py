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
