"""Study export in the layout of OpenDXMC's HDF5 files.

OpenDXMC saves a study with HDF5Wrapper::save (src/libopendxmc/hdf5wrapper.cpp:384-457):
root datasets `dimensions`, `spacing`, the volume arrays (`densityarray`, `ctarray`,
`materialarray`, `organarray`, `dosearray`, `dosevariancearray`,
`doseeventcountarray`) whose dataspace is the dimensions (nx, ny, nz) over the flat
x-fastest buffer, the string lists `organnames`, `materialnames` and
`materialcomposition` (element symbol followed by the weight with six decimals, for
each element), the AEC profile (`aecweights`, `aecstart`, `aecstop`), and one group per
beam, /beams/<Kind>Beams/<n> (n from 1), whose values are attributes
(hdf5wrapper.cpp:460-627).

`study_entries` builds that tree as a flat mapping of path -> numpy array (datasets)
or, for beam groups, path/attribute -> value.  `save_npz` stores it in one .npz
archive with the HDF5 paths as keys.  `save_hdf5` writes a real HDF5 file with the
same tree where the h5py package is installed.  `load_npz` reads an archive back.
"""
from __future__ import annotations

import numpy as np

# element symbols, Z = 1..92
SYMBOLS = ("H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr "
           "Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb "
           "Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U").split()

BEAM_GROUPS = {0: "DXBeams", 1: "CTSpiralBeams", 2: "CTSequentialBeams", 3: "CBCTBeams", 5: "CTSpiralDualEnergyBeams"}


def composition_string(zw: dict) -> str:
    """The materialcomposition entry of a material: symbol + weight (%.6f) per element,
    in ascending Z (hdf5wrapper.cpp:423-431 iterates the material's Z -> weight map)."""
    return "".join(f"{SYMBOLS[int(z) - 1]}{float(w):.6f}" for z, w in sorted(zw.items(), key=lambda kv: int(kv[0])))


def _filtration(filters: dict, Z: int) -> float:
    return float(filters.get(Z, filters.get(str(Z), 0.0))) if filters else 0.0


def beam_attributes(beam: dict) -> tuple[str, dict]:
    """(group kind, {attribute: value}) of a beam description as the library takes it
    (the keys of opendxmc_gb300.native.Beam), following hdf5wrapper.cpp:460-627.
    Values the description does not carry (DX rotation centre and angles) are taken
    from optional keys of the same name and otherwise left out."""
    t = int(beam.get("type", 0))
    if t not in BEAM_GROUPS:
        raise ValueError(f"beam type {t} has no group in the study layout")
    f = beam.get("filters", {})
    a: dict = {}
    u64 = np.uint64

    def tube(suffix="", filters=f, kvp=beam.get("kvp", 0.0)):
        a["tube_voltage" + suffix] = float(kvp)
        a["tube_Al_filtration" + suffix] = _filtration(filters, 13)
        a["tube_Cu_filtration" + suffix] = _filtration(filters, 29)
        a["tube_Sn_filtration" + suffix] = _filtration(filters, 50)

    def organ_aec():
        a["use_organ_aec"] = u64(1 if beam.get("organ_aec") else 0)
        a["compensate_weight_organ_aec"] = u64(1 if beam.get("organ_aec_compensate") else 0)
        a["low_weight_organ_aec"] = float(beam.get("organ_aec_low_weight", 1.0))
        a["start_stop_ramp_angle_organ_aec"] = np.array(
            [beam.get("organ_aec_start_deg", 0.0), beam.get("organ_aec_stop_deg", 0.0),
             beam.get("organ_aec_ramp_deg", 0.0)], dtype=np.float64)

    vec = lambda k: np.asarray(beam.get(k, (0.0, 0.0, 0.0)), dtype=np.float64)  # noqa: E731
    if t == 0:
        for k in ("rotation_center", "source_center_distance", "primary_angle", "secondary_angle"):
            if k in beam:
                a[k] = np.asarray(beam[k], dtype=np.float64) if k == "rotation_center" else float(beam[k])
        a["source_detector_distance"] = float(beam.get("sdd_cm", 0.0))
        a["collimation_half_angles"] = np.degrees(np.asarray(beam.get("half_angles", (0.0, 0.0)), dtype=np.float64))
        a["DAPvalue"] = float(beam.get("dap_mgycm2", 0.0))
        a["number_of_exposures"] = u64(beam.get("n_exposures", 1))
        a["particles_per_exposure"] = u64(beam.get("particles_per_exposure", 0))
        tube()
        a["tube_anode_angle"] = float(beam.get("anode_angle_deg", 12.0))
    elif t == 3:
        a["isocenter"] = vec("position")
        a["source_detector_distance"] = float(beam.get("sdd_cm", 0.0))
        a["start_angle"] = float(beam.get("start_angle_deg", 0.0))
        a["stop_angle"] = float(beam.get("stop_angle_deg", 0.0))
        a["step_angle"] = float(beam.get("step_angle_deg", 0.0))
        a["collimation_half_angles"] = np.degrees(np.asarray(beam.get("half_angles", (0.0, 0.0)), dtype=np.float64))
        a["DAPvalue"] = float(beam.get("dap_mgycm2", 0.0))
        a["particles_per_exposure"] = u64(beam.get("particles_per_exposure", 0))
        tube()
        a["tube_anode_angle"] = float(beam.get("anode_angle_deg", 12.0))
    elif t == 2:
        a["start_position"] = vec("start")
        a["scan_normal"] = vec("rotation_axis") if "rotation_axis" in beam else np.array([0.0, 0.0, 1.0])
        a["scan_field_view"] = float(beam.get("fov_cm", beam.get("scan_fov_cm", 0.0)))
        a["source_detector_distance"] = float(beam.get("sdd_cm", 0.0))
        a["collimation"] = float(beam.get("collimation_cm", 0.0))
        a["start_angle"] = float(beam.get("start_angle_deg", 0.0))
        a["step_angle"] = float(beam.get("step_angle_deg", beam.get("step_deg", 0.0)))
        a["slice_spacing"] = float(beam.get("slice_spacing_cm", 0.0))
        a["CTDIw"] = float(beam.get("ctdi_w_mgy", 0.0))
        a["CTDIdiameter"] = float(beam.get("ctdi_diameter_cm", 32.0))
        tube()
        a["tube_anode_angle"] = float(beam.get("anode_angle_deg", 12.0))
        a["particles_per_exposure"] = u64(beam.get("particles_per_exposure", 0))
        a["number_of_slices"] = u64(beam.get("n_slices", 1))
    else:  # spiral (1) and dual-energy spiral (5)
        a["start_position"] = vec("start")
        a["stop_position"] = vec("stop")
        fov = float(beam.get("fov_cm", beam.get("scan_fov_cm", 0.0)))
        if t == 1:
            a["scan_field_view"] = fov
        else:
            a["scan_field_viewA"] = fov
            a["scan_field_viewB"] = float(beam.get("fov_b_cm", fov))
        a["source_detector_distance"] = float(beam.get("sdd_cm", 0.0))
        a["collimation"] = float(beam.get("collimation_cm", 0.0))
        a["start_angle"] = float(beam.get("start_angle_deg", 0.0))
        a["step_angle"] = float(beam.get("step_angle_deg", beam.get("step_deg", 0.0)))
        a["pitch"] = float(beam.get("pitch", 1.0))
        a["CTDIvol"] = float(beam.get("ctdi_vol_mgy", 0.0))
        a["CTDIdiameter"] = float(beam.get("ctdi_diameter_cm", 32.0))
        if t == 1:
            tube()
        else:
            tube("A")
            tube("B", beam.get("filters_b", f), beam.get("kvp_b", beam.get("kvp", 0.0)))
            w = float(beam.get("tube_a_weight", 0.5))
            a["tube_masA"] = w
            a["tube_masB"] = 1.0 - w
        a["tube_anode_angle"] = float(beam.get("anode_angle_deg", 12.0))
        organ_aec()
        a["particles_per_exposure"] = u64(beam.get("particles_per_exposure", 0))
    return BEAM_GROUPS[t], a


def study_entries(dims, spacing_cm, *, density=None, ct=None, material=None, organ=None, organ_names=None,
                  materials=None, material_names=None, dose=None, variance=None, count=None, aec=None,
                  beams=()) -> dict:
    """The study tree: path -> value.  Volume arrays are flattened x-fastest (the
    order of the library and of OpenDXMC's DataContainer) and kept with their
    dimensions; `aec` is (weights, start[3], stop[3]); `materials` a list of {Z: w}."""
    dims = tuple(int(d) for d in dims)
    n = int(np.prod(dims))
    out: dict = {"dimensions": np.asarray(dims, dtype=np.uint64),
                 "spacing": np.asarray(spacing_cm, dtype=np.float64)}

    def volume(name, arr, dtype):
        if arr is None:
            return
        v = np.ascontiguousarray(arr, dtype=dtype).reshape(-1)
        if v.size != n:
            raise ValueError(f"{name}: {v.size} values for {n} voxels")
        out[name] = v

    volume("densityarray", density, np.float64)
    volume("ctarray", ct, np.float64)
    volume("materialarray", material, np.uint8)
    volume("organarray", organ, np.uint8)
    if organ_names:
        out["organnames"] = np.asarray(list(organ_names), dtype=object)
    if materials:
        names = material_names or [f"material {k}" for k in range(len(materials))]
        out["materialnames"] = np.asarray(list(names), dtype=object)
        out["materialcomposition"] = np.asarray([composition_string(m) for m in materials], dtype=object)
    volume("dosearray", dose, np.float64)
    volume("dosevariancearray", variance, np.float64)
    volume("doseeventcountarray", count, np.float64)
    if aec is not None:
        w, start, stop = aec
        out["aecweights"] = np.asarray(w, dtype=np.float64)
        out["aecstart"] = np.asarray(start, dtype=np.float64)
        out["aecstop"] = np.asarray(stop, dtype=np.float64)
    counters: dict = {}
    for b in beams:
        kind, attrs = beam_attributes(b)
        counters[kind] = counters.get(kind, 0) + 1
        for k, v in attrs.items():
            out[f"beams/{kind}/{counters[kind]}/{k}"] = v
    return out


def save_npz(path, entries: dict) -> None:
    np.savez(path, **{k: np.asarray(v) for k, v in entries.items()})


def load_npz(path) -> dict:
    with np.load(path, allow_pickle=True) as z:
        return {k: z[k] for k in z.files}


def save_hdf5(path, entries: dict) -> None:
    """The same tree as an HDF5 file: volume arrays as datasets of shape (nx, ny, nz)
    over the flat buffer, as OpenDXMC writes them; beam values as group attributes.
    Needs h5py."""
    try:
        import h5py
    except ImportError as e:  # the package is optional
        raise RuntimeError("save_hdf5 needs the h5py package; save_npz writes the same tree") from e
    dims = tuple(int(d) for d in entries["dimensions"])
    volumes = {"densityarray", "ctarray", "materialarray", "organarray", "dosearray", "dosevariancearray",
               "doseeventcountarray"}
    with h5py.File(path, "w") as f:
        for k, v in entries.items():
            if k.startswith("beams/"):
                group, attr = k.rsplit("/", 1)
                f.require_group(group).attrs[attr] = v
            elif k in volumes:
                f.create_dataset(k, data=np.asarray(v).reshape(dims), compression="gzip")
            elif np.asarray(v).dtype == object:
                f.create_dataset(k, data=[str(s) for s in v], dtype=h5py.string_dtype())
            else:
                f.create_dataset(k, data=v)
