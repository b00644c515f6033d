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
same tree where the h5py package is installed.  `load_npz` reads an archive back, and
`study_from_entries` / `load_study` turn a tree into arrays, material compositions
and beam descriptions the library takes, as HDF5Wrapper::load does for OpenDXMC
(hdf5wrapper.cpp:1070-1207).
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
        a["start_position"] = vec("position") if "position" in beam else vec("start")
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


def parse_composition(text: str) -> dict:
    """{Z: weight} of a materialcomposition entry (composition_string's inverse)."""
    import re

    out = {}
    for sym, w in re.findall(r"([A-Z][a-z]?)([0-9]+(?:\.[0-9]*)?)", str(text)):
        out[SYMBOLS.index(sym) + 1] = float(w)
    return out


def _rotate(v, axis, angle):
    """v rotated by `angle` (rad) about the unit vector `axis` (Rodrigues)."""
    v, k = np.asarray(v, dtype=np.float64), np.asarray(axis, dtype=np.float64)
    c, s = np.cos(angle), np.sin(angle)
    return v * c + np.cross(k, v) * s + k * np.dot(k, v) * (1.0 - c)


def _dx_pose(center, distance, primary_deg, secondary_deg):
    """Source position and direction cosines of a DX beam from its rotation centre,
    source-patient distance and angles, as DXBeam::updatePosition computes them
    (dxmc_specialization.cpp:78-90): the cosines (0, 0, 1), (-1, 0, 0) turned about z by
    the primary angle, then about -x by the secondary angle; the source sits `distance`
    back along c0 x c1 from the centre."""
    c0 = _rotate([0.0, 0.0, 1.0], [0.0, 0.0, 1.0], np.radians(primary_deg))
    c1 = _rotate([-1.0, 0.0, 0.0], [0.0, 0.0, 1.0], np.radians(primary_deg))
    c0 = _rotate(c0, [-1.0, 0.0, 0.0], np.radians(secondary_deg))
    c1 = _rotate(c1, [-1.0, 0.0, 0.0], np.radians(secondary_deg))
    d = np.cross(c0, c1)
    pos = np.asarray(center, dtype=np.float64) - d * float(distance)
    return [float(x) for x in pos], [[float(x) for x in c0], [float(x) for x in c1]]


def _beam_from_attributes(kind: str, a: dict) -> dict:
    """A beam description in the library's keys from one stored beam group (the
    inverse of beam_attributes for the values the group carries)."""
    t = {v: k for k, v in BEAM_GROUPS.items()}[kind]
    f = lambda k, d=0.0: float(np.asarray(a.get(k, d)))  # noqa: E731
    vec = lambda k: [float(x) for x in np.asarray(a.get(k, (0.0, 0.0, 0.0)), dtype=np.float64)]  # noqa: E731

    def filters(suffix=""):
        out = {}
        for Z, name in ((13, "Al"), (29, "Cu"), (50, "Sn")):
            v = f(f"tube_{name}_filtration{suffix}")
            if v > 0:
                out[Z] = v
        return out

    b: dict = {"type": t, "anode_angle_deg": f("tube_anode_angle", 12.0),
               "particles_per_exposure": int(np.asarray(a.get("particles_per_exposure", 0)))}
    if t in (0, 3):
        b["kvp"] = f("tube_voltage")
        b["filters"] = filters()
        b["sdd_cm"] = f("source_detector_distance")
        b["half_angles"] = [float(x) for x in np.radians(np.asarray(a.get("collimation_half_angles", (0.0, 0.0)),
                                                                       dtype=np.float64))]
        b["dap_mgycm2"] = f("DAPvalue")
        if t == 0:
            b["n_exposures"] = int(np.asarray(a.get("number_of_exposures", 1)))
            for k in ("source_center_distance", "primary_angle", "secondary_angle"):
                if k in a:
                    b[k] = f(k)
            if "rotation_center" in a:
                b["rotation_center"] = vec("rotation_center")
            b["position"], b["cosines"] = _dx_pose(b.get("rotation_center", [0.0, 0.0, 0.0]),
                                                   b.get("source_center_distance", 0.0),
                                                   b.get("primary_angle", 0.0), b.get("secondary_angle", 0.0))
        else:
            b["position"] = vec("isocenter")
            b["rotation_axis"] = [0.0, 0.0, 1.0]
            for k in ("start_angle", "stop_angle", "step_angle"):
                b[k + "_deg"] = f(k)
        return b
    b["sdd_cm"] = f("source_detector_distance")
    b["collimation_cm"] = f("collimation")
    b["start_angle_deg"] = f("start_angle")
    b["step_angle_deg"] = f("step_angle")
    b["ctdi_diameter_cm"] = f("CTDIdiameter", 32.0)
    if t == 2:
        b["kvp"] = f("tube_voltage")
        b["filters"] = filters()
        b["position"] = vec("start_position")
        b["rotation_axis"] = vec("scan_normal")
        b["scan_fov_cm"] = f("scan_field_view")
        b["slice_spacing_cm"] = f("slice_spacing")
        b["n_slices"] = int(np.asarray(a.get("number_of_slices", 1)))
        b["ctdi_w_mgy"] = f("CTDIw")
        return b
    b["start"] = vec("start_position")
    b["stop"] = vec("stop_position")
    b["pitch"] = f("pitch", 1.0)
    b["ctdi_vol_mgy"] = f("CTDIvol")
    if t == 1:
        b["kvp"] = f("tube_voltage")
        b["filters"] = filters()
        b["scan_fov_cm"] = f("scan_field_view")
    else:
        b["kvp"] = f("tube_voltageA")
        b["filters"] = filters("A")
        b["kvp_b"] = f("tube_voltageB")
        b["filters_b"] = filters("B")
        b["scan_fov_cm"] = f("scan_field_viewA")
        b["fov_b_cm"] = f("scan_field_viewB")
        ma, mb = f("tube_masA", 0.5), f("tube_masB", 0.5)
        b["tube_a_weight"] = ma / (ma + mb) if ma + mb > 0 else 0.5
    if int(np.asarray(a.get("use_organ_aec", 0))):
        b["organ_aec"] = 1
        b["organ_aec_compensate"] = int(np.asarray(a.get("compensate_weight_organ_aec", 0)))
        b["organ_aec_low_weight"] = f("low_weight_organ_aec", 1.0)
        ssr = np.asarray(a.get("start_stop_ramp_angle_organ_aec", (0.0, 0.0, 0.0)), dtype=np.float64)
        b["organ_aec_start_deg"], b["organ_aec_stop_deg"], b["organ_aec_ramp_deg"] = (float(x) for x in ssr)
    return b


def study_from_entries(entries: dict) -> dict:
    """The study in a stored tree: dims (nx, ny, nz), spacing (cm), the volume arrays
    present (shape (nz, ny, nx), x fastest, as the library and the phantoms use them),
    material names and compositions ({Z: weight}), organ names, the AEC profile and
    the beams (library beam descriptions, in their group order)."""
    dims = tuple(int(d) for d in np.asarray(entries["dimensions"]))
    study: dict = {"dims": dims, "spacing": tuple(float(x) for x in np.asarray(entries["spacing"]))}
    shape = dims[::-1]
    for key, name in (("densityarray", "density"), ("ctarray", "ct"), ("materialarray", "material"),
                      ("organarray", "organ"), ("dosearray", "dose"), ("dosevariancearray", "variance"),
                      ("doseeventcountarray", "count")):
        if key in entries:
            study[name] = np.asarray(entries[key]).reshape(shape)
    if "materialnames" in entries:
        study["material_names"] = [str(x) for x in entries["materialnames"]]
    if "materialcomposition" in entries:
        study["materials"] = [parse_composition(x) for x in entries["materialcomposition"]]
    if "organnames" in entries:
        study["organ_names"] = [str(x) for x in entries["organnames"]]
    if "aecweights" in entries:
        study["aec"] = (np.asarray(entries["aecweights"]), np.asarray(entries["aecstart"]),
                        np.asarray(entries["aecstop"]))
    groups: dict = {}
    for k, v in entries.items():
        if k.startswith("beams/"):
            _, kind, n, attr = k.split("/", 3)
            groups.setdefault((kind, int(n)), {})[attr] = v
    order = sorted(groups, key=lambda kn: (list(BEAM_GROUPS.values()).index(kn[0]), kn[1]))
    study["beams"] = [_beam_from_attributes(kind, groups[(kind, n)]) for kind, n in order]
    return study


def load_study(path) -> dict:
    """study_from_entries of an archive written by save_npz."""
    return study_from_entries(load_npz(path))
