"""Seeded synthetic phantoms and the tissue compositions they use.

Compositions are mass percentages per element (Z -> %), the rows of the ICRP
adult-male media table OpenDXMC ships (data/phantoms/icrp/AM/AM_media.dat) and
of data/phantoms/other/media.dat; the line of each row is cited.  Arrays are
returned in the AAVoxelGrid layout: shape (nz, ny, nx), x fastest, grid centred
on the origin, spacing in cm.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

AIR = {7: 80.0, 8: 20.0}  # AM_media.dat:56 "Air"
LUNG = {1: 10.3, 6: 10.7, 7: 3.2, 8: 74.6, 11: 0.2, 15: 0.2, 16: 0.3, 17: 0.3, 19: 0.2}  # AM_media.dat:53
ADIPOSE = {1: 11.4, 6: 58.8, 7: 0.8, 8: 28.7, 11: 0.1, 16: 0.1, 17: 0.1}  # AM_media.dat:52
SOFT_TISSUE = {1: 10.4, 6: 23.1, 7: 2.8, 8: 62.7, 11: 0.1, 15: 0.2, 16: 0.3, 17: 0.2, 19: 0.2}  # AM_media.dat:48
MUSCLE = {1: 10.2, 6: 14.2, 7: 3.4, 8: 71.1, 11: 0.1, 15: 0.2, 16: 0.3, 17: 0.1, 19: 0.4}  # AM_media.dat:32
BONE = {1: 3.6, 6: 15.9, 7: 4.2, 8: 44.8, 11: 0.3, 12: 0.2, 15: 9.4, 16: 0.3, 20: 21.3}  # AM_media.dat:5
WATER = {1: 11.2, 8: 88.8}  # other/media.dat:56

# the six-material set: (name, composition, nominal density g/cm3)
SIX_MATERIALS = [
    ("air", AIR, 0.0012),
    ("lung", LUNG, 0.26),
    ("adipose", ADIPOSE, 0.95),
    ("soft_tissue", SOFT_TISSUE, 1.03),
    ("muscle", MUSCLE, 1.05),
    ("bone", BONE, 1.92),
]


# The five materials CTSegmentationPipeline segments CT numbers into
# (ctsegmentationpipeline.cpp:120-127): air, adipose, soft tissue, muscle and cortical
# bone, with bone's density lowered to 1.09 g/cm3 as there.  DXMClib's NIST
# compositions are not available here; the ICRP media rows above stand in for them.
SEGMENTATION_MATERIALS = [
    ("Air, Dry (near sea level)", AIR, 0.001205),
    ("Adipose Tissue (ICRP)", ADIPOSE, 0.95),
    ("Tissue, Soft (ICRP)", SOFT_TISSUE, 1.03),
    ("Muscle, Skeletal", MUSCLE, 1.04),
    ("Bone, Cortical (ICRP)", BONE, 1.09),
]


@dataclass
class Phantom:
    dims: tuple  # (nx, ny, nz)
    spacing: tuple  # cm
    density: np.ndarray  # float64 (nz, ny, nx)
    material: np.ndarray  # uint8 (nz, ny, nx)
    materials: list  # list of {Z: weight}
    names: list = field(default_factory=list)

    @property
    def n_voxels(self) -> int:
        return int(np.prod(self.dims))


def _axes(dims, spacing):
    nx, ny, nz = dims
    sx, sy, sz = spacing
    x = (np.arange(nx) + 0.5) * sx - 0.5 * nx * sx
    y = (np.arange(ny) + 0.5) * sy - 0.5 * ny * sy
    z = (np.arange(nz) + 0.5) * sz - 0.5 * nz * sz
    return x, y, z


def water_cylinder_phantom(dims=(128, 128, 64), spacing=(0.1, 0.1, 0.25)) -> Phantom:
    """Air (0.0012) holding a water cylinder, 16 cm diameter and 15 cm long along z,
    with a 3 cm diameter bone insert (1.92 g/cm3) centred 4 cm off axis."""
    x, y, z = _axes(dims, spacing)
    X, Y = np.meshgrid(x, y)  # (ny, nx)
    in_z = np.abs(z) <= 7.5
    cyl = X ** 2 + Y ** 2 <= 8.0 ** 2
    ins = (X - 4.0) ** 2 + Y ** 2 <= 1.5 ** 2
    mat2d = np.where(ins, 2, np.where(cyl, 1, 0)).astype(np.uint8)
    material = np.where(in_z[:, None, None], mat2d[None], 0).astype(np.uint8)
    dens_of = np.array([0.0012, 1.0, 1.92])
    density = dens_of[material]
    return Phantom(tuple(dims), tuple(spacing), density, material, [AIR, WATER, BONE], ["air", "water", "bone"])


def torso_phantom(dims=(256, 256, 200), spacing=(0.15, 0.15, 0.15), seed=1, jitter=0.02) -> Phantom:
    """Seeded nested-ellipsoid torso in the six materials (air, lung, adipose, soft
    tissue, muscle, bone), density x U(1 - jitter, 1 + jitter) per voxel."""
    rng = np.random.default_rng(seed)
    x, y, z = _axes(dims, spacing)
    nx, ny, nz = dims

    def perturb(c, a, dc=0.4, da=0.05):
        c = np.asarray(c, float) + rng.normal(0, dc, 3)
        a = np.asarray(a, float) * rng.uniform(1 - da, 1 + da, 3)
        return c, a

    # (material index, centre, semi-axes); later entries overwrite earlier ones
    shapes = [
        (2, *perturb((0, 0, 0), (15.0, 10.5, 1e4), dc=0.2)),      # body: adipose
        (4, *perturb((0, 0, 0), (13.6, 9.2, 1e4), dc=0.2)),       # muscle wall
        (3, *perturb((0, 0.3, 0), (12.4, 8.1, 1e4), dc=0.2)),     # visceral soft tissue
        (1, *perturb((-6.0, 0.8, 5.0), (4.6, 5.8, 11.0))),        # lungs
        (1, *perturb((6.0, 0.8, 5.0), (4.6, 5.8, 11.0))),
        (4, *perturb((1.5, -0.5, 3.0), (4.0, 3.6, 5.0))),         # heart (muscle)
        (3, *perturb((-4.0, 1.0, -7.0), (6.0, 4.5, 6.0))),        # liver-like soft tissue
        (2, *perturb((3.0, 2.0, -9.0), (3.0, 2.5, 4.0))),         # abdominal fat
        (5, *perturb((0, -6.8, 0), (1.7, 1.5, 1e4), dc=0.1)),     # spine
        (5, *perturb((-8.5, -1.5, -12.0), (3.0, 4.0, 3.5))),      # pelvis
        (5, *perturb((8.5, -1.5, -12.0), (3.0, 4.0, 3.5))),
        (5, *perturb((0, 7.6, 6.0), (1.2, 0.7, 6.0))),            # sternum
    ]
    X, Y = np.meshgrid(x, y)  # (ny, nx)
    material = np.zeros((nz, ny, nx), dtype=np.uint8)
    for k in range(nz):
        sl = np.zeros((ny, nx), dtype=np.uint8)
        for m, c, a in shapes:
            dz = (z[k] - c[2]) / a[2]
            if dz * dz >= 1.0:
                continue
            inside = ((X - c[0]) / a[0]) ** 2 + ((Y - c[1]) / a[1]) ** 2 < 1.0 - dz * dz
            if m == 1:  # lungs stay inside the visceral cavity
                inside &= sl == 3
            sl[inside] = m
        material[k] = sl
    nominal = np.array([d for _, _, d in SIX_MATERIALS])
    density = nominal[material] * rng.uniform(1.0 - jitter, 1.0 + jitter, size=material.shape)
    return Phantom(tuple(dims), tuple(spacing), density, material, [c for _, c, _ in SIX_MATERIALS],
                   [n for n, _, _ in SIX_MATERIALS])


# Body bowtie profile (angle rad, relative weight): "Siemens Definition Flash Body W3
# 120kV", data/bowtiefilters/bowtiefilters.json.template:4-33.
BODY_BOWTIE = [
    (0.0, 1.8816799700821794),
    (0.041992107, 1.7771629567485092),
    (0.083836642, 1.4858913256035922),
    (0.166511074, 0.7320820089981582),
    (0.246954945, 0.47181213705409936),
    (0.324269441, 0.35287338971480264),
    (0.390607044, 0.2984982117986585),
]


def dx_beam_params(kvp=70.0, al_mm=2.5, field_cm=10.0, sid_cm=100.0, particles=1_000_000, exposures=10) -> dict:
    """Planar DX beam as OpenDXMC's DXBeam sets it up at 0/0 degrees: source at
    +y, c0 = +z, c1 = -x, beam along -y (dxmc_specialization.cpp:21-26, :78-90);
    square field of `field_cm` at the isocentre distance, half-angles from
    DXBeam::setCollimation (dxmc_specialization.cpp:46-52)."""
    half = float(np.tan(0.5 * field_cm / sid_cm))
    return {
        "type": 0,
        "kvp": kvp,
        "anode_angle_deg": 12.0,
        "filters": {13: al_mm},
        "particles_per_exposure": particles,
        "n_exposures": exposures,
        "position": [0.0, sid_cm, 0.0],
        "cosines": [[0.0, 0.0, 1.0], [-1.0, 0.0, 0.0]],
        "half_angles": [half, half],
    }


def ct_spiral_params(kvp=120.0, al_mm=6.0, pitch=1.0, collimation_cm=4.0, scan_cm=20.0, sdd_cm=119.0,
                     fov_cm=50.0, step_deg=5.0, particles=1_000_000, bowtie=BODY_BOWTIE) -> dict:
    """CTSpiralBeam with OpenDXMC's defaults (SDD 119 cm, 5 degree step;
    beamsettingsmodel.cpp:1165-1169) over a centred scan range."""
    p = {
        "type": 1,
        "kvp": kvp,
        "anode_angle_deg": 12.0,
        "filters": {13: al_mm},
        "particles_per_exposure": particles,
        "start": [0.0, 0.0, -0.5 * scan_cm],
        "stop": [0.0, 0.0, 0.5 * scan_cm],
        "start_angle_deg": 0.0,
        "step_angle_deg": step_deg,
        "pitch": pitch,
        "collimation_cm": collimation_cm,
        "scan_fov_cm": fov_cm,
        "sdd_cm": sdd_cm,
    }
    if bowtie:
        p["bowtie"] = list(bowtie)
    return p


def ct_sequential_params(kvp=120.0, al_mm=6.0, collimation_cm=4.0, n_slices=3, slice_spacing_cm=4.0,
                         position=(0.0, 0.0, -4.0), sdd_cm=119.0, fov_cm=50.0, step_deg=5.0, particles=1_000_000,
                         bowtie=BODY_BOWTIE) -> dict:
    """CTSequentialBeam: axial rotations at `n_slices` table positions `slice_spacing_cm`
    apart from `position` (beamsettingsmodel.cpp:1654-1837)."""
    p = {
        "type": 2, "kvp": kvp, "anode_angle_deg": 12.0, "filters": {13: al_mm}, "particles_per_exposure": particles,
        "position": list(position), "start_angle_deg": 0.0, "step_angle_deg": step_deg,
        "collimation_cm": collimation_cm, "scan_fov_cm": fov_cm, "sdd_cm": sdd_cm, "n_slices": n_slices,
        "slice_spacing_cm": slice_spacing_cm,
    }
    if bowtie:
        p["bowtie"] = list(bowtie)
    return p


def cbct_params(kvp=90.0, al_mm=4.0, sdd_cm=120.0, start_deg=0.0, stop_deg=200.0, step_deg=2.0,
                half_angles=(0.2, 0.12), particles=1_000_000) -> dict:
    """CBCTBeam: a cone of the given half angles rotating about z in `step_deg` steps
    from `start_deg` to `stop_deg` (addCBCTBeam, beamsettingsmodel.cpp:718-901)."""
    return {"type": 3, "kvp": kvp, "anode_angle_deg": 12.0, "filters": {13: al_mm},
            "particles_per_exposure": particles, "position": [0.0, 0.0, 0.0], "rotation_axis": [0.0, 0.0, 1.0],
            "start_angle_deg": start_deg, "stop_angle_deg": stop_deg, "step_angle_deg": step_deg, "sdd_cm": sdd_cm,
            "half_angles": list(half_angles)}


def ct_dual_energy_params(kvp_a=140.0, kvp_b=80.0, filters_a=None, filters_b=None, pitch=1.0, collimation_cm=4.0,
                          scan_cm=12.0, sdd_cm=119.0, fov_a_cm=50.0, fov_b_cm=33.0, step_deg=5.0, tube_a_weight=0.5,
                          particles=1_000_000, bowtie=BODY_BOWTIE, bowtie_b=BODY_BOWTIE) -> dict:
    """CTSpiralDualEnergyBeam: tubes A and B 90 degrees apart, each with its own
    voltage, filtration, field of view and bowtie (addCTSpiralDualEnergyBeam,
    beamsettingsmodel.cpp:1386-1612)."""
    p = {
        "type": 5, "kvp": kvp_a, "kvp_b": kvp_b, "anode_angle_deg": 12.0,
        "filters": dict(filters_a or {13: 6.0}), "filters_b": dict(filters_b or {13: 6.0, 50: 0.4}),
        "particles_per_exposure": particles, "start": [0.0, 0.0, -0.5 * scan_cm], "stop": [0.0, 0.0, 0.5 * scan_cm],
        "start_angle_deg": 0.0, "step_angle_deg": step_deg, "pitch": pitch, "collimation_cm": collimation_cm,
        "scan_fov_cm": fov_a_cm, "fov_b_cm": fov_b_cm, "sdd_cm": sdd_cm, "tube_a_weight": tube_a_weight,
    }
    if bowtie:
        p["bowtie"] = list(bowtie)
    if bowtie_b:
        p["bowtie_b"] = list(bowtie_b)
    return p


def ellipsoid_phantom(dims, spacing, seed=1, jitter=0.02, n_inserts=8) -> Phantom:
    """Seeded six-material ellipsoid phantom of any grid size: an adipose body
    ellipsoid filling 80-90 % of the grid, a muscle wall and a soft-tissue
    interior, and `n_inserts` random ellipsoids of lung, adipose, muscle or bone
    inside it; density x U(1 - jitter, 1 + jitter) per voxel (float32)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = (int(d) for d in dims)
    x, y, z = _axes((nx, ny, nz), spacing)
    ext = np.array([nx * spacing[0], ny * spacing[1], nz * spacing[2]]) * 0.5
    body = ext * rng.uniform(0.8, 0.9, 3)
    shapes = [(2, np.zeros(3), body), (4, np.zeros(3), body * 0.92), (3, np.zeros(3), body * 0.84)]
    for _ in range(n_inserts):
        m = int(rng.choice([1, 2, 4, 5]))
        a = body * 0.84 * rng.uniform(0.08, 0.3, 3)
        c = body * 0.84 * rng.uniform(-0.6, 0.6, 3)
        shapes.append((m, c, a))
    material = np.zeros((nz, ny, nx), dtype=np.uint8)
    for m, c, a in shapes:
        # evaluate each ellipsoid only over its bounding box
        i0, i1 = np.searchsorted(x, c[0] - a[0]), np.searchsorted(x, c[0] + a[0])
        j0, j1 = np.searchsorted(y, c[1] - a[1]), np.searchsorted(y, c[1] + a[1])
        k0, k1 = np.searchsorted(z, c[2] - a[2]), np.searchsorted(z, c[2] + a[2])
        if i0 >= i1 or j0 >= j1 or k0 >= k1:
            continue
        dx = ((x[i0:i1] - c[0]) / a[0]) ** 2
        dy = ((y[j0:j1] - c[1]) / a[1]) ** 2
        dz = ((z[k0:k1] - c[2]) / a[2]) ** 2
        inside = (dz[:, None, None] + dy[None, :, None] + dx[None, None, :]) < 1.0
        box = material[k0:k1, j0:j1, i0:i1]
        box[inside] = m
    nominal = np.array([d for _, _, d in SIX_MATERIALS], dtype=np.float32)
    density = nominal[material] * rng.uniform(1.0 - jitter, 1.0 + jitter, size=material.shape).astype(np.float32)
    return Phantom((nx, ny, nz), tuple(float(s) for s in spacing), density, material,
                   [c for _, c, _ in SIX_MATERIALS], [n for n, _, _ in SIX_MATERIALS])


def batched_jobs(n_jobs=64, seed=1, dim_range=(64, 320), spacing_cm=(0.1, 0.3), kvp_range=(60.0, 140.0),
                 hist_range=(1e6, 1e8)) -> list[dict]:
    """Seeded specs of independent DX / CBCT jobs: grid dimensions uniform in
    `dim_range` per axis, voxel size uniform in `spacing_cm`, kVp uniform in
    `kvp_range`, histories log-uniform in `hist_range`.  Each spec holds the
    phantom arguments and the beam dict (make the phantom with
    ellipsoid_phantom(spec["dims"], spec["spacing"], spec["seed"]))."""
    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(n_jobs):
        dims = tuple(int(v) for v in rng.integers(dim_range[0], dim_range[1] + 1, 3))
        spacing = tuple(float(v) for v in np.round(rng.uniform(spacing_cm[0], spacing_cm[1], 3), 4))
        kvp = float(np.round(rng.uniform(*kvp_range), 1))
        hist = float(np.exp(rng.uniform(np.log(hist_range[0]), np.log(hist_range[1]))))
        ext = np.array(dims) * np.array(spacing)
        if j % 2 == 0:  # DX, 10 exposures, square field over 70 % of the smaller face
            field = float(np.clip(0.7 * min(ext[0], ext[2]), 2.0, 40.0))
            beam = dx_beam_params(kvp=kvp, al_mm=2.5, field_cm=field, particles=max(1, int(hist / 10)),
                                  exposures=10)
        else:  # CBCT, half rotation in 2 degree steps (91 projections)
            sdd = 120.0
            half_xy = float(np.arctan(0.4 * max(ext[0], ext[1]) / (0.5 * sdd)))
            half_z = float(np.arctan(0.4 * ext[2] / (0.5 * sdd)))
            beam = {"type": 3, "kvp": kvp, "anode_angle_deg": 12.0, "filters": {13: 4.0},
                    "particles_per_exposure": max(1, int(hist / 91)), "position": [0.0, 0.0, 0.0],
                    "rotation_axis": [0.0, 0.0, 1.0], "start_angle_deg": 0.0, "stop_angle_deg": 180.0,
                    "step_angle_deg": 2.0, "sdd_cm": sdd, "half_angles": [half_xy, half_z]}
        jobs.append({"dims": dims, "spacing": spacing, "seed": seed * 1000 + j, "kvp": kvp, "beam": beam})
    return jobs
