"""CPU restatement (numpy, FP64) of the per-voxel passes around the transport.

TEST INFRASTRUCTURE ONLY: the tests compare the GPU passes with these functions.
The product never imports this module.  Each function follows the reference file
and lines it cites; the physics behind the tables (attenuation, tube spectrum) is
the oracle's own, so, like the transport, these are PARITY UNPINNED against
DXMClib, whose tables are not available.
"""
from __future__ import annotations

import numpy as np

from . import oracle as O

WATER = {1: 11.19, 8: 88.81}
DRY_AIR = {7: 75.5, 8: 23.2, 18: 1.3}
WATER_DENSITY = 1.0
AIR_DENSITY = 0.001205


def ct_segmentation_table(kvp, al_mm, sn_mm, materials):
    """getMeanCTNumbers (ctsegmentationpipeline.cpp:59-111): spectrum-weighted mean
    CT number and mass attenuation of each (composition, density), with the mean
    attenuation of water and air; separators are the midpoints (:129-133)."""
    E, w = O.tube_spectrum(kvp, {13: max(0.0, al_mm), 50: max(0.0, sn_mm)})
    uw = sum(O.attenuation(WATER, E, 1))
    ua = sum(O.attenuation(DRY_AIR, E, 1))
    out = {"hu": [], "attenuation": [], "water_attenuation": 0.0, "air_attenuation": 0.0,
           "water_density": WATER_DENSITY, "air_density": AIR_DENSITY}
    for k in range(E.size):  # sequential sums, in the library's order
        out["water_attenuation"] += w[k] * uw[k]
        out["air_attenuation"] += w[k] * ua[k]
    for comp, dens in materials:
        um = sum(O.attenuation(comp, E, 1))
        hu = 0.0
        att = 0.0
        for k in range(E.size):
            hu += w[k] * (um[k] * dens - uw[k] * WATER_DENSITY) / (uw[k] * WATER_DENSITY - ua[k] * AIR_DENSITY)
            att += w[k] * um[k]
        out["hu"].append(1000.0 * hu)
        out["attenuation"].append(att)
    out["separator"] = [(a + b) / 2 for a, b in zip(out["hu"][:-1], out["hu"][1:])]
    return out


def ct_segment(table, hu):
    """The per-voxel transforms of CTSegmentationPipeline::updateImageData
    (ctsegmentationpipeline.cpp:135-157): material = first i with hu < separator[i],
    else the last; density = (((w_att w_dens - a_att a_dens) hu / 1000) + w_att
    w_dens) / m_att, clamped at 0 (a NaN stays NaN, as std::max keeps it)."""
    h = np.asarray(hu, dtype=np.float64)
    sep = np.asarray(table["separator"], dtype=np.float64)
    mat = np.zeros(h.shape, dtype=np.uint8)
    undecided = np.ones(h.shape, dtype=bool)
    for i, s in enumerate(sep):
        hit = undecided & (h < s)
        mat[hit] = i
        undecided &= ~hit
    mat[undecided] = len(sep)
    slope = table["water_attenuation"] * table["water_density"] - table["air_attenuation"] * table["air_density"]
    offset = table["water_attenuation"] * table["water_density"]
    att = np.asarray(table["attenuation"], dtype=np.float64)[mat]
    dens = ((slope * h) / 1000.0 + offset) / att
    dens = np.where(dens < 0.0, 0.0, dens)
    return mat, dens


def organ_dose_table(organ, dose, density, spacing_cm, n_organs):
    """DoseTablePipeline::updateImageData (dosetablepipeline.cpp:58-83): per organ
    label, voxels, volume, mass = V sum(density), dose = sum(dose V density) / mass."""
    V = float(np.prod(spacing_cm))
    o = np.asarray(organ).reshape(-1)
    e = np.asarray(dose, dtype=np.float64).reshape(-1) * (V * np.asarray(density, dtype=np.float64).reshape(-1))
    r = np.asarray(density, dtype=np.float64).reshape(-1)
    out = {k: np.zeros(n_organs) for k in ("volume_cm3", "mass_g", "dose")}
    out["n_voxels"] = np.zeros(n_organs, dtype=np.uint64)
    for i in range(n_organs):
        sel = o == i
        n = int(sel.sum())
        if n == 0:
            continue
        out["n_voxels"][i] = n
        out["volume_cm3"][i] = n * V
        out["mass_g"][i] = V * r[sel].sum()
        out["dose"][i] = e[sel].sum() / out["mass_g"][i]
    return out


def dose_postprocess(dose, variance, count, material, delete_air_dose=True):
    """The worker's readout (simulationpipeline.cpp:173-231): zero material-0 voxels,
    switch to uGy (dose x 1e3, variance x 1e6) when the maximum dose is below 1."""
    d = np.asarray(dose, dtype=np.float64).copy()
    v = np.asarray(variance, dtype=np.float64).copy()
    c = np.asarray(count, dtype=np.float64).copy()
    if delete_air_dose:
        air = np.asarray(material) == 0
        d[air] = 0.0
        v[air] = 0.0
        c[air] = 0.0
    micro = bool(d.max() < 1) if d.size else True
    if micro:
        d *= 1e3
        v *= 1e6
    return d, v, c, micro
