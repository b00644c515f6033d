"""Shared helpers for the parity tests: input builders and the statistical
comparison used between the GPU engine and the CPU oracle."""
from __future__ import annotations

import numpy as np

from opendxmc_gb300 import phantoms as P


def uniforms_f32_exact(rng: np.random.Generator, shape) -> np.ndarray:
    """Uniforms of the engine's form (2k+1)/2^24, exactly representable in FP32 and
    FP64, so injected variates are identical on both sides."""
    k = rng.integers(0, 1 << 23, size=shape, dtype=np.int64)
    return (2 * k + 1).astype(np.float64) / float(1 << 24)


def combined_sigma_agreement(e1, v1, e2, v2, frac_of_max=0.05, k_sigma=3.0):
    """Fraction of voxels above `frac_of_max` of the maximum whose difference lies
    within k combined standard errors, and the number of such voxels."""
    thr = frac_of_max * max(e1.max(), e2.max())
    mask = (e1 > thr) | (e2 > thr)
    sig = np.sqrt(np.maximum(v1, 0) + np.maximum(v2, 0))
    ok = np.abs(e1 - e2) <= k_sigma * sig
    return float(ok[mask].mean()), int(mask.sum())


def tally_variance(e, e2, n_hist):
    """Variance of the per-voxel energy sum estimated from per-event sums."""
    return np.maximum(e2 - e * e / float(n_hist), 0.0)


def small_cylinder(scale=2):
    """The 128x128x64 water/bone cylinder at a coarser grid (fast on the CPU)."""
    return P.water_cylinder_phantom(dims=(128 // scale, 128 // scale, 64 // scale),
                                    spacing=(0.1 * scale, 0.1 * scale, 0.25 * scale))


def small_torso(scale=4, seed=3):
    return P.torso_phantom(dims=(256 // scale, 256 // scale, 200 // scale),
                           spacing=(0.15 * scale, 0.15 * scale, 0.15 * scale), seed=seed)



def replicate_totals(world, beam, options_for, k=8):
    """Runs the whole beam k times on independent streams (options_for(r) -> run
    options of replicate r) into the world's tally (cleared first) and returns each
    replicate's deposited energy: their sum is the total of k x the beam's histories,
    and total_sigma estimates its standard error."""
    world.clear()
    return np.array([world.run(beam, options_for(r))["e_deposited"] for r in range(k)])


def total_sigma(totals) -> float:
    """Standard error of the sum of independent, identically distributed totals."""
    b = np.asarray(totals, dtype=np.float64)
    return float(np.sqrt(b.size * np.var(b, ddof=1)))


def total_tolerance(world, beam, options_for, k=32, n_sigma=4.0) -> float:
    """Relative tolerance for the difference of two independent runs' totals of one
    beam: n_sigma standard errors of that difference, sqrt(2) x the spread of a run's
    deposited energy over k replicate runs on the GPU world (options_for(r) gives
    replicate r's independent stream).  The world's tally is cleared afterwards."""
    world.clear()
    t = np.array([world.run(beam, options_for(r))["e_deposited"] for r in range(k)])
    world.clear()
    return float(n_sigma * np.sqrt(2.0) * t.std(ddof=1) / t.mean())


def assert_totals_agree(e_gpu, e_oracle, tol, name="", resolve=3e-3):
    """Total energy imparted of independent GPU and oracle runs: the difference
    within `tol` (total_tolerance), and `tol` no wider than `resolve`, so the test
    can see a bias of that size."""
    rel = float(np.sum(e_gpu) / np.sum(e_oracle) - 1.0)
    print(f"{name}: total GPU/oracle - 1 = {rel:+.2e}, tolerance {tol:.2e} (4 standard errors)")
    assert abs(rel) <= tol, (name, rel, tol)
    assert tol <= resolve, (name, tol)
