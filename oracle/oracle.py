"""ctypes binding of the CPU oracle (oracle/dxmc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by the test-suite, the smoke check and the
benchmark's CPU-baseline leg, as the checker.  The product never imports it.
PARITY UNPINNED against DXMClib (absent from the reference tree); see
dxmc_oracle.h.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle_dxmc.so"

NE = 300
EMIN = 1.0
DE = 0.5
MAX_ELEMENTS = 16

TRANSPARENT = 255  # material index that interacts with nothing
TRACK_WOODCOCK = 0
TRACK_SIDDON = 1
TRACK_MACRO = 2
TRACK_WOODCOCK_BOX = 3  # two-region Woodcock
# the transport kernel's default: two-region Woodcock when the box of the voxels whose
# material is neither 0 nor transparent holds less than this share of the grid
TWO_REGION_BOX_FRACTION = 0.5
BEAM_DX, BEAM_CT_SPIRAL, BEAM_CT_SEQUENTIAL, BEAM_CBCT, BEAM_PENCIL, BEAM_CT_SPIRAL_DUAL = range(6)


class Composition(C.Structure):
    _fields_ = [("n", C.c_int32), ("Z", C.c_int32 * MAX_ELEMENTS), ("w", C.c_double * MAX_ELEMENTS)]

    @classmethod
    def from_dict(cls, zw: dict) -> "Composition":
        c = cls()
        items = [(int(z), float(w)) for z, w in zw.items() if float(w) > 0.0]
        if len(items) > MAX_ELEMENTS:
            raise ValueError("too many elements")
        c.n = len(items)
        for i, (z, w) in enumerate(items):
            c.Z[i] = z
            c.w[i] = w
        return c


class Beam(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("kvp", C.c_double),
        ("anode_angle_deg", C.c_double),
        ("n_filters", C.c_int32),
        ("filter_Z", C.c_int32 * 8),
        ("filter_mm", C.c_double * 8),
        ("particles_per_exposure", C.c_uint64),
        ("n_exposures", C.c_uint64),
        ("position", C.c_double * 3),
        ("cosines", (C.c_double * 3) * 2),
        ("half_angles", C.c_double * 2),
        ("energy_kev", C.c_double),
        ("start", C.c_double * 3),
        ("stop", C.c_double * 3),
        ("start_angle_deg", C.c_double),
        ("stop_angle_deg", C.c_double),
        ("step_angle_deg", C.c_double),
        ("pitch", C.c_double),
        ("collimation_cm", C.c_double),
        ("scan_fov_cm", C.c_double),
        ("sdd_cm", C.c_double),
        ("rotation_axis", C.c_double * 3),
        ("n_slices", C.c_int32),
        ("slice_spacing_cm", C.c_double),
        ("kvp_b", C.c_double),
        ("n_filters_b", C.c_int32),
        ("filter_Z_b", C.c_int32 * 8),
        ("filter_mm_b", C.c_double * 8),
        ("tube_a_weight", C.c_double),
        ("fov_b_cm", C.c_double),
        ("n_bowtie", C.c_int32),
        ("bowtie_angle", C.POINTER(C.c_double)),
        ("bowtie_weight", C.POINTER(C.c_double)),
        ("n_aec", C.c_int32),
        ("aec_start", C.c_double * 3),
        ("aec_stop", C.c_double * 3),
        ("aec_weight", C.POINTER(C.c_double)),
        ("organ_aec", C.c_int32),
        ("organ_aec_start_deg", C.c_double),
        ("organ_aec_stop_deg", C.c_double),
        ("organ_aec_ramp_deg", C.c_double),
        ("organ_aec_low_weight", C.c_double),
        ("organ_aec_compensate", C.c_int32),
        ("dap_mgycm2", C.c_double),
        ("ctdi_vol_mgy", C.c_double),
        ("ctdi_w_mgy", C.c_double),
        ("ctdi_diameter_cm", C.c_double),
        ("air_kerma_mgy", C.c_double),
        ("n_bowtie_b", C.c_int32),
        ("bowtie_b_angle", C.POINTER(C.c_double)),
        ("bowtie_b_weight", C.POINTER(C.c_double)),
    ]


class Exposure(C.Structure):
    _fields_ = [
        ("pos", C.c_double * 3),
        ("c0", C.c_double * 3),
        ("c1", C.c_double * 3),
        ("half", C.c_double * 2),
        ("weight", C.c_double),
        ("tube", C.c_int32),
    ]


class Stats(C.Structure):
    _fields_ = [("e_source", C.c_double), ("e_deposited", C.c_double), ("e_escaped", C.c_double)] + [
        (n, C.c_uint64)
        for n in (
            "n_histories",
            "n_missed",
            "n_visits",
            "n_real",
            "n_photo",
            "n_compton",
            "n_rayleigh",
            "n_deposits",
            "n_cutoff",
            "n_errors",
            "n_interacted",
            "n_crossings",
            "n_fluorescence",
        )
    ]

    def as_dict(self) -> dict:
        return {f[0]: getattr(self, f[0]) for f in self._fields_}


def build() -> Path:
    """Compile the oracle with its Makefile (gcc; seconds)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        build()
    L = C.CDLL(str(LIB_PATH))
    d, i, u64, u32, vp = C.c_double, C.c_int, C.c_uint64, C.c_uint32, C.c_void_p
    pd = C.POINTER(C.c_double)
    L.or_atomic_mass.restype = d
    L.or_atomic_mass.argtypes = [i]
    L.or_sigma_kn.restype = d
    L.or_sigma_kn.argtypes = [d]
    L.or_sigma_photo.restype = d
    L.or_sigma_photo.argtypes = [d, i]
    L.or_sigma_incoh.restype = d
    L.or_sigma_incoh.argtypes = [d, i, i]
    L.or_sigma_coh.restype = d
    L.or_sigma_coh.argtypes = [d, i]
    L.or_kn_energy_transfer_fraction.restype = d
    L.or_kn_energy_transfer_fraction.argtypes = [d]
    L.or_attenuation.argtypes = [C.POINTER(Composition), i, i, pd, pd, pd, pd]
    L.or_tube_spectrum.restype = i
    L.or_tube_spectrum.argtypes = [d, d, i, C.POINTER(C.c_int32), pd, pd, pd, i]
    L.or_tube_mean_energy.restype = d
    L.or_tube_mean_energy.argtypes = [d, i, C.POINTER(C.c_int32), pd]
    L.or_tube_al_hvl_mm.restype = d
    L.or_tube_al_hvl_mm.argtypes = [d, i, C.POINTER(C.c_int32), pd]
    L.or_uniform_from_u32.restype = d
    L.or_uniform_from_u32.argtypes = [u32]
    L.or_beam_exposures.restype = i
    L.or_beam_exposures.argtypes = [C.POINTER(Beam), C.POINTER(Exposure), i]
    L.or_siddon_f32.restype = i
    L.or_siddon_f32.argtypes = [C.POINTER(C.c_float)] * 2 + [C.POINTER(C.c_int32), C.POINTER(C.c_float), i,
                                                              C.POINTER(C.c_int64), C.POINTER(C.c_float)]
    L.or_siddon_f64.restype = i
    L.or_siddon_f64.argtypes = [pd, pd, C.POINTER(C.c_int32), pd, i, C.POINTER(C.c_int64), pd]
    L.or_sample_compton.restype = d
    L.or_sample_compton.argtypes = [d, C.POINTER(Composition), i, pd, i, C.POINTER(C.c_int), pd]
    L.or_compton_quantiles.restype = i
    L.or_compton_quantiles.argtypes = [C.POINTER(Composition), i, i, pd]
    L.or_rayleigh_quantiles.restype = i
    L.or_rayleigh_quantiles.argtypes = [C.POINTER(Composition), i, pd]
    L.or_sample_photoelectric.restype = d
    L.or_sample_photoelectric.argtypes = [d, C.POINTER(Composition), pd, i, C.POINTER(C.c_int), pd]
    L.or_compton_shells.restype = i
    L.or_compton_shells.argtypes = [i, pd, pd, pd]
    L.or_doppler_energy.restype = d
    L.or_doppler_energy.argtypes = [d, d, d, d]
    for f in ("or_k_edge", "or_l_edge", "or_k_alpha", "or_fluorescence_yield_k"):
        getattr(L, f).restype = d
        getattr(L, f).argtypes = [i]
    L.or_sample_rayleigh.restype = d
    L.or_sample_rayleigh.argtypes = [d, C.POINTER(Composition), pd, i, C.POINTER(C.c_int)]
    L.or_world_create.restype = vp
    L.or_world_create.argtypes = [C.POINTER(C.c_int32), pd, pd, C.POINTER(C.c_uint8), C.POINTER(Composition), i, i]
    L.or_world_destroy.argtypes = [vp]
    L.or_world_clear.argtypes = [vp]
    L.or_world_table.restype = i
    L.or_world_table.argtypes = [vp, i, pd, pd, pd]
    L.or_world_majorant.restype = i
    L.or_world_majorant.argtypes = [vp, pd]
    L.or_transport.restype = i
    L.or_transport.argtypes = [vp, C.POINTER(Beam), u64, u32, i, i, u64, u64, C.POINTER(Stats)]
    L.or_world_tally.argtypes = [vp, pd, pd, C.POINTER(C.c_uint64)]
    _lib = L
    return L


def physics_load(path) -> None:
    L = lib()
    L.or_physics_load.restype = C.c_int
    L.or_physics_load.argtypes = [C.c_char_p]
    rc = L.or_physics_load(str(path).encode())
    if rc != 0:
        raise ValueError(f"oracle: bad physics table ({rc})")


def physics_reset() -> None:
    L = lib()
    L.or_physics_reset.restype = None
    L.or_physics_reset()


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(C.POINTER(t))


def energy_grid() -> np.ndarray:
    return EMIN + DE * np.arange(NE)


def attenuation(zw: dict, energies, correction: int = 1):
    E = np.ascontiguousarray(energies, dtype=np.float64)
    p, ic, co = (np.zeros_like(E) for _ in range(3))
    c = Composition.from_dict(zw)
    lib().or_attenuation(C.byref(c), correction, E.size, _p(E, C.c_double), _p(p, C.c_double),
                         _p(ic, C.c_double), _p(co, C.c_double))
    return p, ic, co


def _filters(filters: dict):
    fz = (C.c_int32 * 8)()
    fm = (C.c_double * 8)()
    for k, (z, mm) in enumerate(filters.items()):
        fz[k] = int(z)
        fm[k] = float(mm)
    return len(filters), fz, fm


def tube_spectrum(kvp: float, filters: dict, anode_angle_deg: float = 12.0):
    E = np.zeros(512)
    w = np.zeros(512)
    n, fz, fm = _filters(filters)
    k = lib().or_tube_spectrum(kvp, anode_angle_deg, n, fz, fm, _p(E, C.c_double), _p(w, C.c_double), 512)
    if k <= 0:
        raise ValueError("bad tube voltage")
    return E[:k].copy(), w[:k].copy()


def tube_mean_energy(kvp, filters):
    n, fz, fm = _filters(filters)
    return lib().or_tube_mean_energy(kvp, n, fz, fm)


def tube_al_hvl_mm(kvp, filters):
    n, fz, fm = _filters(filters)
    return lib().or_tube_al_hvl_mm(kvp, n, fz, fm)


def history_stream(seed: int, stream: int, h0: int, n_hist: int, n_draws: int) -> np.ndarray:
    out = np.zeros((n_hist, n_draws), dtype=np.uint32)
    L = lib()
    L.or_history_stream.restype = None
    L.or_history_stream.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_int, C.c_int, C.POINTER(C.c_uint32)]
    L.or_history_stream(seed, stream, h0, n_hist, n_draws, _p(out, C.c_uint32))
    return out


def make_beam(params: dict) -> tuple[Beam, list]:
    """Fill an oracle Beam from a plain dict; returns (beam, keepalive)."""
    b = Beam()
    keep = []
    for k, v in params.items():
        if k in ("filters", "filters_b"):
            n, fz, fm = _filters(v)
            suf = "_b" if k == "filters_b" else ""
            setattr(b, "n_filters" + suf, n)
            setattr(b, "filter_Z" + suf, fz)
            setattr(b, "filter_mm" + suf, fm)
        elif k in ("bowtie", "bowtie_b"):
            ang = np.ascontiguousarray([a for a, _ in v], dtype=np.float64)
            wt = np.ascontiguousarray([w for _, w in v], dtype=np.float64)
            keep += [ang, wt]
            suf = "_b" if k == "bowtie_b" else ""
            setattr(b, "n_bowtie" + suf, len(v))
            setattr(b, "bowtie" + suf + "_angle", _p(ang, C.c_double))
            setattr(b, "bowtie" + suf + "_weight", _p(wt, C.c_double))
        elif k == "aec":
            start, stop, weights = v
            wt = np.ascontiguousarray(weights, dtype=np.float64)
            keep.append(wt)
            b.n_aec = len(wt)
            b.aec_start = (C.c_double * 3)(*start)
            b.aec_stop = (C.c_double * 3)(*stop)
            b.aec_weight = _p(wt, C.c_double)
        elif k == "cosines":
            for r in range(2):
                for cc in range(3):
                    b.cosines[r][cc] = v[r][cc]
        elif isinstance(v, (list, tuple)):
            arr = getattr(b, k)
            for j, x in enumerate(v):
                arr[j] = x
        else:
            setattr(b, k, v)
    return b, keep


def calibration_factor(params: dict, n_hist: int) -> float:
    """Analytic calibration factor of a DX/CBCT (DAP) or pencil (air kerma) beam
    over n_hist histories; 1 without a target."""
    b, keep = make_beam(params)
    L = lib()
    L.or_calibration_factor.restype = C.c_double
    L.or_calibration_factor.argtypes = [C.POINTER(Beam), C.c_uint64]
    return L.or_calibration_factor(C.byref(b), n_hist)


def beam_exposures(params: dict) -> list[dict]:
    b, keep = make_beam(params)
    n = lib().or_beam_exposures(C.byref(b), None, 0)
    arr = (Exposure * max(n, 1))()
    lib().or_beam_exposures(C.byref(b), arr, n)
    out = []
    for e in arr[:n]:
        out.append({"pos": list(e.pos), "c0": list(e.c0), "c1": list(e.c1), "half": list(e.half),
                    "weight": e.weight, "tube": e.tube})
    return out


def siddon_f32(o, d, dims, spacing, cap=4096):
    o = np.ascontiguousarray(o, dtype=np.float32)
    d = np.ascontiguousarray(d, dtype=np.float32)
    n = np.ascontiguousarray(dims, dtype=np.int32)
    sp = np.ascontiguousarray(spacing, dtype=np.float32)
    idx = np.zeros(cap, dtype=np.int64)
    ln = np.zeros(cap, dtype=np.float32)
    k = lib().or_siddon_f32(_p(o, C.c_float), _p(d, C.c_float), _p(n, C.c_int32), _p(sp, C.c_float), cap,
                            _p(idx, C.c_int64), _p(ln, C.c_float))
    if k < 0:
        raise ValueError("cap too small")
    return idx[:k].copy(), ln[:k].copy()


def siddon_f64(o, d, dims, spacing, cap=4096):
    o = np.ascontiguousarray(o, dtype=np.float64)
    d = np.ascontiguousarray(d, dtype=np.float64)
    n = np.ascontiguousarray(dims, dtype=np.int32)
    sp = np.ascontiguousarray(spacing, dtype=np.float64)
    idx = np.zeros(cap, dtype=np.int64)
    ln = np.zeros(cap, dtype=np.float64)
    k = lib().or_siddon_f64(_p(o, C.c_double), _p(d, C.c_double), _p(n, C.c_int32), _p(sp, C.c_double), cap,
                            _p(idx, C.c_int64), _p(ln, C.c_double))
    if k < 0:
        raise ValueError("cap too small")
    return idx[:k].copy(), ln[:k].copy()


def compton_quantiles(zw, correction, energy_index):
    """1 - cos theta of the Compton angle table at the probabilities
    u_j = 1 - (1 - j/(K-1))^2 (K = 256) for table energy EMIN + energy_index * DE."""
    out = np.zeros(256)
    c = Composition.from_dict(zw)
    if lib().or_compton_quantiles(C.byref(c), correction, energy_index, _p(out, C.c_double)) != 256:
        raise ValueError("energy index out of range")
    return out


def rayleigh_quantiles(zw, energy_index):
    """1 - cos theta of the Rayleigh angle table at u_j = 1 - (1 - j/(K-1))^2."""
    out = np.zeros(256)
    c = Composition.from_dict(zw)
    if lib().or_rayleigh_quantiles(C.byref(c), energy_index, _p(out, C.c_double)) != 256:
        raise ValueError("energy index out of range")
    return out


def sample_compton(E, zw, correction, uniforms):
    u = np.ascontiguousarray(uniforms, dtype=np.float64)
    used = C.c_int(0)
    cost = C.c_double(0)
    c = Composition.from_dict(zw)
    Ep = lib().or_sample_compton(E, C.byref(c), correction, _p(u, C.c_double), u.size, C.byref(used), C.byref(cost))
    return Ep, cost.value, used.value


def sample_photoelectric(E, zw, uniforms):
    """(fluorescence energy or 0, z cosine of its direction, uniforms used)"""
    u = np.ascontiguousarray(uniforms, dtype=np.float64)
    used = C.c_int(0)
    dz = C.c_double(0)
    c = Composition.from_dict(zw)
    Ef = lib().or_sample_photoelectric(E, C.byref(c), _p(u, C.c_double), u.size, C.byref(used), C.byref(dz))
    return Ef, dz.value, used.value


def compton_shells(Z):
    """(electrons, binding keV, momentum scale in m_e c) of the level-2 Compton shells"""
    e = (C.c_double * 3)()
    b = (C.c_double * 3)()
    m = (C.c_double * 3)()
    n = lib().or_compton_shells(Z, e, b, m)
    return np.array(e[:n]), np.array(b[:n]), np.array(m[:n])


def doppler_energy(E, A, omu, rho):
    return lib().or_doppler_energy(E, A, omu, rho)


def sample_rayleigh(E, zw, uniforms):
    u = np.ascontiguousarray(uniforms, dtype=np.float64)
    used = C.c_int(0)
    c = Composition.from_dict(zw)
    mu = lib().or_sample_rayleigh(E, C.byref(c), _p(u, C.c_double), u.size, C.byref(used))
    return mu, used.value


class World:
    """Oracle voxel world (mirrors AAVoxelGrid::setData + World::build)."""

    def __init__(self, dims, spacing_cm, density, material, materials: list[dict], correction: int = 1):
        self.dims = tuple(int(x) for x in dims)
        n = np.ascontiguousarray(self.dims, dtype=np.int32)
        sp = np.ascontiguousarray(spacing_cm, dtype=np.float64)
        dens = np.ascontiguousarray(density, dtype=np.float64).ravel(order="C")
        mat = np.ascontiguousarray(material, dtype=np.uint8).ravel(order="C")
        comps = (Composition * len(materials))(*[Composition.from_dict(m) for m in materials])
        self.N = int(np.prod(self.dims))
        assert dens.size == self.N and mat.size == self.N
        fg = (mat != 0) & (mat != TRANSPARENT)
        self.box_fraction = 0.0
        if fg.any():
            m3 = fg.reshape(self.dims[::-1])
            ext = [np.flatnonzero(m3.any(axis=tuple(b for b in range(3) if b != a))) for a in range(3)]
            self.box_fraction = float(np.prod([(e[-1] - e[0] + 1) / m3.shape[a] for a, e in enumerate(ext)]))
        self._h = lib().or_world_create(_p(n, C.c_int32), _p(sp, C.c_double), _p(dens, C.c_double),
                                        _p(mat, C.c_uint8), comps, len(materials), correction)
        if not self._h:
            raise ValueError("oracle world creation failed")

    def close(self):
        if self._h:
            lib().or_world_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def clear(self):
        lib().or_world_clear(self._h)

    def table(self, m):
        p, ic, co = (np.zeros(NE) for _ in range(3))
        lib().or_world_table(self._h, m, _p(p, C.c_double), _p(ic, C.c_double), _p(co, C.c_double))
        return p, ic, co

    def set_macro(self, B: int) -> np.ndarray:
        L = lib()
        L.or_world_set_macro.restype = C.c_int
        L.or_world_set_macro.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
        n = L.or_world_set_macro(self._h, B, None)
        out = np.zeros(max(n, 0))
        L.or_world_set_macro(self._h, B, _p(out, C.c_double))
        return out

    def majorant(self):
        m = np.zeros(NE)
        lib().or_world_majorant(self._h, _p(m, C.c_double))
        return m

    def run(self, beam: dict, seed=1, stream=0, tracking=None, threads=None, hist_begin=0,
            hist_end=2**63):
        """tracking None: Woodcock as the transport kernel chooses by default (two
        regions when the box holds less than TWO_REGION_BOX_FRACTION of the grid)."""
        if tracking is None:
            tracking = TRACK_WOODCOCK_BOX if self.box_fraction < TWO_REGION_BOX_FRACTION else TRACK_WOODCOCK
        b, keep = make_beam(beam)
        st = Stats()
        threads = threads or os.cpu_count() or 1
        rc = lib().or_transport(self._h, C.byref(b), seed, stream, tracking, threads, hist_begin, hist_end,
                                C.byref(st))
        if rc != 0:
            raise RuntimeError(f"oracle transport failed: {rc}")
        return st.as_dict()

    def tally(self):
        e = np.zeros(self.N)
        e2 = np.zeros(self.N)
        c = np.zeros(self.N, dtype=np.uint64)
        lib().or_world_tally(self._h, _p(e, C.c_double), _p(e2, C.c_double), _p(c, C.c_uint64))
        return e, e2, c


def sample_source(world: "World", beam: dict, n: int, seed=1, stream=0, h0=0) -> np.ndarray:
    """Source photons (E, weight, grid-local pos[3], dir[3]) of histories h0..h0+n-1."""
    b, keep = make_beam(beam)
    out = np.zeros((n, 8))
    L = lib()
    L.or_sample_source.restype = C.c_int
    L.or_sample_source.argtypes = [C.c_void_p, C.POINTER(Beam), C.c_uint64, C.c_uint32, C.c_uint64, C.c_int,
                                   C.POINTER(C.c_double)]
    rc = L.or_sample_source(world._h, C.byref(b), seed, stream, h0, n, _p(out, C.c_double))
    if rc != 0:
        raise RuntimeError(f"oracle source sampling failed: {rc}")
    return out
