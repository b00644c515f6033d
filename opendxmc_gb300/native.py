"""ctypes binding of libdxmcg.so (include/dxmcg.h).

The library is the product: every transport call goes to its CUDA kernels.
There is no Python or CPU fallback; if the shared library is missing the import
of the engine fails with an error that says how to build it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_lib" / "libdxmcg.so"

MAX_ELEMENTS = 16
NE = 300
TRACK_WOODCOCK, TRACK_SIDDON, TRACK_MACRO = 0, 1, 2
BEAM_DX, BEAM_CT_SPIRAL, BEAM_CT_SEQUENTIAL, BEAM_CBCT, BEAM_PENCIL, BEAM_CT_SPIRAL_DUAL_ENERGY = range(6)

STATUS = {0: "OK", -1: "ARGUMENT", -2: "CUDA", -3: "STATE", -4: "CANCELLED", -5: "DEVICE", -6: "NO_DEVICE",
          -7: "CAPACITY"}

# every function include/dxmcg.h declares
EXPORTED = [
    "dxmcg_version", "dxmcg_last_error", "dxmcg_device_count", "dxmcg_set_device", "dxmcg_material_attenuation",
    "dxmcg_tube_spectrum",
    "dxmcg_tube_mean_energy", "dxmcg_tube_al_hvl", "dxmcg_physics_load", "dxmcg_physics_reset",
    "dxmcg_physics_write", "dxmcg_beam_exposures", "dxmcg_beam_calibration",
    "dxmcg_world_create",
    "dxmcg_world_set_data", "dxmcg_world_set_data_f32", "dxmcg_world_build", "dxmcg_world_destroy",
    "dxmcg_world_clear_tally", "dxmcg_world_read_tally", "dxmcg_world_read_dose", "dxmcg_world_tables",
    "dxmcg_world_packed_density", "dxmcg_transport_run", "dxmcg_batch_create", "dxmcg_batch_info",
    "dxmcg_batch_run", "dxmcg_batch_destroy", "dxmcg_autotune", "dxmcg_transport_run_noalloc",
    "dxmcg_ct_segmentation_table", "dxmcg_ct_segment", "dxmcg_ct_segment_device", "dxmcg_organ_dose_table",
    "dxmcg_organ_dose_table_device", "dxmcg_world_organ_dose", "dxmcg_world_read_dose_postprocessed",
    "dxmcg_denoiser_create", "dxmcg_denoiser_destroy", "dxmcg_denoiser_set_wait_limit",
    "dxmcg_denoiser_param_count", "dxmcg_denoiser_get_params",
    "dxmcg_denoiser_set_params", "dxmcg_denoiser_get_grads", "dxmcg_denoiser_forward", "dxmcg_denoiser_backward",
    "dxmcg_denoiser_adam", "dxmcg_denoiser_prepare_input", "dxmcg_denoiser_gather_patches", "dxmcg_world_denoise",
    "dxmcg_progress_create",
    "dxmcg_progress_destroy",
    "dxmcg_progress_get", "dxmcg_progress_stop", "dxmcg_progress_reset", "dxmcg_progress_continue",
    "dxmcg_progress_message",
    "dxmcg_siddon_trace", "dxmcg_history_stream", "dxmcg_sample_compton", "dxmcg_sample_rayleigh",
    "dxmcg_sample_photoelectric", "dxmcg_umma_probe",
    "dxmcg_sample_source",
]


class DxmcgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"dxmcg {STATUS.get(code, code)}: {msg}")
        self.code = code


MAX_SEG_MATERIALS = 64


class Segmentation(C.Structure):
    _fields_ = [("n_materials", C.c_int32), ("hu", C.c_double * MAX_SEG_MATERIALS),
                ("separator", C.c_double * (MAX_SEG_MATERIALS - 1)),
                ("attenuation", C.c_double * MAX_SEG_MATERIALS), ("water_attenuation", C.c_double),
                ("water_density", C.c_double), ("air_attenuation", C.c_double), ("air_density", C.c_double)]


class OrganDose(C.Structure):
    _fields_ = [("n_voxels", C.c_uint64), ("volume_cm3", C.c_double), ("mass_g", C.c_double),
                ("dose", C.c_double)]


class DenoiserConfig(C.Structure):
    _fields_ = [("levels", C.c_int32), ("channels", C.c_int32 * 5), ("seed", C.c_uint64),
                ("conv_path", C.c_int32)]


class Material(C.Structure):
    _fields_ = [("n", C.c_int32), ("Z", C.c_int32 * MAX_ELEMENTS), ("w", C.c_double * MAX_ELEMENTS)]

    @classmethod
    def from_dict(cls, zw: dict) -> "Material":
        m = cls()
        items = [(int(z), float(w)) for z, w in zw.items() if float(w) > 0.0]
        if not items or len(items) > MAX_ELEMENTS:
            raise ValueError("a material needs 1..16 elements with positive weight")
        m.n = len(items)
        for i, (z, w) in enumerate(items):
            m.Z[i] = z
            m.w[i] = w
        return m


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
    _fields_ = [("pos", C.c_double * 3), ("c0", C.c_double * 3), ("c1", C.c_double * 3), ("half", C.c_double * 2),
                ("weight", C.c_double), ("tube", C.c_int32)]


class RunOptions(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("stream", C.c_uint32), ("tracking", C.c_int32), ("normalize", C.c_int32),
                ("block_size", C.c_int32), ("blocks_per_sm", C.c_int32), ("chunk_histories_log2", C.c_int32),
                ("hist_begin", C.c_uint64), ("hist_end", C.c_uint64), ("interact_batch", C.c_int32),
                ("refill_batch", C.c_int32), ("macro_cell", C.c_int32),
                ("woodcock_steps", C.c_int32), ("max_steps", C.c_uint32), ("gather_skip", C.c_int32),
                ("two_region", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("e_source", C.c_double), ("e_deposited", C.c_double), ("e_escaped", C.c_double)] + [
        (n, C.c_uint64) for n in ("n_histories", "n_missed", "n_visits", "n_photo", "n_compton", "n_rayleigh",
                                  "n_cutoff", "n_errors", "n_interacted")] + [
        ("kernel_ms", C.c_double), ("total_ms", C.c_double), ("dose_scale", C.c_double),
        ("calibration", C.c_double), ("n_crossings", C.c_uint64),
        ("n_fluorescence", C.c_uint64), ("n_voxel_reads", C.c_uint64), ("n_cell_reads", C.c_uint64),
        ("woodcock_steps", C.c_int32), ("two_region", C.c_int32)]

    def as_dict(self) -> dict:
        return {f[0]: getattr(self, f[0]) for f in self._fields_}


_lib = None


def lib() -> C.CDLL:
    """Load libdxmcg.so; raise if it has not been built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m opendxmc_gb300.build` "
                          "(the engine has no CPU fallback)")
    L = C.CDLL(str(LIB_PATH))
    i, d, u64, vp, cp = C.c_int, C.c_double, C.c_uint64, C.c_void_p, C.c_char_p
    pd, pf, pi32, pu8 = C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_int32), C.POINTER(C.c_uint8)
    pu64, pi64 = C.POINTER(C.c_uint64), C.POINTER(C.c_int64)
    sig = {
        "dxmcg_version": (i, []),
        "dxmcg_last_error": (cp, []),
        "dxmcg_device_count": (i, []),
        "dxmcg_set_device": (i, [i]),
        "dxmcg_material_attenuation": (i, [C.POINTER(Material), i, i, pd, pd, pd, pd]),
        "dxmcg_tube_spectrum": (i, [d, d, i, pi32, pd, pd, pd, i, C.POINTER(C.c_int)]),
        "dxmcg_tube_mean_energy": (i, [d, i, pi32, pd, pd]),
        "dxmcg_tube_al_hvl": (i, [d, i, pi32, pd, pd]),
        "dxmcg_beam_exposures": (i, [C.POINTER(Beam), C.POINTER(Exposure), i, C.POINTER(C.c_int)]),
        "dxmcg_beam_calibration": (i, [C.POINTER(Beam), i, C.POINTER(RunOptions), pd]),
        "dxmcg_physics_load": (i, [cp]),
        "dxmcg_physics_reset": (i, []),
        "dxmcg_physics_write": (i, [cp, i, pi32]),
        "dxmcg_world_create": (i, [pi32, pd, C.POINTER(Material), i, i, C.POINTER(vp)]),
        "dxmcg_world_set_data": (i, [vp, pd, pu8]),
        "dxmcg_world_set_data_f32": (i, [vp, pf, pu8]),
        "dxmcg_world_build": (i, [vp]),
        "dxmcg_world_destroy": (None, [vp]),
        "dxmcg_world_clear_tally": (i, [vp]),
        "dxmcg_world_read_tally": (i, [vp, pd, pd, pu64]),
        "dxmcg_world_read_dose": (i, [vp, pd, pd, pu64]),
        "dxmcg_world_tables": (i, [vp, i, pf, pf]),
        "dxmcg_world_packed_density": (i, [vp, pf, pu8]),
        "dxmcg_transport_run": (i, [vp, C.POINTER(Beam), C.POINTER(RunOptions), vp, C.POINTER(Stats)]),
        "dxmcg_batch_create": (i, [i, C.POINTER(vp), C.POINTER(Beam), C.POINTER(RunOptions), C.POINTER(vp)]),
        "dxmcg_batch_info": (i, [vp, C.POINTER(C.c_int), pu64, pd]),
        "dxmcg_batch_run": (i, [vp, C.POINTER(Stats)]),
        "dxmcg_batch_destroy": (None, [vp]),
        "dxmcg_autotune": (i, [vp, C.POINTER(Beam), C.POINTER(RunOptions), u64, pd]),
        "dxmcg_transport_run_noalloc": (i, [pi32, pd, vp, vp, C.POINTER(Material), i, i, C.POINTER(Beam),
                                            C.POINTER(RunOptions), vp, vp, C.POINTER(Stats)]),
        "dxmcg_ct_segmentation_table": (i, [d, d, d, i, C.POINTER(Material), pd, C.POINTER(Segmentation)]),
        "dxmcg_ct_segment": (i, [C.POINTER(Segmentation), pd, u64, pu8, pd]),
        "dxmcg_ct_segment_device": (i, [C.POINTER(Segmentation), vp, u64, vp, vp, vp]),
        "dxmcg_organ_dose_table": (i, [pu8, pd, pd, u64, pd, i, C.POINTER(OrganDose)]),
        "dxmcg_organ_dose_table_device": (i, [vp, vp, vp, u64, pd, i, C.POINTER(OrganDose), vp]),
        "dxmcg_world_organ_dose": (i, [vp, pu8, i, i, C.POINTER(OrganDose)]),
        "dxmcg_world_read_dose_postprocessed": (i, [vp, i, pd, pd, pd, C.POINTER(C.c_int)]),
        "dxmcg_denoiser_create": (i, [C.POINTER(DenoiserConfig), C.POINTER(vp)]),
        "dxmcg_denoiser_destroy": (None, [vp]),
        "dxmcg_denoiser_set_wait_limit": (i, [vp, C.c_uint32]),
        "dxmcg_denoiser_param_count": (i, [vp, pu64]),
        "dxmcg_denoiser_get_params": (i, [vp, pf]),
        "dxmcg_denoiser_set_params": (i, [vp, pf]),
        "dxmcg_denoiser_get_grads": (i, [vp, pf]),
        "dxmcg_denoiser_forward": (i, [vp, vp, i, i, i, i, vp, vp]),
        "dxmcg_denoiser_backward": (i, [vp, vp, vp, i, i, i, i, pd, vp]),
        "dxmcg_denoiser_adam": (i, [vp, C.c_float, vp]),
        "dxmcg_denoiser_prepare_input": (i, [vp, vp, vp, u64, d, vp, vp]),
        "dxmcg_denoiser_gather_patches": (i, [vp, vp, vp, i, vp, i, i, vp, vp, vp]),
        "dxmcg_world_denoise": (i, [vp, vp, d, pd, pd]),
        "dxmcg_progress_create": (vp, []),
        "dxmcg_progress_destroy": (None, [vp]),
        "dxmcg_progress_get": (None, [vp, pu64, pu64]),
        "dxmcg_progress_stop": (None, [vp]),
        "dxmcg_progress_reset": (None, [vp]),
        "dxmcg_progress_continue": (i, [vp]),
        "dxmcg_progress_message": (i, [vp, cp, i]),
        "dxmcg_siddon_trace": (i, [i, pf, pf, pi32, pf, i, pi64, pf, pi32]),
        "dxmcg_history_stream": (i, [u64, C.c_uint32, u64, i, i, C.POINTER(C.c_uint32)]),
        "dxmcg_sample_compton": (i, [i, pd, C.POINTER(Material), i, pd, i, pd, pd, pi32]),
        "dxmcg_sample_rayleigh": (i, [i, pd, C.POINTER(Material), pd, i, pd, pi32]),
        "dxmcg_sample_photoelectric": (i, [i, pd, C.POINTER(Material), pd, i, pd, pd, pi32]),
        "dxmcg_umma_probe": (i, [i, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
        "dxmcg_sample_source": (i, [vp, C.POINTER(Beam), C.POINTER(RunOptions), i, pd]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != 0:
        raise DxmcgError(rc, lib().dxmcg_last_error().decode(errors="replace"))


def ptr(a: np.ndarray, t):
    return a.ctypes.data_as(C.POINTER(t))


def make_beam(params: dict):
    """Beam parameters (dict, same keys as dxmcg_beam) -> (Beam, keepalive list)."""
    b = Beam()
    keep = []
    for k, v in params.items():
        if k in ("filters", "filters_b"):
            suf = "_b" if k == "filters_b" else ""
            items = list(v.items())
            if len(items) > 8:
                raise ValueError("at most 8 filters")
            setattr(b, "n_filters" + suf, len(items))
            fz = getattr(b, "filter_Z" + suf)
            fm = getattr(b, "filter_mm" + suf)
            for j, (z, mm) in enumerate(items):
                fz[j] = int(z)
                fm[j] = float(mm)
        elif k in ("bowtie", "bowtie_b"):
            ang = np.ascontiguousarray([a for a, _ in v], dtype=np.float64)
            wt = np.ascontiguousarray([w for _, w in v], dtype=np.float64)
            keep += [ang, wt]
            suf = "_b" if k == "bowtie_b" else ""
            setattr(b, "n_bowtie" + suf, len(ang))
            setattr(b, "bowtie" + suf + "_angle", ptr(ang, C.c_double))
            setattr(b, "bowtie" + suf + "_weight", ptr(wt, C.c_double))
        elif k == "aec":
            start, stop, weights = v
            wt = np.ascontiguousarray(weights, dtype=np.float64)
            keep.append(wt)
            b.n_aec = len(wt)
            for j in range(3):
                b.aec_start[j] = start[j]
                b.aec_stop[j] = stop[j]
            b.aec_weight = ptr(wt, C.c_double)
        elif k == "cosines":
            for r in range(2):
                for c in range(3):
                    b.cosines[r][c] = v[r][c]
        elif isinstance(v, (list, tuple, np.ndarray)):
            arr = getattr(b, k)
            for j, x in enumerate(v):
                arr[j] = x
        else:
            setattr(b, k, v)
    return b, keep
