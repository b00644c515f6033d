"""Thin Python handle over the C ABI: a built voxel world on the GPU plus runs.

This is what the tests and the benchmark drive; the dxmc-style mirror classes in
`opendxmc_gb300.api` are built on it.  Every call goes through libdxmcg.so.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native as N


def device_count() -> int:
    return int(N.lib().dxmcg_device_count())


def set_device(device: int) -> None:
    N.check(N.lib().dxmcg_set_device(device))


def attenuation(zw: dict, energies, correction: int = 1):
    E = np.ascontiguousarray(energies, dtype=np.float64)
    p, ic, co = (np.zeros_like(E) for _ in range(3))
    m = N.Material.from_dict(zw)
    N.check(N.lib().dxmcg_material_attenuation(C.byref(m), correction, E.size, N.ptr(E, C.c_double),
                                               N.ptr(p, C.c_double), N.ptr(ic, C.c_double), N.ptr(co, C.c_double)))
    return p, ic, co


def _filters(filters: dict):
    fz = (C.c_int32 * 8)()
    fm = (C.c_double * 8)()
    for k, (z, mm) in enumerate(filters.items()):
        fz[k] = int(z)
        fm[k] = float(mm)
    return len(filters), fz, fm


def tube_spectrum(kvp: float, filters: dict, anode_angle_deg: float = 12.0):
    n_out = C.c_int(0)
    n, fz, fm = _filters(filters)
    N.check(N.lib().dxmcg_tube_spectrum(kvp, anode_angle_deg, n, fz, fm, None, None, 0, C.byref(n_out)))
    E = np.zeros(n_out.value)
    w = np.zeros(n_out.value)
    N.check(N.lib().dxmcg_tube_spectrum(kvp, anode_angle_deg, n, fz, fm, N.ptr(E, C.c_double), N.ptr(w, C.c_double),
                                        E.size, C.byref(n_out)))
    return E, w


def tube_mean_energy(kvp: float, filters: dict) -> float:
    n, fz, fm = _filters(filters)
    out = C.c_double(0)
    N.check(N.lib().dxmcg_tube_mean_energy(kvp, n, fz, fm, C.byref(out)))
    return out.value


def tube_al_hvl(kvp: float, filters: dict) -> float:
    n, fz, fm = _filters(filters)
    out = C.c_double(0)
    N.check(N.lib().dxmcg_tube_al_hvl(kvp, n, fz, fm, C.byref(out)))
    return out.value


def beam_exposures(params: dict) -> list[dict]:
    b, keep = N.make_beam(params)
    n = C.c_int(0)
    N.check(N.lib().dxmcg_beam_exposures(C.byref(b), None, 0, C.byref(n)))
    arr = (N.Exposure * max(n.value, 1))()
    N.check(N.lib().dxmcg_beam_exposures(C.byref(b), arr, n.value, C.byref(n)))
    return [{"pos": list(e.pos), "c0": list(e.c0), "c1": list(e.c1), "half": list(e.half), "weight": e.weight,
             "tube": e.tube} for e in arr[:n.value]]


def physics_load(path) -> None:
    """Load a physics table (dxmcg-physics 1 text format) for the whole process."""
    N.check(N.lib().dxmcg_physics_load(str(path).encode()))


def physics_reset() -> None:
    """Back to the engine's own parametric model."""
    N.check(N.lib().dxmcg_physics_reset())


def physics_write(path, elements) -> None:
    """Write the current numbers of `elements` (atomic numbers) as a physics table."""
    z = np.ascontiguousarray(list(elements), dtype=np.int32)
    N.check(N.lib().dxmcg_physics_write(str(path).encode(), z.size, N.ptr(z, C.c_int32)))


def beam_calibration(params: dict, correction: int = 1, options: N.RunOptions | None = None) -> float:
    """The factor the transport applies to every history weight with normalize set
    (DX/CBCT: DAP, pencil: air kerma, CT: CTDI phantom run, which needs a device)."""
    b, keep = N.make_beam(params)
    o = options if options is not None else run_options(normalize=1)
    out = C.c_double(0)
    N.check(N.lib().dxmcg_beam_calibration(C.byref(b), correction, C.byref(o), C.byref(out)))
    return out.value


def run_options(seed=1, stream=0, tracking=N.TRACK_WOODCOCK, normalize=0, block_size=0, blocks_per_sm=0,
                chunk_log2=0, hist_begin=0, hist_end=0, interact_batch=0, refill_batch=0,
                macro_cell=0, woodcock_steps=0, max_steps=0, gather_skip=0, two_region=0) -> N.RunOptions:
    o = N.RunOptions()
    o.seed = seed
    o.stream = stream
    o.tracking = tracking
    o.normalize = normalize
    o.block_size = block_size
    o.blocks_per_sm = blocks_per_sm
    o.chunk_histories_log2 = chunk_log2
    o.hist_begin = hist_begin
    o.hist_end = hist_end
    o.interact_batch = interact_batch
    o.refill_batch = refill_batch
    o.macro_cell = macro_cell
    o.woodcock_steps = woodcock_steps
    o.max_steps = max_steps
    o.gather_skip = gather_skip
    o.two_region = two_region
    return o


def ct_segmentation_table(kvp=120.0, al_mm=0.0, sn_mm=0.0, materials=None) -> N.Segmentation:
    """CTSegmentationPipeline's CT-number table for a tube setting; `materials` is a
    list of (composition, density) in ascending CT number (default: the pipeline's
    five, phantoms.SEGMENTATION_MATERIALS)."""
    if materials is None:
        from . import phantoms as P

        materials = [(c, d) for _, c, d in P.SEGMENTATION_MATERIALS]
    mats = (N.Material * len(materials))(*[N.Material.from_dict(c) for c, _ in materials])
    dens = np.ascontiguousarray([d for _, d in materials], dtype=np.float64)
    t = N.Segmentation()
    N.check(N.lib().dxmcg_ct_segmentation_table(kvp, al_mm, sn_mm, len(materials), mats, N.ptr(dens, C.c_double),
                                                C.byref(t)))
    return t


def ct_segment(table: N.Segmentation, hu: np.ndarray):
    """HU array -> (uint8 material, float64 density), computed on the GPU."""
    h = np.ascontiguousarray(hu, dtype=np.float64).reshape(-1)
    m = np.zeros(h.size, dtype=np.uint8)
    d = np.zeros(h.size, dtype=np.float64)
    N.check(N.lib().dxmcg_ct_segment(C.byref(table), N.ptr(h, C.c_double), h.size, N.ptr(m, C.c_uint8),
                                     N.ptr(d, C.c_double)))
    return m.reshape(np.shape(hu)), d.reshape(np.shape(hu))


def _organ_rows(out, n_organs):
    return {"n_voxels": np.array([out[i].n_voxels for i in range(n_organs)], dtype=np.uint64),
            "volume_cm3": np.array([out[i].volume_cm3 for i in range(n_organs)]),
            "mass_g": np.array([out[i].mass_g for i in range(n_organs)]),
            "dose": np.array([out[i].dose for i in range(n_organs)])}


def organ_dose_table(organ: np.ndarray, dose: np.ndarray, density: np.ndarray, spacing_cm, n_organs: int) -> dict:
    """DoseTablePipeline's table (per organ: voxels, volume, mass, mean dose), on the GPU."""
    o = np.ascontiguousarray(organ, dtype=np.uint8).reshape(-1)
    d = np.ascontiguousarray(dose, dtype=np.float64).reshape(-1)
    r = np.ascontiguousarray(density, dtype=np.float64).reshape(-1)
    if not (o.size == d.size == r.size):
        raise ValueError("organ, dose and density must have the same size")
    sp = np.ascontiguousarray(spacing_cm, dtype=np.float64)
    out = (N.OrganDose * n_organs)()
    N.check(N.lib().dxmcg_organ_dose_table(N.ptr(o, C.c_uint8), N.ptr(d, C.c_double), N.ptr(r, C.c_double), o.size,
                                           N.ptr(sp, C.c_double), n_organs, out))
    return _organ_rows(out, n_organs)


class Progress:
    """TransportProgress mirror over dxmcg_progress (thread-safe in the library)."""

    def __init__(self):
        self._h = N.lib().dxmcg_progress_create()

    def progress(self) -> tuple[int, int]:
        d = C.c_uint64(0)
        t = C.c_uint64(0)
        N.lib().dxmcg_progress_get(self._h, C.byref(d), C.byref(t))
        return d.value, t.value

    def message(self) -> str:
        buf = C.create_string_buffer(256)
        N.lib().dxmcg_progress_message(self._h, buf, 256)
        return buf.value.decode()

    def continueSimulation(self) -> bool:
        return bool(N.lib().dxmcg_progress_continue(self._h))

    def setStopSimulation(self) -> None:
        N.lib().dxmcg_progress_stop(self._h)

    def __del__(self):
        try:
            if self._h:
                N.lib().dxmcg_progress_destroy(self._h)
        except Exception:
            pass


class GpuWorld:
    """A voxel world resident on the GPU (World<AAVoxelGrid> after build())."""

    def __init__(self, dims, spacing_cm, materials: list[dict], correction: int = 1):
        self.dims = tuple(int(x) for x in dims)
        self.N = int(np.prod(self.dims))
        d = np.ascontiguousarray(self.dims, dtype=np.int32)
        s = np.ascontiguousarray(spacing_cm, dtype=np.float64)
        mats = (N.Material * len(materials))(*[N.Material.from_dict(m) for m in materials])
        h = C.c_void_p()
        N.check(N.lib().dxmcg_world_create(N.ptr(d, C.c_int32), N.ptr(s, C.c_double), mats, len(materials),
                                           correction, C.byref(h)))
        self._h = h

    def set_data(self, density: np.ndarray, material: np.ndarray) -> None:
        m = np.ascontiguousarray(material, dtype=np.uint8).reshape(-1)
        if m.size != self.N or density.size != self.N:
            raise ValueError("array size does not match dimensions")
        if density.dtype == np.float32:
            dd = np.ascontiguousarray(density).reshape(-1)
            N.check(N.lib().dxmcg_world_set_data_f32(self._h, N.ptr(dd, C.c_float), N.ptr(m, C.c_uint8)))
        else:
            dd = np.ascontiguousarray(density, dtype=np.float64).reshape(-1)
            N.check(N.lib().dxmcg_world_set_data(self._h, N.ptr(dd, C.c_double), N.ptr(m, C.c_uint8)))

    def build(self) -> None:
        N.check(N.lib().dxmcg_world_build(self._h))

    def run(self, beam: dict, options: N.RunOptions | None = None, progress: Progress | None = None) -> dict:
        b, keep = N.make_beam(beam)
        st = N.Stats()
        opts = options if options is not None else run_options()
        rc = N.lib().dxmcg_transport_run(self._h, C.byref(b), C.byref(opts), progress._h if progress else None,
                                         C.byref(st))
        N.check(rc)
        return st.as_dict()

    def run_status(self, beam: dict, options=None, progress=None) -> tuple[int, dict]:
        b, keep = N.make_beam(beam)
        st = N.Stats()
        opts = options if options is not None else run_options()
        rc = N.lib().dxmcg_transport_run(self._h, C.byref(b), C.byref(opts), progress._h if progress else None,
                                         C.byref(st))
        return rc, st.as_dict()

    def clear(self) -> None:
        N.check(N.lib().dxmcg_world_clear_tally(self._h))

    def tally(self):
        e = np.zeros(self.N)
        e2 = np.zeros(self.N)
        c = np.zeros(self.N, dtype=np.uint64)
        N.check(N.lib().dxmcg_world_read_tally(self._h, N.ptr(e, C.c_double), N.ptr(e2, C.c_double),
                                               N.ptr(c, C.c_uint64)))
        return e, e2, c

    def dose(self, out=None):
        """(dose mGy, variance, events) per voxel; `out` may supply the three arrays
        (e.g. pinned host memory)."""
        if out is not None:
            d, v, c = out
        else:
            d = np.zeros(self.N)
            v = np.zeros(self.N)
            c = np.zeros(self.N, dtype=np.uint64)
        N.check(N.lib().dxmcg_world_read_dose(self._h, N.ptr(d, C.c_double), N.ptr(v, C.c_double),
                                              N.ptr(c, C.c_uint64)))
        return d, v, c

    def tables(self, material: int):
        xs = np.zeros((N.NE, 4), dtype=np.float32)
        mj = np.zeros(N.NE, dtype=np.float32)
        N.check(N.lib().dxmcg_world_tables(self._h, material, N.ptr(xs, C.c_float), N.ptr(mj, C.c_float)))
        return xs, mj

    def packed_density(self):
        d = np.zeros(self.N, dtype=np.float32)
        m = np.zeros(self.N, dtype=np.uint8)
        N.check(N.lib().dxmcg_world_packed_density(self._h, N.ptr(d, C.c_float), N.ptr(m, C.c_uint8)))
        return d, m

    def sample_source(self, beam: dict, n: int, options=None) -> np.ndarray:
        b, keep = N.make_beam(beam)
        out = np.zeros((n, 8))
        opts = options if options is not None else run_options()
        N.check(N.lib().dxmcg_sample_source(self._h, C.byref(b), C.byref(opts), n, N.ptr(out, C.c_double)))
        return out

    def organ_dose(self, organ: np.ndarray, n_organs: int, delete_air_dose: bool = True) -> dict:
        """Organ dose table straight from the tally (mGy)."""
        o = np.ascontiguousarray(organ, dtype=np.uint8).reshape(-1)
        if o.size != self.N:
            raise ValueError("organ array size does not match the world")
        out = (N.OrganDose * n_organs)()
        N.check(N.lib().dxmcg_world_organ_dose(self._h, N.ptr(o, C.c_uint8), n_organs, int(delete_air_dose), out))
        return _organ_rows(out, n_organs)

    def dose_postprocessed(self, delete_air_dose: bool = True):
        """(dose, variance, count as float64, micro_gray) as the worker stores them:
        air voxels zeroed, uGy (x1e3, variance x1e6) when the maximum is below 1 mGy."""
        d = np.zeros(self.N)
        v = np.zeros(self.N)
        c = np.zeros(self.N)
        mu = C.c_int(0)
        N.check(N.lib().dxmcg_world_read_dose_postprocessed(self._h, int(delete_air_dose), N.ptr(d, C.c_double),
                                                            N.ptr(v, C.c_double), N.ptr(c, C.c_double),
                                                            C.byref(mu)))
        return d, v, c, bool(mu.value)

    def autotune(self, beam: dict, options: N.RunOptions | None = None, sample_histories: int = 0):
        """Fastest launch shape for this beam: (options with block_size, interact_batch
        and refill_batch set, histories per second of the best trial)."""
        b, keep = N.make_beam(beam)
        opts = N.RunOptions.from_buffer_copy(options if options is not None else run_options())
        rate = C.c_double(0)
        N.check(N.lib().dxmcg_autotune(self._h, C.byref(b), C.byref(opts), sample_histories, C.byref(rate)))
        return opts, rate.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().dxmcg_world_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Several (world, beam, options) jobs in one persistent launch over a shared
    history queue, replayed as a CUDA graph by run().  The worlds must outlive it."""

    def __init__(self, jobs: list[tuple[GpuWorld, dict, N.RunOptions | None]]):
        n = len(jobs)
        if n < 1:
            raise ValueError("a batch needs at least one job")
        self.worlds = [w for w, _, _ in jobs]  # keeps the worlds alive
        beams = (N.Beam * n)()
        opts = (N.RunOptions * n)()
        self._keep = []
        for k, (w, beam, o) in enumerate(jobs):
            b, keep = N.make_beam(beam)
            beams[k] = b
            self._keep.append(keep)
            opts[k] = o if o is not None else run_options()
        handles = (C.c_void_p * n)(*[w._h for w in self.worlds])
        h = C.c_void_p()
        N.check(N.lib().dxmcg_batch_create(n, handles, beams, opts, C.byref(h)))
        self._h = h
        self.n_jobs = n

    def info(self):
        """(histories per job, calibration factor per job)"""
        hist = np.zeros(self.n_jobs, dtype=np.uint64)
        cal = np.zeros(self.n_jobs)
        N.check(N.lib().dxmcg_batch_info(self._h, None, N.ptr(hist, C.c_uint64), N.ptr(cal, C.c_double)))
        return hist, cal

    def run(self) -> dict:
        st = N.Stats()
        N.check(N.lib().dxmcg_batch_run(self._h, C.byref(st)))
        return st.as_dict()

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().dxmcg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Denoiser:
    """The dose denoiser (a 3D convolutional encoder-decoder run by the library's
    kernels).  Tensors passed in and out are CUDA tensors (torch is used as the
    device-memory container only): inputs bf16 [B, D, H, W, 16], targets and
    predictions float32 [B, D, H, W]."""

    def __init__(self, channels=(16, 32, 64, 128), seed=0, conv_path=0):
        cfg = N.DenoiserConfig()
        cfg.levels = len(channels)
        for k, c in enumerate(channels):
            cfg.channels[k] = int(c)
        cfg.seed = seed
        cfg.conv_path = conv_path
        h = C.c_void_p()
        N.check(N.lib().dxmcg_denoiser_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self.channels = tuple(int(c) for c in channels)
        n = C.c_uint64(0)
        N.check(N.lib().dxmcg_denoiser_param_count(self._h, C.byref(n)))
        self.n_params = n.value

    @staticmethod
    def _stream(stream):
        return C.c_void_p(stream.cuda_stream) if stream is not None else None

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.n_params, dtype=np.float32)
        N.check(N.lib().dxmcg_denoiser_get_params(self._h, N.ptr(out, C.c_float)))
        return out

    def set_params(self, params) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters")
        N.check(N.lib().dxmcg_denoiser_set_params(self._h, N.ptr(p, C.c_float)))

    def grads(self) -> np.ndarray:
        out = np.zeros(self.n_params, dtype=np.float32)
        N.check(N.lib().dxmcg_denoiser_get_grads(self._h, N.ptr(out, C.c_float)))
        return out

    def forward(self, x, out=None, stream=None):
        import torch

        B, D, H, W, _ = x.shape
        if out is None:
            out = torch.empty((B, D, H, W), dtype=torch.float32, device=x.device)
        N.check(N.lib().dxmcg_denoiser_forward(self._h, C.c_void_p(x.data_ptr()), B, D, H, W,
                                               C.c_void_p(out.data_ptr()), self._stream(stream)))
        return out

    def backward(self, x, target, stream=None, want_loss: bool = True):
        """Forward, L1 loss and gradients; returns the mean loss, or None without
        want_loss (the call then only queues work and does not wait for the GPU)."""
        B, D, H, W, _ = x.shape
        loss = C.c_double(0)
        N.check(N.lib().dxmcg_denoiser_backward(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(target.data_ptr()),
                                                B, D, H, W, C.byref(loss) if want_loss else None,
                                                self._stream(stream)))
        return loss.value if want_loss else None

    def adam(self, lr: float, stream=None) -> None:
        N.check(N.lib().dxmcg_denoiser_adam(self._h, C.c_float(lr), self._stream(stream)))

    def train_step(self, x, target, lr: float, stream=None, want_loss: bool = True):
        loss = self.backward(x, target, stream, want_loss)
        self.adam(lr, stream)
        return loss

    def set_wait_limit(self, polls: int) -> None:
        """Hand-over wait limit of the tcgen05 convolution (0: default); see
        dxmcg_denoiser_set_wait_limit."""
        N.check(N.lib().dxmcg_denoiser_set_wait_limit(self._h, int(polls)))

    def denoise_world(self, world: "GpuWorld", scale: float = 0.0, readback: bool = True):
        """(denoised dose in mGy per voxel, scale used); without readback the dose stays
        in device memory and None is returned in its place."""
        out = np.zeros(world.N) if readback else None
        s = C.c_double(0)
        N.check(N.lib().dxmcg_world_denoise(world._h, self._h, scale, N.ptr(out, C.c_double) if readback else None,
                                            C.byref(s)))
        return out, s.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().dxmcg_denoiser_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def prepare_input(dose, density, material, scale: float, out=None, stream=None):
    """The denoiser's 16 input channels from CUDA tensors (float32 dose and density,
    uint8 material) of one volume [D, H, W]."""
    import torch

    n = dose.numel()
    if out is None:
        out = torch.empty((*dose.shape, 16), dtype=torch.bfloat16, device=dose.device)
    N.check(N.lib().dxmcg_denoiser_prepare_input(C.c_void_p(dose.data_ptr()), C.c_void_p(density.data_ptr()),
                                                 C.c_void_p(material.data_ptr()), n, scale,
                                                 C.c_void_p(out.data_ptr()), Denoiser._stream(stream)))
    return out


def siddon_trace(origins, directions, dims, spacing, cap=4096):
    o = np.ascontiguousarray(origins, dtype=np.float32).reshape(-1, 3)
    d = np.ascontiguousarray(directions, dtype=np.float32).reshape(-1, 3)
    n = o.shape[0]
    dm = np.ascontiguousarray(dims, dtype=np.int32)
    sp = np.ascontiguousarray(spacing, dtype=np.float32)
    idx = np.zeros((n, cap), dtype=np.int64)
    ln = np.zeros((n, cap), dtype=np.float32)
    cnt = np.zeros(n, dtype=np.int32)
    N.check(N.lib().dxmcg_siddon_trace(n, N.ptr(o, C.c_float), N.ptr(d, C.c_float), N.ptr(dm, C.c_int32),
                                       N.ptr(sp, C.c_float), cap, N.ptr(idx, C.c_int64), N.ptr(ln, C.c_float),
                                       N.ptr(cnt, C.c_int32)))
    return [(idx[r, :cnt[r]].copy(), ln[r, :cnt[r]].copy()) for r in range(n)]


def history_stream(seed: int, stream: int, h0: int, n_hist: int, n_draws: int) -> np.ndarray:
    out = np.zeros((n_hist, n_draws), dtype=np.uint32)
    N.check(N.lib().dxmcg_history_stream(seed, stream, h0, n_hist, n_draws, N.ptr(out, C.c_uint32)))
    return out


def sample_compton(energies, zw, correction, uniforms):
    E = np.ascontiguousarray(energies, dtype=np.float64)
    U = np.ascontiguousarray(uniforms, dtype=np.float64)
    n, stride = U.shape
    eo = np.zeros(n)
    co = np.zeros(n)
    used = np.zeros(n, dtype=np.int32)
    m = N.Material.from_dict(zw)
    N.check(N.lib().dxmcg_sample_compton(n, N.ptr(E, C.c_double), C.byref(m), correction, N.ptr(U, C.c_double), stride,
                                         N.ptr(eo, C.c_double), N.ptr(co, C.c_double), N.ptr(used, C.c_int32)))
    return eo, co, used


def sample_photoelectric(energies, zw, uniforms):
    """Correction level 2 photoelectric absorption: (fluorescence energy, its z
    cosine, uniforms used) per energy."""
    E = np.ascontiguousarray(energies, dtype=np.float64)
    U = np.ascontiguousarray(uniforms, dtype=np.float64)
    n, stride = U.shape
    eo = np.zeros(n)
    dz = np.zeros(n)
    used = np.zeros(n, dtype=np.int32)
    m = N.Material.from_dict(zw)
    N.check(N.lib().dxmcg_sample_photoelectric(n, N.ptr(E, C.c_double), C.byref(m), N.ptr(U, C.c_double), stride,
                                               N.ptr(eo, C.c_double), N.ptr(dz, C.c_double),
                                               N.ptr(used, C.c_int32)))
    return eo, dz, used


def sample_rayleigh(energies, zw, uniforms):
    E = np.ascontiguousarray(energies, dtype=np.float64)
    U = np.ascontiguousarray(uniforms, dtype=np.float64)
    n, stride = U.shape
    co = np.zeros(n)
    used = np.zeros(n, dtype=np.int32)
    m = N.Material.from_dict(zw)
    N.check(N.lib().dxmcg_sample_rayleigh(n, N.ptr(E, C.c_double), C.byref(m), N.ptr(U, C.c_double), stride,
                                          N.ptr(co, C.c_double), N.ptr(used, C.c_int32)))
    return co, used
