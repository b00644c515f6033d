"""The allocation-free transport entry point, through the C ABI.

dxmcg_transport_run_noalloc serves callers that may not allocate device memory
while they run (their GPU memory comes from their own pool, or they hold a fixed
device budget): they pass their own device arrays and the library keeps its
scratch in a static device array.  Here torch plays that caller: it owns the
density, material and tally arrays.  The result must match the world-based entry
point (dxmcg_transport_run) on the same inputs and streams, on two calls in a row
that share the static scratch.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from opendxmc_gb300 import phantoms as P

pytestmark = pytest.mark.gpu


def _call(N, ph, d_dens, d_mat, d_tally, beam_params, opts, mats=None):
    b, keep = N.make_beam(beam_params)
    materials = mats if mats is not None else ph.materials
    mat_arr = (N.Material * len(materials))(*[N.Material.from_dict(m) for m in materials])
    dims = (C.c_int32 * 3)(*ph.dims)
    sp = (C.c_double * 3)(*ph.spacing)
    st = N.Stats()
    rc = N.lib().dxmcg_transport_run_noalloc(dims, sp, C.c_void_p(d_dens.data_ptr()), C.c_void_p(d_mat.data_ptr()),
                                             mat_arr, len(materials), 1, C.byref(b), C.byref(opts),
                                             C.c_void_p(d_tally.data_ptr()), None, C.byref(st))
    return rc, st.as_dict()


@pytest.mark.parametrize("two_region", [0, 1])
def test_noalloc_matches_world_entry_point_on_two_calls(gpu, two_region):
    """Both entry points, one or two Woodcock regions (the two-region box of the
    caller's materials is found on the device, into the static scratch)."""
    import torch

    from opendxmc_gb300 import native as N

    ph = P.torso_phantom(dims=(64, 64, 50), spacing=(0.6, 0.6, 0.6), seed=4)
    gw = gpu.GpuWorld(ph.dims, ph.spacing, ph.materials)
    gw.set_data(ph.density, ph.material)
    gw.build()
    # the caller's arrays: the densities exactly as the world entry point stores them
    dens, mat = gw.packed_density()
    d_dens = torch.from_numpy(dens).to("cuda:0")
    d_mat = torch.from_numpy(mat).to("cuda:0")
    d_tally = torch.zeros((ph.n_voxels, 4), dtype=torch.float64, device="cuda:0")  # 32-byte records
    beam = P.ct_spiral_params(particles=1500)

    for seed in (5, 6):
        gw.clear()
        ref = gw.run(beam, gpu.run_options(seed=seed, stream=2, two_region=two_region))
        e_ref, e2_ref, c_ref = gw.tally()
        d_tally.zero_()
        torch.cuda.synchronize()
        rc, st = _call(N, ph, d_dens, d_mat, d_tally, beam, gpu.run_options(seed=seed, stream=2, two_region=two_region))
        assert rc == 0, N.lib().dxmcg_last_error().decode()
        rec = d_tally.cpu().numpy()
        counts = rec[:, 2].copy().view(np.uint64)
        for k in ("n_histories", "n_missed", "n_visits", "n_photo", "n_compton", "n_rayleigh", "n_interacted"):
            assert st[k] == ref[k], k
        np.testing.assert_array_equal(counts, c_ref)
        np.testing.assert_allclose(rec[:, 0], e_ref, rtol=1e-9, atol=0)
        np.testing.assert_allclose(rec[:, 1], e2_ref, rtol=1e-9, atol=0)
        assert st["e_deposited"] == pytest.approx(ref["e_deposited"], rel=1e-9)


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    import torch

    from opendxmc_gb300 import native as N

    ph = P.water_cylinder_phantom(dims=(16, 16, 8), spacing=(0.8, 0.8, 2.0))
    d_dens = torch.from_numpy(ph.density.astype(np.float32)).to("cuda:0")
    d_mat = torch.from_numpy(ph.material).to("cuda:0")
    d_tally = torch.zeros((ph.n_voxels, 4), dtype=torch.float64, device="cuda:0")
    beam = P.dx_beam_params(particles=100, exposures=1)
    rc, _ = _call(N, ph, d_dens, d_mat, d_tally, beam, gpu.run_options(), mats=[P.WATER] * 17)
    assert rc == -7 and b"16 materials" in N.lib().dxmcg_last_error()
    beam_many = dict(beam, n_exposures=5000)
    rc, _ = _call(N, ph, d_dens, d_mat, d_tally, beam_many, gpu.run_options())
    assert rc == -7 and b"4096 exposures" in N.lib().dxmcg_last_error()
    # within limits it runs
    rc, st = _call(N, ph, d_dens, d_mat, d_tally, beam, gpu.run_options())
    assert rc == 0 and st["n_histories"] == 100


def test_noalloc_refuses_ct_calibration(gpu):
    """A CT beam with dose normalisation and a CTDI target needs a CTDI phantom run,
    which allocates: the allocation-free call refuses it with an argument error."""
    import torch

    from opendxmc_gb300 import native as N

    ph = P.water_cylinder_phantom(dims=(16, 16, 8), spacing=(0.8, 0.8, 2.0))
    d_dens = torch.from_numpy(ph.density.astype(np.float32)).to("cuda:0")
    d_mat = torch.from_numpy(ph.material).to("cuda:0")
    d_tally = torch.zeros((ph.n_voxels, 4), dtype=torch.float64, device="cuda:0")
    beam = dict(P.ct_spiral_params(particles=10, scan_cm=2.0), ctdi_vol_mgy=10.0)
    rc, _ = _call(N, ph, d_dens, d_mat, d_tally, beam, gpu.run_options(normalize=1))
    assert rc == -1 and b"CTDI" in N.lib().dxmcg_last_error()
    # without normalisation the same beam runs
    rc, st = _call(N, ph, d_dens, d_mat, d_tally, beam, gpu.run_options(normalize=0))
    assert rc == 0 and st["n_histories"] > 0
