"""OpenDXMC's worker call sequence on the dxmc:: C++ layer gives the same dose,
variance and event arrays as the same runs driven through the C ABI."""
import json
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from opendxmc_gb300 import phantoms as P
import parity

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def test_cpp_worker_matches_c_abi(gpu, tmp_path):
    from opendxmc_gb300 import native

    gxx = shutil.which("g++")
    assert gxx, "g++ is needed to build the C++ drop-in worker"
    exe = tmp_path / "worker_dropin"
    r = subprocess.run([gxx, "-std=c++20", "-O2", f"-I{ROOT / 'include'}", str(ROOT / "tests/cpp/worker_dropin.cpp"),
                        "-o", str(exe), f"-L{native.LIB_PATH.parent}", "-ldxmcg",
                        f"-Wl,-rpath,{native.LIB_PATH.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ph = parity.small_cylinder()
    dens = tmp_path / "d.f64"
    mat = tmp_path / "m.u8"
    out = tmp_path / "out.bin"
    np.ascontiguousarray(ph.density, dtype=np.float64).tofile(dens)
    np.ascontiguousarray(ph.material, dtype=np.uint8).tofile(mat)
    run = subprocess.run([str(exe), *map(str, ph.dims), *map(str, ph.spacing), str(dens), str(mat), str(out)],
                         capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stderr
    info = json.loads(run.stdout)
    N = ph.n_voxels
    raw = np.fromfile(out, dtype=np.uint8)
    d_cpp = raw[: 8 * N].view(np.float64)
    v_cpp = raw[8 * N: 16 * N].view(np.float64)
    c_cpp = raw[16 * N:].view(np.uint64)

    # the same two runs through the C ABI
    gw = gpu.GpuWorld(ph.dims, ph.spacing, [{7: 80.0, 8: 20.0}, P.WATER, P.BONE], 1)
    gw.set_data(ph.density, ph.material)
    gw.build()
    half = float(np.tan(0.05))
    dx = {"type": 0, "kvp": 70.0, "anode_angle_deg": 12.0, "filters": {13: 2.5}, "particles_per_exposure": 50000,
          "n_exposures": 4, "position": [0, 100, 0], "cosines": [[0, 0, 1], [-1, 0, 0]], "half_angles": [half, half],
          "dap_mgycm2": 10.0}
    ct = {"type": 1, "kvp": 120.0, "anode_angle_deg": 12.0, "filters": {13: 6.0}, "particles_per_exposure": 2000,
          "start": [0, 0, -2], "stop": [0, 0, 2], "start_angle_deg": 0.0, "step_angle_deg": 10.0, "pitch": 1.0,
          "collimation_cm": 2.0, "scan_fov_cm": 50.0, "sdd_cm": 119.0, "ctdi_vol_mgy": 5.0, "ctdi_diameter_cm": 32.0,
          "bowtie": [(0.0, 1.88), (0.0839, 1.49), (0.167, 0.73), (0.39, 0.30)]}
    s_dx = gw.run(dx, gpu.run_options(seed=1, stream=0, normalize=1))
    s_ct = gw.run(ct, gpu.run_options(seed=1, stream=1, normalize=1))
    d, v, c = gw.dose()
    assert info["exposures_dx"] == 4 and info["exposures_ct"] == 72
    assert info["progress"] == [72 * 2000, 72 * 2000] and info["message"] == "Done"
    assert s_dx["calibration"] != 1.0 and s_ct["calibration"] != 1.0
    np.testing.assert_array_equal(c_cpp, c)
    np.testing.assert_allclose(d_cpp, d, rtol=1e-9, atol=0)
    np.testing.assert_allclose(v_cpp, v, rtol=1e-6, atol=1e-300)
