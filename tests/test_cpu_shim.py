"""The header-only dxmc:: layer (include/dxmc/) compiles, and OpenDXMC's own beam
specialisation (src/libopendxmc/dxmc_specialization.cpp: the DXBeam wrapper and the
Beam variant over all six beam types) compiles against it unchanged.  No GPU."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
# the reference project tree, when mounted: $OPENDXMC_REFERENCE, else a checkout named
# "reference" beside this repository
REFERENCE = Path(os.environ.get("OPENDXMC_REFERENCE") or ROOT.parent / "reference") / "src" / "libopendxmc"


def gxx():
    g = shutil.which("g++")
    if not g:
        pytest.skip("g++ not available")
    return g


def test_dropin_worker_compiles():
    r = subprocess.run([gxx(), "-std=c++20", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", f"-I{ROOT / 'include'}",
                        str(ROOT / "tests" / "cpp" / "worker_dropin.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("header", sorted(str(p.relative_to(ROOT / "include")) for p in (ROOT / "include").rglob("*.hpp")))
def test_each_header_stands_alone(header, tmp_path):
    src = tmp_path / "one.cpp"
    src.write_text(f'#include "{header}"\nint main() {{ return 0; }}\n')
    r = subprocess.run([gxx(), "-std=c++20", "-Wall", "-Werror", "-fsyntax-only", f"-I{ROOT / 'include'}", str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.skipif(not (REFERENCE / "dxmc_specialization.cpp").exists(), reason="reference tree not mounted (set OPENDXMC_REFERENCE)")
def test_reference_beam_specialisation_compiles_against_the_layer():
    r = subprocess.run([gxx(), "-std=c++20", "-fsyntax-only", f"-I{ROOT / 'include'}", f"-I{REFERENCE}",
                        str(REFERENCE / "dxmc_specialization.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_host_side_layer_runs_without_a_gpu(engine, tmp_path):
    """Tube, Material and beam exposures are host computations of the engine."""
    from opendxmc_gb300 import native

    prog = tmp_path / "host.cpp"
    prog.write_text(r'''
#include <cstdio>
#include "dxmc/beams/ctspiralbeam.hpp"
#include "dxmc/material/material.hpp"
#include "dxmc/material/nistmaterials.hpp"
int main() {
    dxmc::Tube tube(120.0);
    tube.setAlFiltration(6.0);
    const auto e = tube.getEnergy();
    const auto w = tube.getSpecter(e, true);
    double s = 0; for (double x : w) s += x;
    const auto water = dxmc::Material<5>::byNistName("Water, Liquid").value();
    dxmc::CTSpiralBeam<false> ct({0, 0, -10}, {0, 0, 10}, {{13, 6.0}});
    ct.setCollimation(4.0);
    ct.setStepAngleDeg(5.0);
    std::printf("%zu %.12f %.6f %.6f %llu %.6f\n", e.size(), s, tube.mmAlHalfValueLayer(),
        water.attenuationValues(60.0).sum(), (unsigned long long)ct.numberOfExposures(),
        dxmc::NISTMaterials::density("Water, Liquid"));
    return 0;
}
''')
    exe = tmp_path / "host"
    r = subprocess.run([gxx(), "-std=c++20", "-O1", f"-I{ROOT / 'include'}", str(prog), "-o", str(exe),
                        f"-L{native.LIB_PATH.parent}", "-ldxmcg", f"-Wl,-rpath,{native.LIB_PATH.parent}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert int(out[0]) == 120
    assert float(out[1]) == pytest.approx(1.0)
    assert float(out[2]) == pytest.approx(engine.tube_al_hvl(120.0, {13: 6.0}), rel=1e-5)
    p, ic, co = engine.attenuation({1: 11.19, 8: 88.81}, [60.0])
    assert float(out[3]) == pytest.approx(float(p[0] + ic[0] + co[0]), rel=1e-5)
    assert int(out[4]) == 360
    assert float(out[5]) == 1.0
