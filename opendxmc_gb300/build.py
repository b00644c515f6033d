"""Build libdxmcg.so (the CUDA engine + C ABI) in-tree with nvcc for sm_103a.

Translation units compile in parallel; the result lands in
opendxmc_gb300/_lib/libdxmcg.so next to the package (git-ignored).
Run as `python -m opendxmc_gb300.build` or through __graft_entry__.build().
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_lib"
OBJ_DIR = PKG / "_build"
LIB = OUT_DIR / "libdxmcg.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no contraction into fused multiply-adds, so that x86-64 and aarch64 hosts
# round the FP64 table and geometry arithmetic alike
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden,-O2,-ffp-contract=off",
          f"-I{ROOT / 'include'}"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libdxmcg")


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _compile(src: Path, verbose_ptxas: bool) -> Path:
    obj = OBJ_DIR / (src.name + ".o")
    deps = [src] + list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "dxmcg.h"]
    if obj.exists() and obj.stat().st_mtime > max(d.stat().st_mtime for d in deps if d.exists()):
        return obj
    cmd = [nvcc(), *ARCH, *COMMON, "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cu" and verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas and r.stderr.strip():
        (OBJ_DIR / (src.name + ".ptxas.txt")).write_text(r.stderr)
    return obj


def build(verbose_ptxas: bool = True, force: bool = False) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    OBJ_DIR.mkdir(exist_ok=True)
    if force:
        for o in OBJ_DIR.glob("*.o"):
            o.unlink()
    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    if LIB.exists() and LIB.stat().st_mtime > max(o.stat().st_mtime for o in objs):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    p = build(force="--force" in sys.argv)
    print(p)
    for f in sorted(OBJ_DIR.glob("*.ptxas.txt")):
        print(f.read_text())
