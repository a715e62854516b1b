"""Build the CUDA library libtailor_gb300.so in-tree for sm_103a.

Each translation unit is compiled in parallel: CUDA sources with nvcc,
host-only C++ sources (*.cpp) with the system compiler; the files that
must reproduce the reference's arithmetic bit for bit are compiled with
--fmad=false (no contraction of a*b+c into one fused operation).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT_DIR = HERE / "lib"
LIB = OUT_DIR / "libtailor_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
          "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
EXACT = {"tlr_fields.cu", "tlr_assemble.cu", "tlr_points.cu", "tlr_bc.cu"}


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required")
    return exe


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _compile(src: Path, obj: Path, verbose: bool) -> str:
    if src.suffix == ".cpp":  # host-only code: the system C++ compiler
        cxx = shutil.which("g++") or "c++"
        cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c", str(src),
               "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{cxx} failed for {src.name}:\n{r.stderr}")
        return r.stderr
    flags = list(COMMON)
    if src.name in EXACT:
        flags.append("--fmad=false")
    if verbose:
        flags += ["-Xptxas", "-v"]
    cmd = [nvcc(), *ARCH, *flags, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stderr}")
    return r.stderr


def build(force: bool = False, verbose: bool = False) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    srcs = sources()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [
        HERE.parent / "include" / "tailor_gb300.h"]
    newest = max(p.stat().st_mtime for p in srcs + headers)
    if LIB.exists() and not force and LIB.stat().st_mtime > newest:
        return LIB
    objs = [OUT_DIR / (s.stem + ".o") for s in srcs]
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        logs = list(ex.map(lambda so: _compile(*so, verbose), zip(srcs, objs)))
    if verbose:
        for s, log in zip(srcs, logs):
            print(f"== {s.name}\n{log}", file=sys.stderr)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    for o in objs:
        o.unlink(missing_ok=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
