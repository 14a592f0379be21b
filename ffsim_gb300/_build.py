"""In-tree build of the CUDA library ``libffgb.so`` (sm_103a).

``build()`` regenerates the window code, then compiles the translation units
in parallel with nvcc and links the shared library next to this file.
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
BUILD = HERE / "_build"
LIB = HERE / "libffgb.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-Xptxas", "-O3"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build ffsim_gb300")


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose and (res.stdout or res.stderr):
        print(res.stdout + res.stderr, flush=True)


# window-stage kernels: (window size, first class, last class) per translation
# unit; the large classes of 7- and 8-orbital windows get units of their own
STAGE_UNITS = [(4, 0, 4), (5, 0, 5), (6, 0, 6), (7, 0, 2), (7, 3, 3), (7, 4, 4), (7, 5, 7),
               (8, 0, 2), (8, 3, 3), (8, 4, 4), (8, 5, 5), (8, 6, 8)]


def build(verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    subprocess.run([sys.executable, str(CSRC / "gen_windows.py"), str(BUILD / "windows_gen.cuh")],
                   check=True)
    nvcc = _nvcc()
    inc = ["-I", str(BUILD), "-I", str(CSRC)]
    flags = NVFLAGS + (extra_flags or [])
    units = [("ffgb.cu", "ffgb.o", []), ("plan.cpp", "plan.o", []), ("stages.cu", "stages.o", []), ("grad.cu", "grad.o", []), ("peaks.cu", "peaks.o", []), ("resident.cu", "resident.o", [])] + [
        (f"inst_{i}.cu", f"inst_{i}.o", []) for i in range(5)] + [
        ("stage_inst.cu", f"stage_b{b}_k{k0}.o", [f"-DWIN_B={b}", f"-DWIN_K0={k0}", f"-DWIN_K1={k1}"])
        for b, k0, k1 in STAGE_UNITS]
    cmds = [[nvcc, *ARCH, *flags, *defs, *inc, "-c", str(CSRC / src), "-o", str(BUILD / obj)]
            for src, obj, defs in units]
    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        list(ex.map(lambda c: _run(c, verbose), cmds))
    tmp = BUILD / "libffgb.so.tmp"
    _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *[str(BUILD / o) for _, o, _ in units],
          "-lcudart"], verbose)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
