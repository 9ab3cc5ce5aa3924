"""Build the CUDA library ``hydroexa_gb300/libhydroexa_gb300.so`` for sm_103a.

Eight translation units compiled in parallel, then linked:

* ``hx_exact.cu``  -- exact arithmetic form, ``--fmad=false`` (no multiply-add
  contraction, the reference's host rounding); tags and restriction kernels.
* ``hx_fast.cu``   -- fast arithmetic form (shared reciprocals, contraction).
* ``hx_capi.cu``   -- the C ABI declared in ``include/hydroexa_gb300.h``.
* ``hx_noalloc.cu`` -- the allocation-free time loop (scratch in a static device array).
* ``hx_ensemble.cu`` -- the batched-ensemble plan, dt initialisation and CUDA-graph replay.
* ``hx_adjoint.cu`` -- the hand-written adjoint of the hydrostatic-Roe time loop and its drivers.
* ``hx_roofs.cu`` -- the FP64 issue-rate probe (the roof the FP64-bound kernels are reported against).
* ``hx_boxlevel.cu`` -- the multi-box level (same-level ghosts read from neighbouring boxes).

The build is in-tree (objects in ``_build/``), takes well under a minute, and
needs only nvcc; the CUDA runtime is linked statically so the library loads
with or without PyTorch in the process.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = ROOT / "_build"
LIB = PKG / "libhydroexa_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(ROOT / "include")]
UNITS = {
    "hx_exact": ["--fmad=false"],
    "hx_fast": [],
    "hx_capi": [],
    "hx_noalloc": [],
    "hx_ensemble": [],
    "hx_adjoint": [],
    "hx_roofs": [],
    "hx_boxlevel": [],
    "hx_plotfile": [],
}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (Path(cand).exists() or cand == "nvcc"):
            return cand
    return "nvcc"


def _sources_newer(target: Path) -> bool:
    if not target.exists():
        return True
    mt = target.stat().st_mtime
    deps = list(CSRC.glob("*")) + [ROOT / "include" / "hydroexa_gb300.h", Path(__file__)]
    return any(d.stat().st_mtime > mt for d in deps if d.is_file())


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link the library if any source is newer than it."""
    if not force and not _sources_newer(LIB):
        return LIB
    OBJ.mkdir(exist_ok=True)
    nvcc = _nvcc()

    def compile_unit(name: str):
        cmd = [nvcc, *ARCH, *COMMON, *UNITS[name], "-c", str(CSRC / f"{name}.cu"), "-o", str(OBJ / f"{name}.o")]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}.cu:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        logs = list(ex.map(compile_unit, UNITS))
    if verbose:
        for log in logs:
            sys.stderr.write(log)
    tmp = LIB.with_suffix(f".so.{os.getpid()}.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *[str(OBJ / f"{n}.o") for n in UNITS]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
