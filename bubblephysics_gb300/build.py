"""Builds the native library in-tree: libbubblephysics_gb300.so (CUDA, sm_103a only).

Translation units compile in parallel with nvcc; the library is linked with -shared. Flags that matter for parity:
-fmad=false (no multiply-add fusion in device code) and the default IEEE division / square root (no fast math),
so every FP32 operation rounds exactly like the CPU oracle's written order; host code gets -ffp-contract=off.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE_DIR = Path(__file__).resolve().parent
CSRC = PACKAGE_DIR / "csrc"
BUILD_DIR = PACKAGE_DIR / "_build"
LIBRARY = PACKAGE_DIR / "libbubblephysics_gb300.so"
SOURCES = ["bp_step.cu", "bp_noalloc.cu", "bp_capi.cu", "bp_aux.cu", "bp_server.cu", "bp_contour.cu", "bp_sensor.cu", "bp_events.cu",
           "bp_rigid.cu"]
# bp_step_variant.cu is compiled once per (kernel, block width, tree) variant: the persistent step kernels are the
# largest functions of the library and compile in parallel this way.
VARIANT_SOURCE = "bp_step_variant.cu"
VARIANTS = [(kind, threads, tree) for kind in (0, 1) for threads in (128, 256, 512) for tree in (0, 1)]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-Xcompiler", "-fPIC,-ffp-contract=off", "-diag-suppress", "177"]


def _nvcc() -> str:
    for candidate in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if candidate and Path(candidate).exists():
            return candidate
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build bubblephysics_gb300")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compiles every CUDA translation unit for sm_103a and links the shared library. Returns its path."""
    nvcc = _nvcc()
    BUILD_DIR.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [PACKAGE_DIR.parent / "include" / "bubblephysics.h"]
    objects = []
    jobs = []
    units = [(CSRC / name, BUILD_DIR / (name + ".o"), []) for name in SOURCES]
    for kind, threads, tree in VARIANTS:
        tag = f"{'served' if kind else 'persistent'}_{threads}_{tree}"
        units.append((CSRC / VARIANT_SOURCE, BUILD_DIR / f"bp_step_{tag}.o",
                      [f"-DBP_VARIANT_KIND={kind}", f"-DBP_VARIANT_THREADS={threads}", f"-DBP_VARIANT_TREE={tree}"]))
    for src, obj, defines in units:
        objects.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *defines, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        result = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or result.returncode != 0:
            sys.stderr.write(result.stdout + result.stderr)
        if result.returncode != 0:
            raise RuntimeError("nvcc failed: " + " ".join(cmd))

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as pool:
        list(pool.map(run, jobs))
    if force or jobs or _stale(LIBRARY, objects):
        tmp = LIBRARY.with_suffix(".so.tmp")
        run([nvcc, *ARCH, "-shared", "--cudart", "static", "-o", str(tmp), *map(str, objects)])
        os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="--force" in sys.argv))
