"""Build recipe of the GB300 library: nvcc for the kernels, the host C++
compiler for the driver, the C ABI and the headless CLI.

Outputs (git-ignored, in-tree):
    lib/libbubble_gb300.so   the C-ABI shared library (include/bubble.h)
    lib/bubble-sim           the --headless command-line driver

Three kernel translation units differ only in their arithmetic flags:
    kernels_strict.cu  --fmad=false  (bit-identical with an IEEE CPU restatement)
    kernels_fast.cu    --fmad=true   (FMA contraction, approximate rcp/sqrt)
    kernels_f64.cu     --fmad=false  (the FP64 CUDA oracle)
All are compiled for sm_103a only.  Usage: python build.py [--force] [-j N]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "lib"
INCLUDE = HERE.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def nvcc() -> str:
    return str(cuda_home() / "bin" / "nvcc")


NVCC_COMMON = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                      "--expt-relaxed-constexpr", "-I", str(INCLUDE)]
CXX_COMMON = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wextra", "-Wno-unused-parameter"]

KERNEL_UNITS = {
    "kernels_strict.cu": ["--fmad=false"],
    "kernels_fast.cu": ["--fmad=true"],
    "kernels_f64.cu": ["--fmad=false"],
    "diag_noalloc.cu": ["--fmad=false"],
    "render.cu": ["--fmad=false"],
}
HOST_UNITS = ["physics.cpp", "simulation.cpp", "capi.cpp", "tma.cpp", "batch.cpp", "capi_batch.cpp", "server.cpp",
              "render_host.cpp", "checkpoint.cpp"]
CLI_UNITS = ["headless.cpp"]
HEADERS = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def compile_unit(src: str, force: bool, verbose_ptxas: bool = False) -> Path:
    s = CSRC / src
    obj = BUILD / (src + ".o")
    deps = [s] + HEADERS
    if not force and not _stale(obj, deps):
        return obj
    if src.endswith(".cu"):
        cmd = [nvcc()] + NVCC_COMMON + KERNEL_UNITS[src] + ["-c", str(s), "-o", str(obj)]
        if verbose_ptxas:
            cmd += ["-Xptxas", "-v"]
    else:
        cxx = os.environ.get("CXX", "g++")
        cmd = [cxx] + CXX_COMMON + ["-I", str(cuda_home() / "include"), "-I", str(INCLUDE),
                                    "-c", str(s), "-o", str(obj)]
    _run(cmd)
    return obj


def build(force: bool = False, jobs: int | None = None, verbose_ptxas: bool = False) -> Path:
    """Compile every translation unit in parallel and link the library and CLI.

    Returns the path of the shared library."""
    BUILD.mkdir(exist_ok=True)
    LIB.mkdir(exist_ok=True)
    units = list(KERNEL_UNITS) + HOST_UNITS + CLI_UNITS
    jobs = jobs or min(len(units), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = dict(zip(units, ex.map(lambda u: compile_unit(u, force, verbose_ptxas), units)))
    lib = LIB / "libbubble_gb300.so"
    lib_objs = [objs[u] for u in list(KERNEL_UNITS) + HOST_UNITS]
    if force or _stale(lib, lib_objs):
        _run([nvcc()] + ARCH + ["-shared", "-cudart", "static", "-Xcompiler", "-fPIC",
                                "-o", str(lib)] + [str(o) for o in lib_objs] +
             ["-lpthread", "-ldl", "-lrt"])
    cli = LIB / "bubble-sim"
    if force or _stale(cli, [objs["headless.cpp"], lib]):
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-o", str(cli), str(objs["headless.cpp"]), "-L", str(LIB),
              "-lbubble_gb300", "-Wl,-rpath,$ORIGIN"])
    return lib


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-j", "--jobs", type=int, default=None)
    ap.add_argument("--ptxas-v", action="store_true", help="print register/smem usage")
    a = ap.parse_args()
    lib = build(force=a.force, jobs=a.jobs, verbose_ptxas=a.ptxas_v)
    print(lib)
    return 0


if __name__ == "__main__":
    sys.exit(main())
