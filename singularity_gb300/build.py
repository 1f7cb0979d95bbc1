"""In-tree build of the native parts: the CUDA library, the C++ CLI and shim.

Everything is compiled for sm_103a only, with plain nvcc / g++ calls run in
parallel (no cmake).  Outputs land in ``singularity_gb300/_build/``:

* ``libsgx.so``      — kernels + C ABI (include/sgx.h)
* ``singularity_cuda_cli`` — the cuda_cli-compatible command line renderer
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code: no floating-point contraction, so x86-64 (which has no FMA in its
# baseline) and aarch64 (whose compilers contract a*b + c by default) give the
# same host results, e.g. the orbital camera the reference computes.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++20", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}"]
CXX_FLAGS = ["-O2", "-std=c++20", "-fPIC", "-Wall", "-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}"]

CUDA_UNITS = ["sgx_trace.cu", "sgx_api.cu", "sgx_batch.cu", "sgx_post.cu", "sgx_probe.cu", "sgx_noalloc.cu", "sgx_diff.cu", "sgx_diff64.cu"]
HOST_UNITS = ["sgx_host.cpp"]


def _nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = Path(cuda) / "bin" / "nvcc"
    return str(cand) if cand.exists() else (shutil.which("nvcc") or "nvcc")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    """Compile libsgx.so (and the CLI) if any source is newer than the output."""
    BUILD.mkdir(parents=True, exist_ok=True)
    headers = (list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.hpp")) + list((CSRC / "render_api").glob("*.hpp"))
               + list(INCLUDE.glob("*.h")))
    nvcc = _nvcc()
    cuda = Path(nvcc).resolve().parent.parent
    jobs = []
    objs = []
    for unit in CUDA_UNITS:
        src = CSRC / unit
        obj = BUILD / (unit + ".o")
        objs.append(obj)
        if force or not _newer(obj, [src] + headers):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    for unit in HOST_UNITS:
        src = CSRC / unit
        obj = BUILD / (unit + ".o")
        objs.append(obj)
        if force or not _newer(obj, [src] + headers):
            jobs.append(["g++", *CXX_FLAGS, f"-I{cuda / 'include'}", "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    lib = BUILD / "libsgx.so"
    if force or jobs or not lib.exists():
        _run([nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart"])
    cli = BUILD / "singularity_cuda_cli"
    cli_srcs = [CSRC / "cuda_backend.cpp", CSRC / "cli_main.cpp"]
    if all(s.exists() for s in cli_srcs) and (force or not _newer(cli, cli_srcs + headers + [lib])):
        _run(["g++", *CXX_FLAGS, f"-I{CSRC / 'render_api'}", "-pthread", f"-I{cuda / 'include'}", *map(str, cli_srcs),
              str(BUILD / "sgx_host.cpp.o"), "-o", str(cli), f"-L{BUILD}", "-lsgx", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print(f"built {lib}")
    return lib


def library_path() -> Path:
    return BUILD / "libsgx.so"


if __name__ == "__main__":
    build_library(force=True, verbose=True)
