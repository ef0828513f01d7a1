"""In-tree build of the native parts.

* ``_build/libnanogi.so`` -- the C-ABI library (host C++ + sm_103a CUDA), the product.
* ``_build/nanogi``       -- the command-line renderer linked against it.

Compilation is parallel and incremental (objects are rebuilt when a source or header is
newer). Only g++ and nvcc are needed; no cmake.
"""
from __future__ import annotations

import concurrent.futures
import os
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
ROOT = PKG.parent
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

HOST_SOURCES = ["yaml_lite.cpp", "obj_loader.cpp", "scene.cpp", "image_io.cpp", "texture.cpp", "capi.cpp"]
CUDA_SOURCES = ["render.cu", "bvh_build.cu"]
LIB = OUT / "libnanogi.so"
CLI = OUT / "nanogi"


class BuildError(RuntimeError):
    pass


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise BuildError("command failed:\n  " + " ".join(cmd) + "\n" + proc.stdout)


def _headers() -> list[Path]:
    hs = list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    return hs


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


# render.cu: FP32 division and square root as the hardware approximations (within 2 ulp) instead of
# the IEEE-rounded sequences. This changes the FP32 shading arithmetic only: the traversal and the
# watertight triangle test are written with explicit round-to-nearest intrinsics (__fdiv_rn,
# __fmul_rn, __frcp_rn), which the flags leave alone, and FP64 arithmetic is unaffected. Measured on
# the 1.55M-triangle terrain: path-logic launches 0.261 -> 0.242 ms, 15.04 -> 14.71 ms per 16-spp
# render; Cornell box 4357 -> 4482 Mrays/s.
CUDA_FLAGS = {"render.cu": ["-prec-div=false", "-prec-sqrt=false"]}


def _compile(src: Path, obj: Path, headers: list[Path]) -> Path:
    if not _stale(obj, [src, Path(__file__)] + headers):
        return obj
    inc = ["-I", str(CSRC), "-I", str(ROOT / "include")]
    if src.suffix == ".cu":
        cmd = [NVCC, "-std=c++17", "-O3", "-lineinfo", *CUDA_FLAGS.get(src.name, []), *ARCH, "-Xcompiler",
               "-fPIC,-fvisibility=hidden", *inc, "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-fvisibility=hidden", "-Wall", "-Wextra",
               "-I", str(CUDA_HOME / "include"), *inc, "-c", str(src), "-o", str(obj)]
    _run(cmd)
    return obj


def build_library(jobs: int | None = None, verbose: bool = False) -> Path:
    """Compiles every translation unit for sm_103a and links libnanogi.so and the CLI."""
    OUT.mkdir(exist_ok=True)
    headers = _headers()
    srcs = [CSRC / s for s in HOST_SOURCES + CUDA_SOURCES]
    objs = [OUT / (s.stem + (".cu.o" if s.suffix == ".cu" else ".o")) for s in srcs]
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(_compile, s, o, headers) for s, o in zip(srcs, objs)]
        for f in futs:
            f.result()
    if _stale(LIB, objs):
        _run([NVCC, "-shared", *ARCH, "-o", str(LIB), *map(str, objs), "-Xcompiler", "-fPIC"])
    cli_src = CSRC / "cli.cpp"
    if _stale(CLI, [cli_src, LIB] + headers):
        _run(["g++", "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(cli_src), "-o", str(CLI),
              "-L", str(OUT), "-lnanogi", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print(f"built {LIB} and {CLI}")
    return LIB


if __name__ == "__main__":
    build_library(verbose=True)
