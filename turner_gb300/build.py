"""In-tree build of the native libraries (no CMake, no torch extension).

Outputs (git-ignored, rebuilt on every machine):
  turner_gb300/lib/libturner_gb300.so   C ABI + sm_103a kernels + host tree/scenes
  turner_gb300/lib/turner_pathtracer     command-line renderer (pathtracer flags)
  oracle/liboracle.so                    CPU oracle (test infrastructure)
  oracle/libinputs.so                    the host scene generator and kd-tree
                                         builder alone (no CUDA), which the
                                         CPU reference arm of bench.py uses to
                                         make its input
  oracle/_ref/libturner_ref.so           reference checker, only where the
                                         reference sources are present

Host code is compiled with -ffp-contract=off and no -march so it rounds the
same way on x86-64 and aarch64; the wavefront kernels with -fmad=false.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "turner_gb300"
CSRC = PKG / "csrc"
LIB = PKG / "lib"
ORACLE = ROOT / "oracle"
BUILD = ROOT / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(ROOT / "include"), "-I", str(CSRC)]
GXX_COMMON = ["-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-I", str(ROOT / "include")]

# (source, extra flags)
CUDA_UNITS = [
    (CSRC / "trace_kernels.cu", ["-fmad=false"]),
    (CSRC / "capi.cu", []),
    (CSRC / "guide.cu", []),
    (CSRC / "kdtree_gpu.cu", []),
]
HOST_UNITS = [
    CSRC / "host" / "scenes.cpp",
    CSRC / "host" / "kdtree_build.cpp",
    CSRC / "host" / "p3.cpp",
    CSRC / "host" / "tree_file.cpp",
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run_all(cmds: list[list[str]]) -> None:
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((c, out.decode(errors="replace")))
    if failed:
        msg = "\n\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError(f"build failed:\n{msg}")


def build_native(verbose: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    LIB.mkdir(exist_ok=True)
    objs, cmds = [], []
    for src, extra in CUDA_UNITS:
        obj = BUILD / (src.stem + ".o")
        cmds.append([nvcc, *ARCH, *NVCC_COMMON, *extra, "-c", str(src), "-o", str(obj)])
        objs.append(obj)
    for src in HOST_UNITS:
        obj = BUILD / (src.stem + ".host.o")
        cmds.append(["g++", *GXX_COMMON, "-c", str(src), "-o", str(obj)])
        objs.append(obj)
    oracle_cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                  "-o", str(ORACLE / "liboracle.so"), str(ORACLE / "oracle.cpp"), "-lpthread"]
    cmds.append(oracle_cmd)
    # the CPU reference arm's input (synthetic scene + the reference's tree)
    # without the product library and its kernels
    cmds.append(["g++", *GXX_COMMON, "-shared", "-o", str(ORACLE / "libinputs.so"),
                 str(CSRC / "host" / "scenes.cpp"), str(CSRC / "host" / "kdtree_build.cpp"), "-lpthread"])
    if verbose:
        for c in cmds:
            print(" ".join(c))
    _run_all(cmds)
    so = LIB / "libturner_gb300.so"
    _run_all([[nvcc, *ARCH, "-shared", "-o", str(so), *map(str, objs), "-lpthread"]])
    cli = LIB / "turner_pathtracer"
    _run_all([["g++", *GXX_COMMON, "-o", str(cli), str(CSRC / "host" / "cli.cpp"), f"-L{LIB}",
               "-lturner_gb300", f"-Wl,-rpath,{LIB}", "-lpthread"]])
    return so


def reference_root() -> Path:
    """The reference's source tree: $TURNER_REFERENCE, else a checkout named
    `reference` beside this repository (absent on machines without it)."""
    env = os.environ.get("TURNER_REFERENCE")
    return Path(env) if env else ROOT.parent / "reference"


def build_reference_checker() -> None:
    """oracle/_ref from the reference's own sources, only where they exist."""
    ref = reference_root()
    if (ref / "lib" / "kdtree.cpp").exists():
        subprocess.run(["bash", str(ORACLE / "build_ref.sh"), str(ref)], check=True,
                       stdout=subprocess.DEVNULL)


def build(verbose: bool = False) -> None:
    build_native(verbose)
    build_reference_checker()


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
