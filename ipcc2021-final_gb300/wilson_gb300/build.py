"""Build recipe for libwilson_gb300.so (sm_103a) and the C++ compatibility layer.

Each CUDA translation unit is compiled by nvcc for sm_103a only, in parallel,
then linked into one shared library next to this file (in-tree, git-ignored).
No cmake: plain nvcc/g++ invocations, rebuilt only when a source is newer than
its object.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent          # .../ipcc2021-final_gb300/wilson_gb300
ROOT = PKG.parent                              # .../ipcc2021-final_gb300
CSRC = ROOT / "csrc"
COMPAT = ROOT / "compat"
REPO = ROOT.parent
INCLUDE = REPO / "include"
BUILD = REPO / "_build"
LIB = PKG / "libwilson_gb300.so"
COMPAT_LIB = PKG / "liblattice_gb300.so"
MAIN_BIN = PKG / "wilson_main"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp",
              "--expt-relaxed-constexpr", "-I" + str(INCLUDE)]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-I" + str(INCLUDE)]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, ptxas_info: bool = False) -> Path:
    """Compile every kernel for sm_103a and link libwilson_gb300.so; returns its path."""
    BUILD.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [INCLUDE / "wilson_gb300.h"]
    jobs = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp")):
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        if not _stale(obj, [src] + headers):
            continue
        if src.suffix == ".cu":
            cmd = [nvcc()] + ARCH + NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_info else []) + \
                  ["-c", str(src), "-o", str(obj)]
        else:
            cmd = ["g++"] + CXX_FLAGS + ["-c", str(src), "-o", str(obj)]
        jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for cmd, _ in zip(jobs, ex.map(_run, jobs)):
                if verbose:
                    print(" ".join(cmd))
    if jobs or not LIB.exists():
        _run([nvcc()] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] + ["-lgomp"])
    return LIB


def build_compat(verbose: bool = False) -> Path:
    """Build the C++ layer with the reference's API (lattice_fermion, DslashNew, CGinvert, ...)."""
    lib = build(verbose)
    srcs = sorted((COMPAT / "src").glob("*.cpp"))
    if not srcs:
        return lib
    deps = srcs + sorted((COMPAT / "include").glob("*.h")) + sorted((COMPAT / "src").glob("*.h")) + [lib]
    if _stale(COMPAT_LIB, deps):
        cmd = ["g++"] + CXX_FLAGS + ["-I" + str(COMPAT / "include"), "-shared", "-o", str(COMPAT_LIB)] + \
              [str(s) for s in srcs] + ["-L" + str(PKG), "-lwilson_gb300", "-Wl,-rpath,$ORIGIN"]
        _run(cmd)
    main_src = COMPAT / "wilson_main.cpp"
    if _stale(MAIN_BIN, [main_src, COMPAT_LIB]):
        _run(compat_program_cmd(main_src, MAIN_BIN))
    return COMPAT_LIB


def compat_program_cmd(src: Path, out: Path) -> list[str]:
    """g++ command that builds a program against the reference-API layer."""
    return ["g++", "-O2", "-std=c++17", "-I" + str(COMPAT / "include"), "-o", str(out), str(src),
            "-L" + str(PKG), "-llattice_gb300", "-lwilson_gb300", "-Wl,-rpath," + str(PKG)]


if __name__ == "__main__":
    print(build(verbose=True))
    print(build_compat(verbose=True))
