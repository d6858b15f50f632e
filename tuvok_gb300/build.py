"""Build recipe for the native parts of tuvok_gb300.

* ``tuvok_gb300/libtvk.so``  -- the product: C ABI (include/tvk.h) over the
  sm_103a CUDA kernels, built with nvcc for ``-gencode arch=compute_103a,code=sm_103a``.
* ``oracle/liboracle.so``    -- the CPU oracle used by the tests and the CPU
  baseline (g++, OpenMP).

Objects go to ``_build/`` and are rebuilt when a source or header is newer.
Everything compiles in parallel; a cold build takes well under a minute.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "tuvok_gb300"
CSRC = PKG / "csrc"
BUILD = ROOT / "_build"
LIB = PKG / "libtvk.so"
ORACLE_LIB = ROOT / "oracle" / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = "-fPIC,-ffp-contract=off,-O3,-Wall"
# per-file extra flags: the ray march and the volume generator keep every
# multiply and add separate unless the source writes fmaf, so they match their
# host restatements bit for bit
EXTRA = {"raycast.cu": ["-fmad=false"], "volgen.cu": ["-fmad=false"]}
SOURCES = ["api.cpp", "bricking.cu", "cnn.cu", "codecs.cpp", "eo.cpp", "lod.cu", "raycast.cu",
           "rebrick.cu", "tf1d.cpp", "uvf.cpp", "volgen.cu"]
HEADERS = [CSRC / "tvk_internal.h", ROOT / "include" / "tvk.h"]
ORACLE_SOURCES = [ROOT / "oracle" / "bricking.cpp", ROOT / "oracle" / "raycast.cpp",
                  ROOT / "oracle" / "rebrick.cpp", ROOT / "oracle" / "volgen.cpp"]
ORACLE_HEADERS = [ROOT / "oracle" / "oracle.h"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build tuvok_gb300")
    return cand


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(str(c) for c in cmd), flush=True)
    r = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}):\n{' '.join(map(str, cmd))}\n"
                           f"{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)
    return r


def build_library(verbose: bool = False, ptxas_verbose: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    jobs = []
    objs = []
    for src in SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if not _stale(o, [s, *HEADERS]) and not ptxas_verbose:
            continue
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", HOST_FLAGS,
               *EXTRA.get(src, []), "-c", s, "-o", o]
        if ptxas_verbose and src.endswith(".cu"):
            cmd.insert(1, "-Xptxas=-v")
        jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for r in ex.map(lambda c: _run(c, verbose), jobs):
            if ptxas_verbose:
                print(r.stderr)
    if jobs or not LIB.exists():
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"], verbose)
    return LIB


def build_counting_library(verbose: bool = False) -> Path:
    """``_build/libtvk_counts.so``: the library with the ray march's event
    counters compiled in (TVK_PROFILE_COUNTS=1: leap iterations, steps leapt,
    candidate-brick slab tests, brick marches).  A diagnostic build; its atomics
    slow the march, so it is never the one timed."""
    build_library(verbose)
    nvcc = _nvcc()
    src = CSRC / "raycast.cu"
    o = BUILD / "raycast_counts.cu.o"
    out = BUILD / "libtvk_counts.so"
    if _stale(o, [src, *HEADERS]):
        _run([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", HOST_FLAGS,
              *EXTRA["raycast.cu"], "-DTVK_PROFILE_COUNTS=1", "-c", src, "-o", o], verbose)
    objs = [o if s == "raycast.cu" else BUILD / (s + ".o") for s in SOURCES]
    if _stale(out, objs):
        _run([nvcc, *ARCH, "-shared", "-o", out, *objs, "-lcudart"], verbose)
    return out


def build_oracle(verbose: bool = False) -> Path:
    if _stale(ORACLE_LIB, [*ORACLE_SOURCES, *ORACLE_HEADERS]):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared",
              "-o", ORACLE_LIB, *ORACLE_SOURCES], verbose)
    return ORACLE_LIB


def build_reference(verbose: bool = False, ref: Path | None = None) -> Path | None:
    """Builds oracle/_ref (the reference's own converter) when its sources exist.

    ref: the reference source tree (passed to the Makefile as REF); None keeps
    the Makefile's default."""
    mk = ROOT / "oracle" / "ref" / "Makefile"
    if not mk.exists():
        return None
    cmd = ["make", "-s", "-C", str(mk.parent), f"-j{os.cpu_count() or 4}"]
    if ref is not None:
        cmd.append(f"REF={ref}")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if verbose:
        print(r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")
    out = ROOT / "oracle" / "_ref" / "libtuvok_ref.so"
    return out if out.exists() else None


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        fl = ex.submit(build_library, verbose)
        fo = ex.submit(build_oracle, verbose)
        fl.result()
        fo.result()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    if "--ptxas" in sys.argv:
        build_library(verbose=True, ptxas_verbose=True)
    if "--ref" in sys.argv:
        print(build_reference(verbose=True))
