"""Build recipe of libgba_gb300.so and the bench_bal CLI (nvcc, sm_103a only).

Every translation unit is compiled in parallel with
`nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo`; objects are
rebuilt when a source or any header under csrc/ or include/ is newer. Host code
is compiled with -ffp-contract=off so x86 and Arm hosts round identically.

Usage: python build.py [--clean] [--verbose]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "lib" / "libgba_gb300.so"
BENCH = PKG / "bin" / "bench_bal"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_SOURCES = [
    "structure.cu",
    "edge.cu",
    "blocks.cu",
    "dense.cu",
    "pcg.cu",
    "mlp.cu",
    "noalloc.cu",
    "lm.cpp",
    "capi.cpp",
    "bal_io.cpp",
    "synthetic.cpp",
]


def nvcc() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgba_gb300")


def _flags() -> list[str]:
    return [
        "-std=c++17",
        "-O3",
        "-lineinfo",
        *ARCH,
        "-Xcompiler",
        "-fPIC,-ffp-contract=off",
        f"-I{ROOT / 'include'}",
        f"-I{CSRC}",
    ]


def _newest_header() -> float:
    t = 0.0
    for d in (CSRC, ROOT / "include"):
        for p in d.rglob("*"):
            if p.suffix in (".h", ".hpp", ".cuh"):
                t = max(t, p.stat().st_mtime)
    return t


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compiles the library (and bench_bal) if out of date; returns the .so path."""
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB.parent.mkdir(parents=True, exist_ok=True)
    BENCH.parent.mkdir(parents=True, exist_ok=True)
    cc = nvcc()
    hdr = _newest_header()
    jobs = jobs or min(len(LIB_SOURCES), os.cpu_count() or 4)

    def obj_for(src: str) -> Path:
        return BUILD / (src + ".o")

    todo = []
    for src in LIB_SOURCES:
        s = CSRC / src
        o = obj_for(src)
        if not o.exists() or o.stat().st_mtime < max(s.stat().st_mtime, hdr):
            todo.append(src)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(_run, [cc, *_flags(), "-c", str(CSRC / s), "-o", str(obj_for(s))], verbose) for s in todo]
        for f in futs:
            f.result()
    objs = [obj_for(s) for s in LIB_SOURCES]
    newest_obj = max(o.stat().st_mtime for o in objs)
    if todo or not LIB.exists() or LIB.stat().st_mtime < newest_obj:
        tmp = LIB.with_suffix(".so.tmp")
        _run([cc, "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-lpthread"], verbose)
        os.replace(tmp, LIB)
    bsrc = CSRC / "bench_bal.cpp"
    if not BENCH.exists() or BENCH.stat().st_mtime < max(bsrc.stat().st_mtime, LIB.stat().st_mtime, hdr):
        _run(
            [
                cc,
                *_flags(),
                "-o",
                str(BENCH),
                str(bsrc),
                f"-L{LIB.parent}",
                "-lgba_gb300",
                "-Xlinker",
                "-rpath,$ORIGIN/../lib",
            ],
            verbose,
        )
    return LIB


def clean() -> None:
    for p in (BUILD, LIB.parent, BENCH.parent):
        if p.exists():
            shutil.rmtree(p)


if __name__ == "__main__":
    if "--clean" in sys.argv:
        clean()
    print(build(verbose="--verbose" in sys.argv))
