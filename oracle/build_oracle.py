"""Build recipe of the test oracle (CPU). Test infrastructure only.

  oracle/liboracle.so            CPU FP64 restatement of the reference LM (lm_oracle.cpp) and the
                                 seeded workload generator (synthetic_oracle.cpp), g++
  oracle/_ref/libgba_ref_reader.so
                                 the reference's own src/bal_reader.cpp compiled from its
                                 source where it lies, plus ref_shim.cpp (extern "C" wrappers)
  oracle/_ref/libgba_ref_lm_host.so
                                 the reference's own LM driver: src/lm.cu compiled UNMODIFIED
                                 by nvcc (sm_103a device code, host code for this CPU) against
                                 eigen_shim/ (the <Eigen/Dense> subset it uses), with
                                 src/bal_reader.cpp, ref_lm_shim.cpp (extern "C" entry) and
                                 ref_host_runtime.cpp, a CPU stand-in for the CUDA runtime that
                                 runs the driver's three kernels as CPU restatements. It runs
                                 the reference's host LM logic on a machine without a GPU.
  oracle/_ref/ref_test_launch_bounds
                                 the reference's own tests/test_launch_bounds.cpp, unmodified,
                                 linked against the same objects

The reference checkout is read from GBA_REFERENCE_DIR, else from the sibling
directory `reference/` next to the repository root. The _ref outputs are only
built where that checkout exists; they stay in oracle/_ref/ (git-ignored) and
are never part of the product.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"
REF_SO = REF_DIR / "libgba_ref_reader.so"
REF_LM_SO = REF_DIR / "libgba_ref_lm_host.so"
REF_LB_EXE = REF_DIR / "ref_test_launch_bounds"
EIGEN_SHIM = HERE / "eigen_shim"
REFERENCE = Path(os.environ.get("GBA_REFERENCE_DIR", str(HERE.parent.parent / "reference")))

FLAGS = ["-std=c++17", "-O3", "-ffp-contract=off", "-fPIC", "-shared"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr}")


def _stale(out: Path, inputs) -> bool:
    return not out.exists() or out.stat().st_mtime < max(p.stat().st_mtime for p in inputs)


def build_oracle() -> Path:
    srcs = [HERE / "lm_oracle.cpp", HERE / "synthetic_oracle.cpp"]
    if _stale(ORACLE_SO, srcs):
        tmp = ORACLE_SO.with_suffix(".so.tmp")
        _run(["g++", *FLAGS, "-o", str(tmp), *map(str, srcs), "-lpthread"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_reference_reader() -> Path | None:
    ref_src = REFERENCE / "src" / "bal_reader.cpp"
    if not ref_src.exists():
        return REF_SO if REF_SO.exists() else None
    shim = HERE / "ref_shim.cpp"
    REF_DIR.mkdir(exist_ok=True)
    if _stale(REF_SO, [ref_src, shim]):
        tmp = REF_SO.with_suffix(".so.tmp")
        _run(["g++", *FLAGS, f"-I{REFERENCE / 'include'}", "-o", str(tmp), str(ref_src), str(shim)])
        os.replace(tmp, REF_SO)
    return REF_SO


def _cuda_include() -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return str(Path(nvcc).resolve().parent.parent / "include")


def build_reference_lm() -> Path | None:
    """The reference's LM driver (src/lm.cu, unmodified) for the CPU, see the module docstring."""
    lm_src = REFERENCE / "src" / "lm.cu"
    reader_src = REFERENCE / "src" / "bal_reader.cpp"
    lb_src = REFERENCE / "tests" / "test_launch_bounds.cpp"
    if not lm_src.exists():
        return REF_LM_SO if REF_LM_SO.exists() else None
    REF_DIR.mkdir(exist_ok=True)
    inc = REFERENCE / "include"
    shim_hdr = EIGEN_SHIM / "Eigen" / "Dense"
    runtime, entry = HERE / "ref_host_runtime.cpp", HERE / "ref_lm_shim.cpp"
    headers = [inc / "gba" / "lm.hpp", inc / "gba" / "bal_problem.hpp", inc / "gba" / "schur.cuh", shim_hdr]
    objs = {
        REF_DIR / "lm.o": (["nvcc", "-std=c++17", "-O3", "-DNDEBUG", "-gencode", "arch=compute_103a,code=sm_103a",
                            "-Xcompiler", "-fPIC", f"-I{EIGEN_SHIM}", f"-I{inc}", "-c", str(lm_src)],
                           [lm_src, *headers]),
        REF_DIR / "bal_reader.o": (["g++", "-std=c++17", "-O3", "-DNDEBUG", "-fPIC", f"-I{inc}", "-c",
                                    str(reader_src)], [reader_src, *headers]),
        REF_DIR / "ref_lm_shim.o": (["g++", "-std=c++17", "-O3", "-fPIC", f"-I{inc}", "-c", str(entry)],
                                    [entry, *headers]),
        REF_DIR / "ref_host_runtime.o": (["g++", "-std=c++17", "-O3", "-fPIC", f"-I{_cuda_include()}", "-c",
                                          str(runtime)], [runtime]),
    }
    jobs = [(cmd + ["-o", str(out)]) for out, (cmd, deps) in objs.items() if _stale(out, deps)]
    with ThreadPoolExecutor(max_workers=4) as ex:
        list(ex.map(_run, jobs))
    o = [str(p) for p in objs]
    if _stale(REF_LM_SO, list(objs)):
        tmp = REF_LM_SO.with_suffix(".so.tmp")
        # -Bsymbolic: the library's references bind to its own CUDA-runtime stand-in even
        # in a process that has already loaded the real CUDA runtime
        _run(["g++", "-shared", "-Wl,-Bsymbolic", "-o", str(tmp), *o, "-lpthread"])
        os.replace(tmp, REF_LM_SO)
    if lb_src.exists():
        lb_obj = REF_DIR / "test_launch_bounds.o"
        if _stale(lb_obj, [lb_src, *headers]):
            _run(["g++", "-std=c++17", "-O3", "-DNDEBUG", f"-I{inc}", "-c", str(lb_src), "-o", str(lb_obj)])
        if _stale(REF_LB_EXE, [lb_obj, *objs]):
            _run(["g++", "-o", str(REF_LB_EXE), str(lb_obj), *o, "-lpthread"])
    return REF_LM_SO


if __name__ == "__main__":
    print(build_oracle())
    print(build_reference_reader())
    print(build_reference_lm())
    sys.exit(0)
