"""Build recipe of the test oracle (CPU, g++). Test infrastructure only.

  oracle/liboracle.so            CPU FP64 restatement of the reference LM (lm_oracle.cpp)
  oracle/_ref/libgba_ref_reader.so
                                 the reference's own src/bal_reader.cpp compiled from
                                 its source where it lies (reference checkout), plus
                                 ref_shim.cpp (extern "C" wrappers). Only built when
                                 the reference checkout is present; its outputs stay
                                 in oracle/_ref/ (git-ignored).

The reference's LM driver src/lm.cu includes <Eigen/Dense>; Eigen is not
installed, so that file is not buildable here and is not attempted.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"
REF_SO = REF_DIR / "libgba_ref_reader.so"
REFERENCE = Path(os.environ.get("GBA_REFERENCE_DIR", "/root/reference"))

FLAGS = ["-std=c++17", "-O3", "-ffp-contract=off", "-fPIC", "-shared"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr}")


def build_oracle() -> Path:
    src = HERE / "lm_oracle.cpp"
    if not ORACLE_SO.exists() or ORACLE_SO.stat().st_mtime < src.stat().st_mtime:
        tmp = ORACLE_SO.with_suffix(".so.tmp")
        _run(["g++", *FLAGS, "-o", str(tmp), str(src), "-lpthread"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_reference_reader() -> Path | None:
    ref_src = REFERENCE / "src" / "bal_reader.cpp"
    if not ref_src.exists():
        return REF_SO if REF_SO.exists() else None
    shim = HERE / "ref_shim.cpp"
    REF_DIR.mkdir(exist_ok=True)
    newest = max(ref_src.stat().st_mtime, shim.stat().st_mtime)
    if not REF_SO.exists() or REF_SO.stat().st_mtime < newest:
        tmp = REF_SO.with_suffix(".so.tmp")
        _run(["g++", *FLAGS, f"-I{REFERENCE / 'include'}", "-o", str(tmp), str(ref_src), str(shim)])
        os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle())
    print(build_reference_reader())
    sys.exit(0)
