"""Build ``liblsim.so`` (the sm_103a kernels + C ABI) in-tree with nvcc.

Translation units compile in parallel; the shared library is written next
to this file.  ``python -m larndsim_gb300.build`` rebuilds it.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR.parent / "csrc"
INCLUDE = PKG_DIR.parent.parent / "include"
LIB_PATH = PKG_DIR / "liblsim.so"
SOURCES = ("lsim_segments.cu", "lsim_accum.cu", "lsim_main.cu", "lsim_fee.cu", "lsim_lut.cu", "lsim_chop.cu", "lsim_records.cu", "lsim_tracks.cu", "lsim_fee_prob.cu", "lsim_losses.cu", "lsim_prob_loss.cu", "lsim_api.cu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblsim.so")
    return cand


def _compile(src: Path, obj: Path, log: Path) -> None:
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}",
           "-Xptxas", "-v", "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    log.write_text(res.stdout + res.stderr)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stderr[-4000:]}")


def build(verbose: bool = False) -> Path:
    out_dir = PKG_DIR.parent / "_build"
    out_dir.mkdir(exist_ok=True)
    srcs = [CSRC / s for s in SOURCES]
    objs = [out_dir / (s.stem + ".o") for s in srcs]
    logs = [out_dir / (s.stem + ".log") for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        list(ex.map(_compile, srcs, objs, logs))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr[-4000:]}")
    os.replace(tmp, LIB_PATH)
    if verbose:
        for log in logs:
            print(log.read_text())
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
