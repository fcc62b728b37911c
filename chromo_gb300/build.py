"""Compile the CUDA library in place (sm_103a only).

``python -m chromo_gb300.build`` writes ``chromo_gb300/_lib/libchromo_gb300.so``.
The translation units are compiled in parallel and linked with nvcc.
Device code is built with ``-fmad=false`` so that every floating-point
operation is individually rounded, as in the CPU restatement used to check it.
"""
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
LIB = OUT / "libchromo_gb300.so"
SOURCES = ["cg_mc.cu", "cg_spec.cu", "cg_spec_f8.cu", "cg_spec_f16.cu", "cg_spec_f32.cu", "cg_spec_d32.cu",
           "cg_capi.cu", "cg_static.cu", "cg_grad.cu", "cg_guard.cu", "cg_steric.cu", "cg_hostio.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
         f"-I{PKG.parent / 'include'}"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [PKG.parent / "include" / "chromo_gb300.h"]
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not stale():
        return LIB
    OUT.mkdir(exist_ok=True)
    nv = nvcc()
    objs, procs = [], []
    for src in SOURCES:
        obj = OUT / (Path(src).stem + ".o")
        objs.append(obj)
        cmd = [nv, *ARCH, *FLAGS, "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        procs.append(subprocess.Popen(cmd))
    if any(p.wait() != 0 for p in procs):
        raise RuntimeError("nvcc compilation failed")
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.check_call([nv, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
