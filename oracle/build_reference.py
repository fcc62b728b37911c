"""Build the mounted chromo reference in place under ``oracle/_ref/``.

Test infrastructure only.  The reference is Python + Cython
(``setup.py:14-31`` cythonises 8 modules with ``language="c++"``).  This
script copies ``chromo/`` out of the read-only mount into ``oracle/_ref/``
(git-ignored), applies the one change Cython 3 needs (``cpdef list
move_list`` in ``chromo/mc/moves.pxd:41-43`` is rejected by Cython 3, so the
declaration is dropped and the definition at ``chromo/mc/moves.pyx:345``
becomes a plain module global), cythonises the same 8 modules plus
``oracle/ref_shim.pyx`` and compiles them with g++.  The arithmetic of the
reference is untouched.  ``oracle/ref_stubs`` supplies pandas / numba /
matplotlib / pyximport stand-ins at import time.

Usage:  python oracle/build_reference.py [--src /path/to/reference]

The checkout is taken from ``--src``, else from the ``CHROMO_REFERENCE``
environment variable, else from the mount point of this build container
(``reference_source()``).
"""
import argparse
import os
import shutil
import subprocess
import sys
import sysconfig
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
MODULES = [
    "chromo/mc/move_funcs.pyx",
    "chromo/polymers.pyx",
    "chromo/fields.pyx",
    "chromo/binders.pyx",
    "chromo/util/bead_selection.pyx",
    "chromo/util/linalg.pyx",
    "chromo/mc/mc_sim.pyx",
    "chromo/mc/moves.pyx",
]


def _patch_moves(root: Path) -> None:
    pxd = root / "chromo/mc/moves.pxd"
    txt = pxd.read_text()
    start = txt.index("cpdef list move_list")
    end = txt.index("]", start) + 1
    pxd.write_text(txt[:start] + txt[end:])
    pyx = root / "chromo/mc/moves.pyx"
    txt = pyx.read_text()
    pyx.write_text(txt.replace("cpdef list move_list =", "move_list =", 1))


def _compile(cpp: Path, so: Path, inc: list) -> None:
    cmd = ["g++", "-O2", "-shared", "-fPIC", "-w", "-o", str(so), str(cpp)]
    cmd += [f"-I{p}" for p in inc]
    subprocess.check_call(cmd)


def build(src: Path) -> Path:
    import numpy as np
    from Cython.Build import cythonize
    if OUT.exists():
        shutil.rmtree(OUT)
    OUT.mkdir(parents=True)
    shutil.copytree(src / "chromo", OUT / "chromo",
                    ignore=shutil.ignore_patterns("*.c", "*.cpp", "*.so", "*.html"))
    _patch_moves(OUT)
    shutil.copy(HERE / "ref_shim.pyx", OUT / "ref_shim.pyx")
    cwd = os.getcwd()
    os.chdir(OUT)
    try:
        cythonize(MODULES + ["ref_shim.pyx"], language="c++", quiet=True,
                  compiler_directives={"cdivision": False, "language_level": 3},
                  nthreads=8)
    finally:
        os.chdir(cwd)
    inc = [sysconfig.get_paths()["include"], np.get_include(), str(OUT)]
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    jobs = []
    for mod in MODULES + ["ref_shim.pyx"]:
        cpp = OUT / mod.replace(".pyx", ".cpp")
        so = OUT / mod.replace(".pyx", ext)
        jobs.append(subprocess.Popen(
            ["g++", "-O2", "-shared", "-fPIC", "-w", "-o", str(so), str(cpp)]
            + [f"-I{p}" for p in inc]))
    if any(j.wait() != 0 for j in jobs):
        raise RuntimeError("reference build failed")
    return OUT


def reference_source():
    """The reference checkout to build from: $CHROMO_REFERENCE, else the
    container's read-only mount; None when neither holds chromo/."""
    for cand in (os.environ.get("CHROMO_REFERENCE"), "/root/reference"):
        if cand and (Path(cand) / "chromo").is_dir():
            return Path(cand)
    return None


def sys_path_entries() -> list:
    """Paths to prepend to ``sys.path`` to import the built reference."""
    return [str(HERE / "ref_stubs"), str(OUT)]


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=None)
    a = ap.parse_args()
    src = Path(a.src) if a.src else reference_source()
    if src is None:
        sys.exit("no reference checkout: pass --src or set CHROMO_REFERENCE")
    print(build(src))
