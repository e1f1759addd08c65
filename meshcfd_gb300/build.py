"""Compile the native library for sm_103a (in-tree, no build system needed).

``python -m meshcfd_gb300.build`` or :func:`build` writes
``meshcfd_gb300/_build/libmeshcfd_gb300.so``.  The kernel translation unit is
compiled with ``-fmad=false`` (reference operation order); host code with
``-ffp-contract=off`` (GCC on aarch64 would otherwise contract a*b+c).

Extra nvcc options may be given in the environment variable
``MESHCFD_GB300_NVCC_FLAGS`` (split on whitespace), for example
``-DMCFD_INT_MUL=3`` to choose which products of the exact-arithmetic
kernels run on the integer pipe (the default is per variant, see
mcfd_kernels_impl.cuh); a build with other options than the existing
library's is forced.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIBNAME = "libmeshcfd_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra flags)
UNITS = [
    ("mcfd_kernels_exact.cu", ["-fmad=false"]),
    ("mcfd_kernels_fast.cu", ["-fmad=false"]),
    ("mcfd_kernels_fma.cu", ["-fmad=true"]),
    ("mcfd_kernels_common.cu", ["-fmad=false"]),
    ("mcfd_implicit.cu", ["-fmad=false"]),
    ("mcfd_jvp.cu", ["-fmad=false"]),
    ("mcfd_vjp.cu", ["-fmad=true"]),
    ("mcfd_parabolic.cu", ["-fmad=false"]),
    ("mcfd_boundary.cu", ["-fmad=false"]),
    ("mcfd_viscous.cu", ["-fmad=false"]),
    ("mcfd_api.cu", []),
    ("mcfd_noalloc.cu", ["-fmad=false"]),
    ("mcfd_stencil.cu", []),
    ("mcfd_geometry.cu", ["-fmad=false"]),
]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(path).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build meshcfd_gb300")
    return path


def _sources_newer(target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    deps = list(CSRC.glob("*")) + [HERE.parent / "include" / "meshcfd_gb300.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    target = BUILD / LIBNAME
    extra_flags = os.environ.get("MESHCFD_GB300_NVCC_FLAGS", "").split()
    stamp = BUILD / "nvcc_flags.txt"
    flags_changed = (stamp.read_text() if stamp.exists() else "") != " ".join(extra_flags)
    if not force and not flags_changed and not _sources_newer(target):
        return target
    common = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v" if verbose else "-O3", *extra_flags]

    def compile_unit(unit):
        src, extra = unit
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [*common, *extra, "-c", str(CSRC / src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
        return obj, res.stderr

    with ThreadPoolExecutor(max_workers=len(UNITS)) as pool:
        results = list(pool.map(compile_unit, UNITS))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    tmp = BUILD / (LIBNAME + f".tmp{os.getpid()}")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *[str(o) for o, _ in results]]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, target)
    stamp.write_text(" ".join(extra_flags))
    return target


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
