"""Build the glass_gb300 CUDA library (sm_103a) in-tree.

``python -m glass_gb300.build`` compiles every ``csrc/*.cu`` translation
unit in parallel with nvcc (one ``-gencode`` for sm_103a) and links
``glass_gb300/_build/libglassgb300.so``.  No cmake, no torch extension
machinery: the library exports the plain C ABI of ``include/glass_gb300.h``.
"""

from __future__ import annotations

import concurrent.futures
import os
import pathlib
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
LIB = OUT / "libglassgb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-Xcompiler",
    "-fPIC",
    "--expt-relaxed-constexpr",
    "-Xptxas",
    "-warn-spills",
]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not pathlib.Path(cand).exists():
        raise RuntimeError("nvcc not found: the glass_gb300 CUDA library cannot be built")
    return cand


def _compile(src: pathlib.Path, extra: list[str]) -> pathlib.Path:
    obj = OUT / (src.stem + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, force: bool = False) -> pathlib.Path:
    """Compile and link the library; skip when it is newer than every source."""
    OUT.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu"))
    deps = srcs + sorted(CSRC.glob("*.cuh")) + [HERE.parent / "include" / "glass_gb300.h"]
    if not force and LIB.exists() and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    extra = ["-Xptxas", "-v"] if verbose else []
    workers = min(len(srcs), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(workers) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
