"""Compile the sm_103a transport library in-tree.

Produces ``monki/_native/libmonki_cuda.so`` from ``csrc/*.cu`` with nvcc, one
``-gencode`` for GB300 (compute_103a / sm_103a), translation units compiled in
parallel. Nothing here runs at import time; ``monki.execution.native`` only loads the
library and fails loudly when it is missing.
"""

from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE_ROOT = Path(__file__).resolve().parent
SOURCES = PACKAGE_ROOT / "csrc"
OUTPUT = PACKAGE_ROOT / "monki" / "_native" / "libmonki_cuda.so"
UNITS = ("session.cu", "tail.cu", "multi.cu", "probes.cu", "mlp.cu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
# The transport units: the FP32 product path with fast single-precision math — division and
# square root to within 2 ulp, FP32 subnormals flushed to zero, and the hardware
# approximations of exp, log, sin and cos — checked statistically against the oracle and
# for its bias against the FP64 build (double-precision arithmetic is unchanged by these
# options). Division and square root alone gave +10 % on the box and layered clouds; the
# transcendental approximations a further +8 % on the box cloud (2.55 -> 2.75 G scatters/s
# through CUDA(), three repeats each): the peel-off and scattering kernels are issue bound.
# The device probes (probes.cu) keep full-precision math: they check the helpers' algorithm.
TRANSPORT_FLAGS = ["-use_fast_math"]
UNIT_FLAGS = {"session.cu": TRANSPORT_FLAGS, "tail.cu": TRANSPORT_FLAGS, "multi.cu": TRANSPORT_FLAGS}


def nvcc() -> str:
    candidates = [shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]

    for candidate in candidates:
        if candidate and Path(candidate).is_file():
            return candidate

    raise FileNotFoundError("nvcc is required to build the CUDA transport library")


def _digest() -> str:
    hasher = hashlib.sha256()

    for path in sorted(SOURCES.iterdir()):
        if path.suffix in {".cu", ".cuh", ".h"}:
            hasher.update(path.name.encode())
            hasher.update(path.read_bytes())

    hasher.update(" ".join(ARCH + FLAGS + sorted(f"{u}:{' '.join(f)}" for u, f in UNIT_FLAGS.items())).encode())
    return hasher.hexdigest()


def build(force: bool = False, verbose: bool = False) -> Path:
    """Build the library unless an identical build (same sources and flags) exists."""

    stamp = OUTPUT.with_suffix(".sha256")
    digest = _digest()

    if not force and OUTPUT.is_file() and stamp.is_file() and stamp.read_text() == digest:
        return OUTPUT

    OUTPUT.parent.mkdir(parents=True, exist_ok=True)
    work = PACKAGE_ROOT / "_build"
    work.mkdir(exist_ok=True)
    compiler = nvcc()

    def compile_unit(name: str) -> Path:
        obj = work / (Path(name).stem + ".o")
        command = [compiler, *ARCH, *FLAGS, *UNIT_FLAGS.get(name, []), "-c", str(SOURCES / name), "-o", str(obj)]

        if verbose:
            print(" ".join(command), file=sys.stderr)

        result = subprocess.run(command, capture_output=True, text=True)

        if result.returncode:
            raise RuntimeError(f"nvcc failed for {name}:\n{result.stderr[-4000:]}")

        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as pool:
        objects = list(pool.map(compile_unit, UNITS))

    temporary = OUTPUT.with_suffix(f".tmp{os.getpid()}.so")
    link = [compiler, *ARCH, "-shared", *map(str, objects), "-o", str(temporary)]
    result = subprocess.run(link, capture_output=True, text=True)

    if result.returncode:
        raise RuntimeError(f"nvcc link failed:\n{result.stderr[-4000:]}")

    temporary.replace(OUTPUT)
    stamp.write_text(digest)
    return OUTPUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
