"""Build recipe for the CPU oracle (test infrastructure, not product code).

Compiles ``monki_oracle.cpp`` (the FP64 restatement of the reference Fortran transport)
into ``oracle/build/libmonki_oracle.so`` with OpenMP. Only tests, the smoke check and the
benchmark's CPU-baseline legs load it.
"""

from __future__ import annotations

import hashlib
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent
SOURCE = ROOT / "monki_oracle.cpp"
OUTPUT = ROOT / "build" / "libmonki_oracle.so"
# No FMA contraction, so x86 and Arm hosts round the restatement identically.
FLAGS = ["-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off"]


def build(force: bool = False) -> Path:
    digest = hashlib.sha256(SOURCE.read_bytes() + " ".join(FLAGS).encode()).hexdigest()
    stamp = OUTPUT.with_suffix(".sha256")

    if not force and OUTPUT.is_file() and stamp.is_file() and stamp.read_text() == digest:
        return OUTPUT

    OUTPUT.parent.mkdir(parents=True, exist_ok=True)
    temporary = OUTPUT.with_suffix(f".tmp{os.getpid()}.so")
    result = subprocess.run(
        ["g++", *FLAGS, str(SOURCE), "-o", str(temporary)], capture_output=True, text=True
    )

    if result.returncode:
        raise RuntimeError(f"oracle build failed:\n{result.stderr[-4000:]}")

    temporary.replace(OUTPUT)
    stamp.write_text(digest)
    return OUTPUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
