"""Build the engine library in place: ``python -m medimage_gb300.build``.

Compiles medimage_gb300/csrc/*.cu for sm_103a with nvcc (parallel make) into
medimage_gb300/libat_engine.so.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def build_engine(jobs: int | None = None) -> str:
    jobs = jobs or max(2, min(8, os.cpu_count() or 2))
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "csrc"), f"-j{jobs}"], check=True)
    path = os.path.join(HERE, "libat_engine.so")
    if not os.path.exists(path):
        raise RuntimeError("engine build produced no libat_engine.so")
    return path


if __name__ == "__main__":
    print(build_engine(int(sys.argv[1]) if len(sys.argv) > 1 else None))
