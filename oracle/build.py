"""Build recipe for the CPU oracle (test infrastructure, not product code).

Compiles ``oracle/gfref.cpp`` twice into ``oracle/_build/``:

* ``libgfref.so``      serial, -O3 -ffp-contract=off (the reference as shipped:
                       its OpenMP pragmas are inert because no build passes -fopenmp);
* ``libgfref_omp.so``  the same source with -fopenmp (element loops parallel,
                       assembly loops serial, as the reference's pragmas are placed).

``-ffp-contract=off`` keeps x86_64 and aarch64 bit-identical (GCC contracts to FMA
by default on aarch64).

The reference itself (GooseFEM, header-only C++) is not compiled: it needs xtensor
and, for Matrix*.h, Eigen, neither of which is available, so there is no
``oracle/_ref`` build.
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "gfref.cpp")

FLAGS = ["-O3", "-ffp-contract=off", "-fno-fast-math", "-std=c++17", "-shared", "-fPIC"]


def targets():
    return {
        "libgfref.so": FLAGS,
        "libgfref_omp.so": FLAGS + ["-fopenmp"],
    }


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    procs = []
    for name, flags in targets().items():
        dst = os.path.join(OUT, name)
        if not force and os.path.exists(dst) and os.path.getmtime(dst) >= os.path.getmtime(SRC):
            continue
        cmd = ["g++"] + flags + [SRC, "-o", dst]
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd)))
    for cmd, p in procs:
        if p.wait() != 0:
            raise RuntimeError("oracle build failed: " + " ".join(cmd))


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
