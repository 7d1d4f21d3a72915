"""Build recipe for the CPU oracle (test infrastructure only).

Compiles the plain-C restatement in this folder into ``oracle/liboracle.so``.
``-ffp-contract=off`` keeps every multiply and add separately rounded on every
host (gcc fuses them by default on aarch64), matching the reference's x86-64
build, which has no FMA.

The reference itself (C++ on Cantera 3.2, SUNDIALS, Eigen, Boost and TBB) does
not build here: none of those libraries is installed, so there is no
``oracle/_ref`` recipe.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["oracle_tridiag.c", "oracle_chem.c", "oracle_bdf.c", "oracle_testode.c", "oracle_transport.c",
           "oracle_convection.c", "oracle_qss_adjoint.c"]
TARGET = os.path.join(HERE, "liboracle.so")


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, s) for s in SOURCES if os.path.exists(os.path.join(HERE, s))]
    deps = srcs + [os.path.join(HERE, "oracle.h")]
    if not force and os.path.exists(TARGET):
        t = os.path.getmtime(TARGET)
        if all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d)):
            return TARGET
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-pthread", "-o", TARGET + ".tmp"] + srcs + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(TARGET + ".tmp", TARGET)
    return TARGET


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
