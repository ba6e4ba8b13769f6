"""Build the oracle's C pieces (test infrastructure).

* ``oracle/csrc/*.c`` -> ``oracle/_build/liboracle.so`` (restatements, built anywhere);
* when the reference checkout is present, ``oracle/ref_trace`` compiles the
  reference's own rng.h / adaptive_trace_estimator.cpp into
  ``oracle/_ref/libref_trace.so`` (used to pin the restatement).

The checkout is the directory named by the environment variable
CBX_REFERENCE_SRC, else the read-only mount this recipe was written for.
"""
from __future__ import annotations

import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_trace.so")
REFERENCE = os.environ.get("CBX_REFERENCE_SRC", "/root/reference")


def build() -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(HERE, "csrc", "*.c")))
    # no contraction into FMA: the restatements keep the reference's written operation order
    # on every architecture
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-o", LIB, *srcs], check=True)
    if os.path.isdir(os.path.join(REFERENCE, "src", "core")):
        subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref_trace"), f"REF={REFERENCE}"],
                       check=True)
    return LIB


if __name__ == "__main__":
    print(build())
