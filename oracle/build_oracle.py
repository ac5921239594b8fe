"""Build recipe for the oracle (test infrastructure): oracle/_build/liberp_oracle.so.

The oracle is a CPU restatement of the reference loop used only by tests/,
the smoke check and bench.py's CPU legs.  The reference itself is Rust and
cannot be built with the toolchains of this project (no cargo/rustc), so there
is no oracle/_ref build.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liberp_oracle.so")
SOURCES = ["erp_oracle.c"]
HEADERS = ["erp_oracle.h", "spectral_impl.h"]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(os.path.join(HERE, f)) > t for f in SOURCES + HEADERS)


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and not _stale():
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-Wall", "-Wno-unused-function", "-Wno-maybe-uninitialized",
           "-o", LIB + ".tmp"] + [os.path.join(HERE, s) for s in SOURCES] + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
