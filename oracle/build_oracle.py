"""Build recipe for the oracle (test infrastructure): oracle/_build/liberp_oracle.so
and oracle/_build/liberp_synth.so.

The oracle is a CPU restatement of the reference loop used only by tests/,
the smoke check and bench.py's CPU legs.  The reference itself is Rust and
cannot be built with the toolchains of this project (no cargo/rustc), so there
is no oracle/_ref build.

liberp_synth.so is the seeded synthetic netlist generator compiled on its own
from the package's generator source (reda_erplacer_gb300/csrc/synth.cpp, host
C++, no CUDA).  It lets bench.py's reference arm build the same input design
as the GPU arm without loading the product library.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liberp_oracle.so")
SYNTH_LIB = os.path.join(OUT_DIR, "liberp_synth.so")
SOURCES = ["erp_oracle.c"]
HEADERS = ["erp_oracle.h", "spectral_impl.h"]
SYNTH_SOURCE = os.path.join(ROOT, "reda_erplacer_gb300", "csrc", "synth.cpp")
SYNTH_HEADER = os.path.join(ROOT, "include", "erplacer.h")


def _stale(lib, deps):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(f) > t for f in deps)


def build_synth(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and not _stale(SYNTH_LIB, [SYNTH_SOURCE, SYNTH_HEADER]):
        return SYNTH_LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), SYNTH_SOURCE, "-o", SYNTH_LIB + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(SYNTH_LIB + ".tmp", SYNTH_LIB)
    return SYNTH_LIB


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    build_synth(force)
    if not force and not _stale(LIB, [os.path.join(HERE, f) for f in SOURCES + HEADERS]):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-Wall", "-Wno-unused-function", "-Wno-maybe-uninitialized",
           "-o", LIB + ".tmp"] + [os.path.join(HERE, s) for s in SOURCES] + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
