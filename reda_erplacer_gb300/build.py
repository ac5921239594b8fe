"""Build recipe of liberplacer_gb300.so (in-tree, sm_103a only).

Each CUDA translation unit is compiled separately (in parallel) with
``-gencode arch=compute_103a,code=sm_103a``; k_place.cu additionally with
``-fmad=false`` so that its float expressions keep the reference's operation
order.  Host code is compiled with ``-ffp-contract=off`` so that x86 and Arm
hosts evaluate the set-up arithmetic identically.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liberplacer_gb300.so")
CLI = os.path.join(HERE, "erplacer_gb300")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")

CU_SOURCES = {
    "k_place.cu": ["-fmad=false"],
    "k_spectral.cu": [],
    "erp_api.cu": [],
    "erp_noalloc.cu": [],
    "k_snapshot.cu": [],
    "k_dctgemm.cu": [],
}
CPP_SOURCES = ["synth.cpp", "lefdef.cpp"]
CLI_SOURCE = "erplacer_cli.cpp"   # the command-line driver, linked against the library
HEADERS = ["erp_internal.cuh", "reduce.cuh", "bulk_copy.cuh", "dfloat.h", "fixedpoint.h", "binrange.h",
           "packed.h", "arena.h"]


def _deps():
    files = [os.path.join(CSRC, f) for f in list(CU_SOURCES) + CPP_SOURCES + [CLI_SOURCE] + HEADERS]
    files.append(os.path.join(INCLUDE, "erplacer.h"))
    files.append(os.path.abspath(__file__))
    return files


def _stale():
    if not os.path.exists(LIB) or not os.path.exists(CLI):
        return True
    t = min(os.path.getmtime(LIB), os.path.getmtime(CLI))
    return any(os.path.getmtime(f) > t for f in _deps())


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    common = ["-O3", "-std=c++17", "-lineinfo", "-I", INCLUDE, "-I", CSRC,
              "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]
    jobs = []
    objs = []
    for src, extra in CU_SOURCES.items():
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        cmd = [NVCC] + ARCH + common + extra + ["-Xptxas", "-v"] * bool(verbose) + \
              ["-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append(cmd)
    for src in CPP_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", INCLUDE,
                     "-c", os.path.join(CSRC, src), "-o", obj])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    _run([NVCC] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs)
    os.replace(LIB + ".tmp", LIB)
    _run(["g++", "-O2", "-std=c++17", "-I", INCLUDE, os.path.join(CSRC, CLI_SOURCE), "-o", CLI + ".tmp",
          "-L", HERE, "-l:" + os.path.basename(LIB), "-Wl,-rpath,$ORIGIN"])
    os.replace(CLI + ".tmp", CLI)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
