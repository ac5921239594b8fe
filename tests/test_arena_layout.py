"""The layout of a context's device arrays inside its one allocation
(reda_erplacer_gb300/csrc/arena.h), compiled for the host: for random sequences
of arrays (element sizes 1 to 48 bytes, counts from 0 to a million), every array
starts at a 256-byte boundary of the allocation, holds at least one element and
its count, follows the previous one without overlap, and ends inside the bytes
the plan asks for."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = r'''
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>
#include "arena.h"
using namespace erp;

struct E1 { char v; };
struct E8 { double v; };
struct E12 { float v[3]; };
struct E48 { double v[6]; };

int main() {
    std::mt19937_64 rng(11);
    long long bad = 0, checked = 0;
    for (int trial = 0; trial < 2000; ++trial) {
        const int n = 1 + (int)(rng() % 60);
        std::vector<void *> ptrs(n, nullptr);
        std::vector<size_t> need(n);
        ArenaPlan ap;
        for (int i = 0; i < n; ++i) {
            const size_t count = (rng() % 4 == 0) ? 0 : (size_t)(rng() % (trial % 5 ? 5000 : 1000000));
            const size_t eff = count ? count : 1;
            switch (rng() % 4) {
            case 0: ap.add(reinterpret_cast<E1 **>(&ptrs[i]), count); need[i] = eff * sizeof(E1); break;
            case 1: ap.add(reinterpret_cast<E8 **>(&ptrs[i]), count); need[i] = eff * sizeof(E8); break;
            case 2: ap.add(reinterpret_cast<E12 **>(&ptrs[i]), count); need[i] = eff * sizeof(E12); break;
            default: ap.add(reinterpret_cast<E48 **>(&ptrs[i]), count); need[i] = eff * sizeof(E48); break;
            }
        }
        char *base = reinterpret_cast<char *>(uintptr_t(1) << 40);   // never dereferenced
        ap.place(base);
        const size_t bytes = ap.bytes();
        size_t prev_end = 0;
        for (int i = 0; i < n; ++i) {
            ++checked;
            const size_t off = (size_t)(static_cast<char *>(ptrs[i]) - base);
            if (off % kArenaAlign || off < prev_end || off + need[i] > bytes) ++bad;
            prev_end = off + need[i];
        }
        if (bytes == 0 || bytes % kArenaAlign) ++bad;
    }
    printf("%s %lld %lld\n", bad ? "FAIL" : "ok", checked, bad);
    return bad ? 1 : 0;
}
'''


def test_arena_layout(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "arena.cpp"
    src.write_text(SRC)
    exe = tmp_path / "arena"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "reda_erplacer_gb300", "csrc"), str(src),
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout
