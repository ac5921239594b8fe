"""The block-to-instance mapping of the batches' packed launches
(reda_erplacer_gb300/csrc/packed.h), compiled for the host: for random block
counts per instance (one instance to thousands, one block to hundreds each),
every block of the grid finds the instance whose range holds it, and its block
index within that instance runs from 0 to the instance's own grid size."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = r'''
#include <cstdio>
#include <random>
#include <vector>
#include "packed.h"
using namespace erp;

int main() {
    std::mt19937 rng(5);
    long long bad = 0, checked = 0;
    for (int trial = 0; trial < 400; ++trial) {
        const int n = 1 + (int)(rng() % (trial < 200 ? 8 : 3000));
        std::vector<int32_t> b0(1, 0);
        for (int i = 0; i < n; ++i) b0.push_back(b0.back() + 1 + (int)(rng() % (trial % 3 ? 4 : 300)));
        std::vector<int> seen(n, 0);
        for (int b = 0; b < b0[n]; ++b) {
            const int i = packed_instance(b0.data(), n, b);
            ++checked;
            if (i < 0 || i >= n || !(b0[i] <= b && b < b0[i + 1]) || b - b0[i] != seen[i]) ++bad;
            else ++seen[i];
        }
        for (int i = 0; i < n; ++i)
            if (seen[i] != b0[i + 1] - b0[i]) ++bad;
    }
    printf("%s %lld %lld\n", bad ? "FAIL" : "ok", checked, bad);
    return bad ? 1 : 0;
}
'''


def test_packed_block_to_instance_map(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "pk.cpp"
    src.write_text(SRC)
    exe = tmp_path / "pk"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "reda_erplacer_gb300", "csrc"), str(src),
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout
