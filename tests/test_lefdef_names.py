"""The LEF/DEF reader's name table (the open-addressing NameTable of
csrc/lefdef.cpp, compiled for the host), against std::unordered_map: 200,000
names with shared prefixes and one-character differences, lookups of present
and absent names, duplicate inserts that keep the first owner, owners that
move (the table holds indices, not pointers), and growth from empty."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = r'''
#include "lefdef.cpp"
#include <random>

int main() {
    std::vector<std::string> owners;
    NameTable t;
    std::unordered_map<std::string, int> ref;
    auto name_of = [&](int i) -> std::string_view { return owners[i]; };
    std::mt19937_64 rng(3);
    long bad = 0;
    for (int i = 0; i < 200000; ++i) {
        std::string n;
        switch (i % 4) {
            case 0: n = "inst" + std::to_string(i); break;                        // shared prefix
            case 1: n = "u_core/u_alu/reg_" + std::to_string(i / 4) + "_"; break;  // long, hierarchical
            case 2: n = std::string(1 + rng() % 24, 'a' + (char)(rng() % 26)); break;  // repeats likely
            default: n = "x" + std::to_string(rng() % 50000); break;              // duplicates likely
        }
        const int owner = (int)owners.size();
        const bool fresh = ref.emplace(n, owner).second;
        if (t.insert(n, owner, name_of) != fresh) ++bad;
        owners.push_back(n);   // reallocates: the table must not hold pointers
    }
    for (const auto &kv : ref)
        if (t.find(kv.first, name_of) != kv.second) ++bad;   // the first owner of each name
    for (int i = 0; i < 100000; ++i) {
        const std::string q = "absent" + std::to_string(i) + "/" + std::to_string(rng());
        if (t.find(q, name_of) != -1) ++bad;
    }
    NameTable empty;
    if (empty.find("x", name_of) != -1 || !empty.empty()) ++bad;
    std::printf("%s %ld %zu\n", bad ? "FAIL" : "ok", bad, ref.size());
    return bad ? 1 : 0;
}
'''


def test_name_table_matches_unordered_map(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "names.cpp"
    src.write_text(SRC)
    exe = tmp_path / "names"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(ROOT, "reda_erplacer_gb300", "csrc"), str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout[-1000:]
