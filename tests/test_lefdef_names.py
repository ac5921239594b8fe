"""Internals of csrc/lefdef.cpp compiled for the host.

* The reader's name table (the open-addressing NameTable) against
  std::unordered_map: 200,000 names with shared prefixes and one-character
  differences, lookups of present and absent names, duplicate inserts that
  keep the first owner, owners that move (the table holds indices, not
  pointers), and growth from empty.
* The writers' micron formatting (um: an integer fast path for grids that
  divide 10^6) against snprintf("%.15g") itself."""
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


UM_SRC = r'''
#include "lefdef.cpp"
#include <random>

int main() {
    const int64_t dens[] = {1, 2, 4, 5, 8, 10, 16, 20, 25, 40, 50, 64, 100, 125, 200, 250, 400, 500, 1000,
                            2000, 2500, 4000, 5000, 8000, 10000, 20000, 40000, 50000, 100000, 200000,
                            500000, 1000000, 3, 7, 1024, 3000, 2000000};
    std::mt19937_64 rng(17);
    long bad = 0, n_checked = 0;
    auto check = [&](int64_t n, int64_t den) {
        char b[64];
        std::snprintf(b, sizeof b, "%.15g", (double)n / (double)den);
        const std::string got = um(n, den);
        ++n_checked;
        if (got != b) { if (bad < 10) std::printf("um(%lld, %lld) = %s, want %s\n", (long long)n, (long long)den, got.c_str(), b); ++bad; }
    };
    for (int64_t den : dens) {
        for (int64_t n = -30000; n <= 30000; ++n) check(n, den);               // dense near zero: 1e-4 boundary
        for (int k = 0; k < 200000; ++k) {
            const int64_t mag = (int64_t)(rng() % 15);
            int64_t p = 1;
            for (int j = 0; j < mag; ++j) p *= 10;
            const int64_t n = (int64_t)(rng() % (uint64_t)p) * ((rng() & 1) ? 1 : -1);
            check(n, den);
        }
        for (int64_t e = 1, j = 0; j < 15; ++j, e *= 10) {                      // around powers of ten
            for (int64_t d = -3; d <= 3; ++d) { check(e + d, den); check(-(e + d), den); }
        }
        check(99999999999999LL, den); check(-99999999999999LL, den);
        check(100000000000000LL, den); check(INT64_MAX / 2, den);
    }
    std::printf("%s %ld %ld\n", bad ? "FAIL" : "ok", bad, n_checked);
    return bad ? 1 : 0;
}
'''


def test_micron_formatting_matches_printf(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "um.cpp"
    src.write_text(UM_SRC)
    exe = tmp_path / "um"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(ROOT, "reda_erplacer_gb300", "csrc"), str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout[-1500:]
