"""The integer-only FP32 <-> 64-bit fixed-point conversions of the density path
(reda_erplacer_gb300/csrc/fixedpoint.h), compiled for the host and checked
against the C library's round-to-nearest-even conversions: every float bit
pattern of the exponents where rounding happens, a stride through the rest,
and the tie / carry patterns of every 64-bit magnitude."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = r'''
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <random>
#include "fixedpoint.h"
using namespace erp;

static float from_bits(uint32_t b) { float v; memcpy(&v, &b, 4); return v; }

int main() {
    long long bad = 0, n = 0;
    // float -> u64: exponents 0..189 (v < 2^63); exhaustive where v < 2^24
    // (rounding happens) and around it, a stride elsewhere
    for (uint32_t e = 0; e < 190; ++e) {
        const uint32_t step = (e >= 118 && e <= 152) ? 1 : 61;
        for (uint32_t m = 0; m < (1u << 23); m += step) {
            const float v = from_bits((e << 23) | m);
            const uint64_t want = (uint64_t)llrintf(v);
            const uint64_t got = fxp_rint_u64(v);
            ++n;
            if (got != want) { if (bad < 5) printf("rint %a: %llu != %llu\n", v, (unsigned long long)got, (unsigned long long)want); ++bad; }
        }
    }
    // out of range: 0
    const float odd[] = {-0.0f, -1.0f, -3.5e9f, INFINITY, -INFINITY, NAN, 9.3e18f};
    for (float v : odd) if (fxp_rint_u64(v) != 0 && !(v == -0.0f)) { printf("odd %a\n", v); ++bad; }
    // u64 -> float: every magnitude, tie / carry patterns and random mantissas
    std::mt19937_64 rng(7);
    auto check = [&](uint64_t q) {
        const float want = (float)q, got = fxp_u64_to_float(q);
        ++n;
        if (memcmp(&want, &got, 4) != 0) { if (bad < 10) printf("u2f %llu: %a != %a\n", (unsigned long long)q, got, want); ++bad; }
    };
    check(0); check(1); check(~0ull); check(1ull << 63); check((1ull << 63) - 1);
    for (int e = 0; e < 64; ++e) {
        const uint64_t p = 1ull << e;
        for (int k = 0; k < 2000; ++k) {
            const uint64_t r = rng();
            const uint64_t q = p | (e ? (r & (p - 1)) : 0);
            check(q);
            if (e >= 24) {   // the kept 24 bits, then exact ties and neighbours
                const int cut = e - 23;
                const uint64_t kept = q & ~((1ull << cut) - 1), half = 1ull << (cut - 1);
                check(kept); check(kept | half); check((kept | half) - 1); check(kept | half | 1);
                check(kept | ((1ull << cut) - 1));
            }
        }
    }
    for (int k = 0; k < 4000000; ++k) check(rng() >> (rng() % 64));
    printf("%s %lld %lld\n", bad ? "FAIL" : "ok", n, bad);
    return bad ? 1 : 0;
}
'''


def test_fixedpoint_conversions_match_the_c_library(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "fxp.cpp"
    src.write_text(SRC)
    exe = tmp_path / "fxp"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "reda_erplacer_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout[-2000:]
