"""The 32-bit bin range of the electric force (reda_erplacer_gb300/csrc/binrange.h),
compiled for the host, against the reference's rule evaluated in 64-bit
integers as the oracle does (`to_isize().unwrap_or(0)`, lower end raised to 0,
upper end + 1 with negative values wrapping, then cut to the bin count): the
visited bins are the same next to every integer of a band around the grids
(truncation changes only there), through a stride of all floats, and at the
special values."""
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
#include "binrange.h"
using namespace erp;

static long to_isize0(float v) {
    if (!(v == v) || v >= 9.2e18f || v <= -9.2e18f) return 0;
    return (long)v;
}
static long lo_ref(float v) { long l = to_isize0(v); return l < 0 ? 0 : l; }
static long hi_ref(float v, int nb) { long h = to_isize0(v) + 1; return (h < 0 || h > nb) ? nb : h; }

int main() {
    long long bad = 0, n = 0;
    const int nbs[] = {16, 64, 100, 512, 1024, 4096};
    auto check = [&](float v) {
        for (int nb : nbs) {
            ++n;
            const long lr = lo_ref(v), hr = hi_ref(v, nb);
            const int l = force_bin_lo(v, nb), h = force_bin_hi(v, nb);
            // the same visited range: equal upper ends; equal lower ends, or
            // both at or beyond the upper end (empty)
            const bool ok = h == hr && (l == lr || (l >= h && lr >= hr)) && l >= 0 && l <= nb;
            if (!ok) { if (bad < 5) printf("v=%a nb=%d: [%d,%d) vs [%ld,%ld)\n", v, nb, l, h, lr, hr); ++bad; }
        }
    };
    // truncation changes only at integers: 64 floats on each side of every
    // integer of a band around the grids, and the integers themselves
    for (int k = -8; k <= 4200; ++k) {
        float lo = (float)k, hi = (float)k;
        check((float)k);
        for (int j = 0; j < 64; ++j) {
            lo = nextafterf(lo, -INFINITY);
            hi = nextafterf(hi, INFINITY);
            check(lo);
            check(hi);
        }
        check((float)k + 0.5f);
    }
    for (uint32_t b = 0; b < 0xffffffffu - 4093; b += 4093) { float v; memcpy(&v, &b, 4); check(v); }
    const float sp[] = {NAN, -NAN, INFINITY, -INFINITY, 9.2e18f, -9.2e18f, nextafterf(9.2e18f, 0.0f),
                        nextafterf(-9.2e18f, 0.0f), 3e9f, -3e9f, 2147483648.0f, -2147483648.0f, -2.0f,
                        nextafterf(-2.0f, 0.0f), -1.0f, -0.0f, 0.0f, 1.0f};
    for (float v : sp) check(v);
    printf("%s %lld %lld\n", bad ? "FAIL" : "ok", n, bad);
    return bad ? 1 : 0;
}
'''


def test_force_bin_range_matches_the_64_bit_rule(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "br.cpp"
    src.write_text(SRC)
    exe = tmp_path / "br"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "reda_erplacer_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout[-2000:]
