"""The double-float arithmetic of the step's reductions
(reda_erplacer_gb300/csrc/dfloat.h), compiled for the host: TwoSum is exact,
and a sum taken the way the kernels take it (short per-thread sequential
chains, then a pairwise tree) stays within a few units of 2^-44 of the exactly
rounded sum, where plain FP32 summation is off by orders of magnitude more."""
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SRC = r'''
#include <cstdio>
#include <cstdint>
#include <vector>
#include "dfloat.h"
using namespace erp;

int main(int argc, char **argv) {
    FILE *f = fopen(argv[1], "rb");
    int64_t n;
    if (fread(&n, 8, 1, f) != 1) return 2;
    std::vector<float> x(n);
    if (fread(x.data(), 4, n, f) != (size_t)n) return 2;
    fclose(f);
    // TwoSum exactness over consecutive pairs (their exponents differ by less
    // than 29, so both sides are exact in double)
    long long bad = 0;
    for (int64_t i = 0; i + 1 < n; ++i) {
        float s, e;
        two_sum(x[i], x[i + 1], s, e);
        if ((double)s + (double)e != (double)x[i] + (double)x[i + 1]) ++bad;
    }
    // chains of 8 (one thread's values), then a pairwise tree (shuffles, block, grid)
    std::vector<Df> level;
    for (int64_t i = 0; i < n; i += 8) {
        Df a = df_zero();
        for (int64_t k = i; k < i + 8 && k < n; ++k) a = df_add(a, x[k]);
        level.push_back(a);
    }
    while (level.size() > 1) {
        std::vector<Df> up;
        for (size_t i = 0; i < level.size(); i += 2)
            up.push_back(i + 1 < level.size() ? df_add(level[i], level[i + 1]) : level[i]);
        level.swap(up);
    }
    float naive = 0.0f;
    for (int64_t i = 0; i < n; ++i) naive += x[i];
    printf("%lld %.17g %.17g\n", bad, df_value(level[0]), (double)naive);
    return 0;
}
'''


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("dfloat")
    src = d / "df.cpp"
    src.write_text(SRC)
    out = d / "df"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I",
                    os.path.join(ROOT, "reda_erplacer_gb300", "csrc"), str(src), "-o", str(out)], check=True)
    return out


def _run(exe, x, tmp_path):
    p = tmp_path / "x.bin"
    with open(p, "wb") as f:
        f.write(np.int64(x.size).tobytes())
        f.write(x.astype(np.float32).tobytes())
    r = subprocess.run([str(exe), str(p)], capture_output=True, text=True, timeout=120, check=True)
    bad, df, naive = r.stdout.split()
    return int(bad), float(df), float(naive)


@pytest.mark.parametrize("kind", ["overflow", "lipschitz", "signed"])
def test_double_float_sums(exe, tmp_path, kind):
    rng = np.random.default_rng({"overflow": 1, "lipschitz": 2, "signed": 3}[kind])
    n = 1 << 20
    if kind == "overflow":     # per-bin overflow: many zeros, values below a bin area
        x = np.where(rng.random(n) < 0.6, 0.0, rng.random(n) * 3.7)
    elif kind == "lipschitz":  # squared step / gradient differences: wide dynamic range
        x = np.exp(rng.uniform(-12, 6, n)) ** 2
    else:                      # psi * rho products of both signs
        x = rng.normal(size=n) * np.exp(rng.uniform(-4, 4, n))
    x = x.astype(np.float32)
    bad, df, naive = _run(exe, x, tmp_path)
    assert bad == 0
    exact = math.fsum(x.astype(np.float64))
    mag = float(np.abs(x.astype(np.float64)).sum())
    err = abs(df - exact) / mag
    assert err <= 16 * 2.0 ** -44, err                      # about 44 bits
    assert abs(naive - exact) / mag > 1000 * max(err, 2.0 ** -52)   # FP32 alone is far off
