"""The seeded synthetic netlist generator (csrc/synth.cpp, host code) built
alone with AddressSanitizer and UndefinedBehaviorSanitizer, with no recovery:
random valid parameter sets give designs that satisfy every invariant the C
ABI's design validation checks, and invalid ones (NaN, infinite, negative or
too large sizes) are rejected with ERP_EINVAL."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

DRIVER = r'''
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <limits>
#include <random>
#include <vector>
#include "erplacer.h"

static int check(const erp_design &d) {
    if (d.num_nodes < d.num_movable || d.num_movable < 2) return 1;
    if (d.net_ptr[0] != 0 || d.net_ptr[d.num_nets] != d.num_pins) return 2;
    for (int e = 0; e < d.num_nets; ++e) {
        if (d.net_ptr[e + 1] < d.net_ptr[e]) return 3;
        if (e < d.n_2nets && d.net_ptr[e + 1] - d.net_ptr[e] != 2) return 4;
        for (int k = d.net_ptr[e]; k < d.net_ptr[e + 1]; ++k) {
            const int p = d.net_pins[k];
            if (p < 0 || p >= d.num_pins) return 5;
            for (int j = d.net_ptr[e]; j < k; ++j)   // distinct instances in a net
                if (d.pin_inst[d.net_pins[j]] == d.pin_inst[p]) return 6;
        }
    }
    std::vector<char> seen(d.num_pins, 0);
    if (d.inst_pin_ptr[0] != 0 || d.inst_pin_ptr[d.num_nodes] != d.num_pins) return 7;
    for (int i = 0; i < d.num_nodes; ++i) {
        if (!std::isfinite(d.x[i]) || !std::isfinite(d.y[i]) || d.w[i] < 0 || d.h[i] < 0) return 8;
        if (d.x[i] < 0 || d.y[i] < 0 || d.x[i] + d.w[i] > d.die_w * 1.0001f || d.y[i] + d.h[i] > d.die_h * 1.0001f) return 9;
        if (d.num_pins_f[i] != (float)(d.inst_pin_ptr[i + 1] - d.inst_pin_ptr[i])) return 10;
        for (int k = d.inst_pin_ptr[i]; k < d.inst_pin_ptr[i + 1]; ++k) {
            const int p = d.inst_pins[k];
            if (p < 0 || p >= d.num_pins || seen[p] || d.pin_inst[p] != i) return 11;
            seen[p] = 1;
        }
    }
    if (!(d.die_w > 0) || !(d.movable_area > 0) || !(d.cell_utilization > 0)) return 12;
    return 0;
}

int main() {
    std::mt19937_64 rng(5);
    auto U = [&](double a, double b) { return a + (b - a) * std::uniform_real_distribution<double>(0, 1)(rng); };
    auto I = [&](int a, int b) { return (int)std::uniform_int_distribution<int>(a, b)(rng); };
    long ok = 0;
    for (int it = 0; it < 400; ++it) {
        erp_synth_params p{};
        p.seed = (int64_t)rng();
        p.num_cells = it < 20 ? 2 + it : I(2, 6000);
        p.num_nets = I(1, p.num_cells * 2);
        p.num_io = I(0, 200);
        p.num_macros = I(0, 16);
        p.macro_area_frac = (float)U(0.0, 0.89 / (p.num_macros + 1));
        p.utilization = (float)U(0.05, 0.99);
        p.site_w = (float)U(0.05, 1.0);
        p.row_h = (float)U(0.5, 4.0);
        p.min_sites = I(1, 8);
        p.max_sites = p.min_sites + I(0, 12);
        p.jitter_frac = (float)U(0.0, 0.01);
        erp_synth *s = nullptr;
        if (erp_synth_create(&p, &s) != ERP_OK) { printf("valid parameters rejected at %d\n", it); return 1; }
        erp_design d;
        if (erp_synth_design(s, &d) != ERP_OK) return 1;
        const int c = check(d);
        if (c) { printf("invariant %d broken at %d\n", c, it); return 1; }
        erp_synth_destroy(s);
        ++ok;
    }
    // rejected parameter sets
    const float nan = std::numeric_limits<float>::quiet_NaN(), inf = std::numeric_limits<float>::infinity();
    erp_synth_params base{};
    base.seed = 1; base.num_cells = 100; base.num_nets = 100; base.utilization = 0.7f;
    base.site_w = 0.2f; base.row_h = 2.0f; base.min_sites = 2; base.max_sites = 8; base.jitter_frac = 0.001f;
    std::vector<erp_synth_params> bad(12, base);
    bad[0].utilization = nan; bad[1].site_w = inf; bad[2].row_h = -1.0f; bad[3].macro_area_frac = nan;
    bad[4].jitter_frac = nan; bad[5].num_cells = 1; bad[6].num_nets = 0; bad[7].max_sites = 1;
    bad[8].num_macros = 10; bad[8].macro_area_frac = 0.1f;
    bad[9].num_cells = INT32_MAX - 5; bad[9].num_io = 10;
    bad[10].num_io = -1; bad[11].utilization = inf;
    for (size_t k = 0; k < bad.size(); ++k) {
        erp_synth *s = nullptr;
        if (erp_synth_create(&bad[k], &s) != ERP_EINVAL) { printf("invalid set %zu accepted\n", k); return 1; }
    }
    if (erp_synth_create(nullptr, nullptr) != ERP_EINVAL) return 1;
    printf("done %ld\n", ok);
    return 0;
}
'''


def test_synth_under_address_and_ub_sanitizers(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    drv = tmp_path / "driver.cpp"
    drv.write_text(DRIVER)
    exe = tmp_path / "driver"
    b = subprocess.run([cxx, "-std=c++17", "-O1", "-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined",
                        "-fno-sanitize-recover=all", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), str(drv),
                        os.path.join(ROOT, "reda_erplacer_gb300", "csrc", "synth.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    if b.returncode != 0 and "sanitize" in b.stderr:
        pytest.skip("the compiler has no sanitizer runtime")
    assert b.returncode == 0, b.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.startswith("done"), (r.returncode, r.stdout[-500:], r.stderr[-4000:])
