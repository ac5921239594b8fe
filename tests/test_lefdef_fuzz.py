"""Robustness of the LEF/DEF reader and writers (host code of the library).

Every truncation of each golden file and seeded byte / token / line mutations
either parse, after which the database, the names, the placed DEF and the
export all work, or fail with an error status and a message.

* The library's own build runs the cases through ctypes in a child process,
  so a crash fails the test instead of the test run.
* `csrc/lefdef.cpp` (host C++ with no other dependency) is also built with
  AddressSanitizer and UndefinedBehaviorSanitizer, with no recovery, into a
  small driver that runs the same cases: an out-of-bounds access or undefined
  behaviour that happens not to crash still fails the test.
"""
import itertools
import os
import random
import shutil
import struct
import subprocess
import sys

import pytest

from conftest import ROOT

GOLD = os.path.join(ROOT, "tests", "golden", "lefdef")
NAMES = ["tiny_tech.lef", "tiny_cells.lef", "tiny.def"]
JUNK = [b"(", b")", b";", b"-", b"+", b"END", b"MACRO", b"PIN", b"NETS", b"COMPONENTS", b"1e40", b"-7",
        b"nan", b"99999999999999999999", b"\x00", b"\xff", b"#", b"\n", b'"', b"*"]


def cases(mutations=1500, seed=11, truncations=True):
    """The golden triple, every truncation of each file, then seeded mutations."""
    orig = [open(os.path.join(GOLD, n), "rb").read() for n in NAMES]
    yield list(orig)
    for k in range(3 if truncations else 0):
        for n in range(len(orig[k])):
            t = list(orig)
            t[k] = orig[k][:n]
            yield t
    rng = random.Random(seed)
    for _ in range(mutations):
        k = rng.randrange(3)
        b = bytearray(orig[k])
        for _ in range(rng.randint(1, 4)):
            op = rng.randrange(4)
            p = rng.randrange(len(b) + 1)
            if op == 0 and b:                               # replace a byte
                b[min(p, len(b) - 1)] = rng.randrange(256)
            elif op == 1:                                   # insert a token
                b[p:p] = b" " + rng.choice(JUNK) + b" "
            elif op == 2 and b:                             # delete a span
                del b[p:p + rng.randint(1, 12)]
            else:                                           # duplicate a line
                lines = bytes(b).split(b"\n")
                j = rng.randrange(len(lines))
                lines.insert(j, lines[j])
                b = bytearray(b"\n".join(lines))
        t = list(orig)
        t[k] = bytes(b)
        yield t


CHILD = r'''
import os, sys, tempfile
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, os.path.join(sys.argv[1], "tests"))
import numpy as np
import reda_erplacer_gb300 as R
from reda_erplacer_gb300 import lefdef
from test_lefdef_fuzz import NAMES, cases
tmp = tempfile.mkdtemp()
ok = err = 0
for i, texts in enumerate(cases()):
    paths = []
    for n, t in zip(NAMES, texts):
        p = os.path.join(tmp, n)
        with open(p, "wb") as f:
            f.write(t)
        paths.append(p)
    try:
        nl = lefdef.Netlist.read(paths[:2], paths[2])
    except R.ErpError as e:
        assert str(e), "an error without a message"
        err += 1
        continue
    with nl:
        d = nl.design()
        st = nl.stats()
        assert st["num_nodes"] == d.num_nodes and st["num_nets"] == d.num_nets
        for j in (0, d.num_nodes - 1):
            if d.num_nodes:
                nl.node_name(j)
        for e in (0, d.num_nets - 1):
            if d.num_nets:
                nl.net_name(e)
        x = np.asarray(d.x, np.float32)[: d.num_movable] + 1.0
        y = np.asarray(d.y, np.float32)[: d.num_movable] + 1.0
        for call in (lambda: nl.write_placed(x, y, os.path.join(tmp, "placed.def")),
                     lambda: nl.write(os.path.join(tmp, "out.lef"), os.path.join(tmp, "out.def"))):
            try:
                call()
            except R.ErpError as e:
                assert str(e)
    ok += 1
    if i == 0:
        assert ok == 1, "the golden files must parse"
print("done", ok, err)
'''

DRIVER = r'''
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "erplacer.h"

// Runs every case of a corpus file (per case: three u32-length-prefixed files,
// technology LEF, cells LEF, DEF) through the reader, then the accessors and
// both writers of each design that parses.
int main(int argc, char **argv) {
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    const std::string dir = argv[2];
    const std::string p[3] = {dir + "/tech.lef", dir + "/cells.lef", dir + "/in.def"};
    long ok = 0, err = 0;
    for (;;) {
        bool end = false;
        for (int k = 0; k < 3 && !end; ++k) {
            uint32_t n;
            if (fread(&n, 4, 1, f) != 1) { end = true; break; }
            std::vector<char> b(n);
            if (n && fread(b.data(), 1, n, f) != n) return 3;
            FILE *o = fopen(p[k].c_str(), "wb");
            if (n) fwrite(b.data(), 1, n, o);
            fclose(o);
        }
        if (end) break;
        const char *lefs[2] = {p[0].c_str(), p[1].c_str()};
        erp_netlist *nl = nullptr;
        if (erp_lefdef_read(lefs, 2, p[2].c_str(), &nl) != ERP_OK) {
            const char *m = erp_lefdef_last_error();
            if (!m || !*m) { printf("error without a message\n"); return 4; }
            ++err;
            continue;
        }
        erp_design d;
        erp_lefdef_stats st;
        if (erp_netlist_design(nl, &d) != ERP_OK || erp_netlist_stats(nl, &st) != ERP_OK) return 5;
        for (int i = 0; i < d.num_nodes; ++i) if (!erp_netlist_node_name(nl, i)) return 6;
        for (int e = 0; e < d.num_nets; ++e) if (!erp_netlist_net_name(nl, e)) return 6;
        std::vector<float> x(d.num_movable + 1), y(d.num_movable + 1);
        for (int i = 0; i < d.num_movable; ++i) { x[i] = d.x[i] + 1.0f; y[i] = d.y[i] + 1.0f; }
        erp_def_write_placed(nl, x.data(), y.data(), (dir + "/placed.def").c_str());
        erp_lefdef_write(nl, (dir + "/out.lef").c_str(), (dir + "/out.def").c_str());
        erp_netlist_destroy(nl);
        ++ok;
    }
    printf("done %ld %ld\n", ok, err);
    return 0;
}
'''


def test_reader_survives_truncations_and_mutations(built):
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.returncode, r.stdout[-1500:], r.stderr[-3000:])
    assert r.stdout.startswith("done")


def test_reader_under_address_and_ub_sanitizers(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    drv = tmp_path / "driver.cpp"
    drv.write_text(DRIVER)
    exe = tmp_path / "driver"
    flags = ["-std=c++17", "-O1", "-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined",
             "-fno-sanitize-recover=all", "-I", os.path.join(ROOT, "include")]
    b = subprocess.run([cxx, *flags, str(drv), os.path.join(ROOT, "reda_erplacer_gb300", "csrc", "lefdef.cpp"),
                        "-o", str(exe)], capture_output=True, text=True)
    if b.returncode != 0 and "sanitize" in b.stderr:
        pytest.skip("the compiler has no sanitizer runtime")
    assert b.returncode == 0, b.stderr[-3000:]
    corpus = tmp_path / "corpus.bin"
    with open(corpus, "wb") as f:
        for texts in itertools.chain(cases(), cases(mutations=5000, seed=29, truncations=False)):
            for t in texts:
                f.write(struct.pack("<I", len(t)))
                f.write(t)
    work = tmp_path / "w"
    work.mkdir()
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([str(exe), str(corpus), str(work)], capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0 and r.stdout.startswith("done"), (r.returncode, r.stdout[-500:], r.stderr[-4000:])
