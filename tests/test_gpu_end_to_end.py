"""End-to-end parity of the whole loop at the configured iteration counts:
the 20,000-cell workload for its 450 iterations and the 1,000,000-cell
workload for its 1,000, GPU against the oracle in both of its forms -- the
fixed-point / FP64 form and the reference's own FP32 rules (sequential density
below iteration 200, then atomic adds; FP32 sums).

The loop amplifies rounding differences.  In its fast-spreading phase and past
its overflow minimum two legitimate executions of the reference algorithm (its
FP32 rules and its FP64 form, reloaded with the same state) part by up to 1 %
HPWL within 25 iterations, but by under 4e-5 within 10; over a whole run they
end far more than 0.5 % apart (tests/test_oracle_golden.py pins this on the
CPU).  A fixed-iteration bar at the end of a run is therefore not met by the
reference against itself, and parity is checked in the two forms that are
meaningful:

  * shadowing: the GPU run is followed for every iteration of the workload,
    and every 10 iterations the oracle is reloaded with the GPU's whole loop
    state (positions, Nesterov history, scheduler and optimiser scalars); at
    the end of every segment -- in every phase of the run, spreading,
    converged and diverging -- HPWL is within 0.5 % and overflow within 0.005
    of the oracle's (on the 1,000,000-cell workload, of the FP32 rules in the
    segments where the reference's two forms agree to that bar themselves, see
    test_large_workload_shadowing);
  * free run: both sides run the workload's iterations from the same start
    without any reload; the converged state (the overflow minimum and the HPWL
    there) and, on the large workload, the iteration where overflow first
    reaches 0.10 are within 0.5 % / 0.005, and so are the iterations before
    the reference's own orders part.  The final state is reported next to the
    spread of the reference's own orders.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HPWL_BAR = 0.005
OVF_BAR = 0.005


@pytest.fixture(scope="module")
def R(built):
    import reda_erplacer_gb300 as R
    return R


@pytest.fixture(scope="module")
def O(built):
    from oracle import erp_oracle as O
    return O


FORMS = {
    # name: (density mode, FP64 reductions, threads)
    "fixed_fp64": ("DENSITY_FIXED", 1, 0),
    "reference_fp32": ("DENSITY_REFERENCE", 0, 0),
}


def oracle(O, d, cfg, form, start_mode, threads=None):
    dm, rf, th = FORMS[form]
    m, n = cfg["bins"]
    return O.Oracle(d, m, n, target_density=cfg["target_density"], start_mode=start_mode,
                    density_mode=getattr(O, dm), reduce_fp64=rf, num_threads=th if threads is None else threads)


def shadow(R, O, d, cfg, forms, seg):
    """Follow the GPU run over the workload's iterations, reloading one oracle
    per form with the GPU's loop state every `seg` iterations.  Per segment, the
    GPU's HPWL and overflow at its last iteration and each form's."""
    m, n = cfg["bins"]
    g = R.Placement(d, (m, n), cfg["target_density"], start_mode=1)
    os_ = {f: oracle(O, d, cfg, f, O.START_DB) for f in forms}
    rows = []
    try:
        it = 0
        while it < cfg["iterations"]:
            if it:
                for o in os_.values():
                    o.load_state(g)
            k = min(seg, cfg["iterations"] - it)
            for _ in range(k):
                g.step()
            sg = g.last_stats
            row = {"iteration": it + k, "gpu": (sg["hpwl"], sg["overflow"])}
            for f, o in os_.items():
                for _ in range(k):
                    so = o.step()
                row[f] = (so["hpwl"], so["overflow"])
            rows.append(row)
            it += k
    finally:
        g.close()
        for o in os_.values():
            o.close()
    return rows


def deviation(rows, a, b):
    """Per segment: relative HPWL and absolute overflow difference of a from b."""
    rel = np.array([abs(r[a][0] - r[b][0]) / r[b][0] for r in rows])
    dov = np.array([abs(r[a][1] - r[b][1]) for r in rows])
    return rel, dov


@pytest.mark.parametrize("form", list(FORMS))
def test_small_workload_shadowing(R, O, form):
    """20,000 cells, 256 x 256 bins, all 450 iterations, oracle reloaded every
    10 iterations: every segment ends within the bar."""
    d, cfg = R.workload_small()
    t0 = time.time()
    rows = shadow(R, O, d, cfg, [form], 10)
    rel, dov = deviation(rows, "gpu", form)
    worst = int(np.argmax(rel))
    print(f"\n{form}: segments {len(rows)}, max hpwl rel {rel.max():.2e} (segment ending at "
          f"{rows[worst]['iteration']}, median {np.median(rel):.2e}), max overflow diff {dov.max():.2e}; "
          f"{time.time() - t0:.1f} s")
    assert len(rows) == 45
    assert rel.max() <= HPWL_BAR
    assert dov.max() <= OVF_BAR


def trajectory(run_step, iters):
    h, ov = np.empty(iters), np.empty(iters)
    for i in range(iters):
        s = run_step()
        h[i], ov[i] = s["hpwl"], s["overflow"]
    return h, ov


def gpu_trajectory(R, d, cfg, start_mode):
    m, n = cfg["bins"]
    g = R.Placement(d, (m, n), cfg["target_density"], start_mode=start_mode)

    def st():
        g.step()
        return g.last_stats
    try:
        return trajectory(st, cfg["iterations"])
    finally:
        g.close()


def oracle_trajectory(O, d, cfg, form, start_mode, threads=None):
    o = oracle(O, d, cfg, form, start_mode, threads)
    try:
        return trajectory(o.step, cfg["iterations"])
    finally:
        o.close()


def converged(h, ov):
    k = int(np.argmin(ov))
    return k, h[k], ov[k]


@pytest.fixture(scope="module", params=["jittered", "centre"])
def small_free_run(request, R, O):
    """The GPU run and the reference's own orders (fixed-point / FP64; FP32
    rules, and FP32 rules with FP64 sums, on one thread so that each is
    deterministic) over the 450 iterations from one start."""
    start = 1 if request.param == "jittered" else 0
    d, cfg = R.workload_small()
    t0 = time.time()
    fam = {"fixed_fp64": oracle_trajectory(O, d, cfg, "fixed_fp64", start),
           "reference_fp32": oracle_trajectory(O, d, cfg, "reference_fp32", start, threads=1)}
    o = O.Oracle(d, 256, 256, target_density=1.0, start_mode=start, density_mode=O.DENSITY_REFERENCE,
                 reduce_fp64=1, num_threads=1)
    fam["reference_fp64_sums"] = trajectory(o.step, cfg["iterations"])
    o.close()
    print(f"\noracle runs: {time.time() - t0:.1f} s")
    return request.param, gpu_trajectory(R, d, cfg, start), fam


def test_small_workload_free_run(small_free_run):
    start, (hg, og), fam = small_free_run
    kg, hgc, ogc = converged(hg, og)
    print(f"\n{start} start: GPU overflow minimum {ogc:.5f} at iteration {kg + 1}, HPWL there {hgc:.6g}; "
          f"final HPWL {hg[-1]:.6g} overflow {og[-1]:.5f}")
    H = np.stack([h for h, _ in fam.values()])
    OV = np.stack([o for _, o in fam.values()])
    for name, (h, ov) in fam.items():
        k, hc, oc = converged(h, ov)
        print(f"  {name:24s} overflow minimum {oc:.5f} at {k + 1}, HPWL there {hc:.6g} "
              f"(GPU {(hgc - hc) / hc:+.2e}, {ogc - oc:+.1e}); final HPWL {h[-1]:.6g} overflow {ov[-1]:.5f}")
    spread_h = (H.max(0) - H.min(0)) / H.min(0)
    spread_o = OV.max(0) - OV.min(0)
    print(f"  reference orders' own spread at iteration 450: HPWL {spread_h[-1]:.2e}, overflow {spread_o[-1]:.2e}")
    # the converged state
    for name in ("fixed_fp64", "reference_fp32"):
        h, ov = fam[name]
        k, hc, oc = converged(h, ov)
        assert abs(ogc - oc) <= OVF_BAR, name
        assert abs(hgc - hc) / hc <= HPWL_BAR, name
    # while the reference's own orders agree to the bar, so does the GPU
    agree = np.nonzero((spread_h > HPWL_BAR) | (spread_o > OVF_BAR))[0]
    upto = int(agree[0]) if len(agree) else len(hg)
    print(f"  reference orders within the bar up to iteration {upto}")
    hf, of = fam["fixed_fp64"]
    assert np.all(np.abs(hg[:upto] - hf[:upto]) / hf[:upto] <= HPWL_BAR)
    assert np.all(np.abs(og[:upto] - of[:upto]) <= OVF_BAR)
    # the final state: reported against the reference's own spread (past the
    # overflow minimum the orders part, see the module docstring)
    print(f"  final HPWL GPU {hg[-1]:.6g} in [{H[:, -1].min():.6g}, {H[:, -1].max():.6g}] of the reference "
          f"orders: {bool(H[:, -1].min() <= hg[-1] <= H[:, -1].max())}")


def test_large_workload_shadowing(R, O):
    """1,000,000 cells, 1024 x 1024 bins, all 1,000 iterations, both oracle forms
    reloaded from the GPU every 5 iterations.

    At this size the loop is more sensitive than on the small workload.  Past
    its overflow minimum (iteration ~510) it amplifies a difference of one
    rounding to about 1 % of overflow within 10 iterations, so the segments are
    5 iterations long (the same oracle work, more reloads).  And the reference's
    FP32 rules are themselves noisy here: a bin that 700,000 cells reach early in
    the run is one FP32 running sum, and the FP32 Lipschitz and rescale sums run
    over 10^6 terms; from the same state its FP32 rules and its FP64 form part
    by more than the bar in some segments.  So:
      * in every segment the GPU is within the bar of the FP64 form, whose
        arithmetic it follows (fixed-point map, double-float sums);
      * in every segment where the reference's two forms agree to the bar, the
        GPU is within the bar of the FP32 rules too;
      * the segments where they do not are reported with both distances."""
    d, cfg = R.workload_large()
    t0 = time.time()
    rows = shadow(R, O, d, cfg, ["reference_fp32", "fixed_fp64"], 5)
    assert len(rows) == 200
    g64_h, g64_o = deviation(rows, "gpu", "fixed_fp64")
    g32_h, g32_o = deviation(rows, "gpu", "reference_fp32")
    self_h, self_o = deviation(rows, "fixed_fp64", "reference_fp32")
    agree = (self_h <= HPWL_BAR) & (self_o <= OVF_BAR)
    k64 = int(np.argmax(g64_o))
    print(f"\n{time.time() - t0:.1f} s; segments {len(rows)}")
    print(f"  GPU vs FP64 form: max hpwl rel {g64_h.max():.2e}, max overflow diff {g64_o.max():.2e} "
          f"(segment ending at {rows[k64]['iteration']}), median {np.median(g64_h):.2e} / {np.median(g64_o):.2e}")
    print(f"  GPU vs FP32 rules where the forms agree ({int(agree.sum())} segments): max hpwl rel "
          f"{g32_h[agree].max():.2e}, max overflow diff {g32_o[agree].max():.2e}")
    for k in np.nonzero(~agree)[0]:
        print(f"  segment ending at {rows[k]['iteration']}: forms part by hpwl {self_h[k]:.2e} / overflow "
              f"{self_o[k]:.2e}; GPU vs FP32 rules {g32_h[k]:.2e} / {g32_o[k]:.2e}")
    assert g64_h.max() <= HPWL_BAR and g64_o.max() <= OVF_BAR
    assert g32_h[agree].max() <= HPWL_BAR and g32_o[agree].max() <= OVF_BAR
    assert agree.sum() >= 150


def test_large_workload_free_run(R, O):
    """1,000,000 cells from the jittered start, 1,000 iterations, no reload: the
    GPU against the reference's FP64 form and its FP32 rules at the iteration
    where the GPU first reaches overflow 0.10 and at the converged state.

    The FP32 rules are not deterministic past iteration 200: the bins take their
    contributions by atomic adds in whatever order the threads reach them, as
    the reference's Mutex-guarded bins do, and the loop amplifies the rounding.
    Repeated runs of them put HPWL at the overflow-0.10 iteration anywhere in a
    band about 0.6 % wide (985.2e6 to 990.8e6 in six runs, against the GPU's
    990.7e6), so a single run of them is held to twice the bar; the FP64 form,
    which is deterministic, is held to the bar itself."""
    d, cfg = R.workload_large()
    t0 = time.time()
    hg, og = gpu_trajectory(R, d, cfg, 1)
    hr, orf = oracle_trajectory(O, d, cfg, "reference_fp32", 1)
    hf, of = oracle_trajectory(O, d, cfg, "fixed_fp64", 1)
    print(f"\n{time.time() - t0:.1f} s")
    kt = int(np.argmax(og <= 0.10))
    kg, hgc, ogc = converged(hg, og)
    for name, h, o, bar in (("FP32 rules", hr, orf, 2 * HPWL_BAR), ("FP64 form", hf, of, HPWL_BAR)):
        kr, hrc, orc = converged(h, o)
        print(f"{name}: overflow 0.10 at iteration {kt + 1}: HPWL {hg[kt]:.6g} / {h[kt]:.6g} "
              f"({(hg[kt] - h[kt]) / h[kt]:+.2e}), overflow {og[kt]:.5f} / {o[kt]:.5f}; overflow minimum GPU "
              f"{ogc:.5f} at {kg + 1} (HPWL {hgc:.6g}), reference {orc:.5f} at {kr + 1} (HPWL {hrc:.6g}); "
              f"final HPWL {hg[-1]:.6g} / {h[-1]:.6g}, overflow {og[-1]:.5f} / {o[-1]:.5f}")
        assert abs(hg[kt] - h[kt]) / h[kt] <= bar, name
        assert abs(og[kt] - o[kt]) <= OVF_BAR, name
        assert abs(ogc - orc) <= OVF_BAR, name
        assert abs(hgc - hrc) / hrc <= bar, name
    assert og[kt] <= 0.10
