"""GPU parity: every stage of the CUDA path, called through the C ABI, against
the oracle on the same seeded inputs.

Bars (per stage, identical inputs on both sides):
  * integer work — the int64 fixed-point density map and the fixed-cell map —
    bit-exact;
  * WA pin/instance gradients, potential, fields, electric force: relative L2
    <= 1e-5 (FP32);
  * HPWL / overflow totals: relative 1e-6 (double-float on the device, FP64 in
    the oracle);
  * scheduler: the same FP32 density weight and gamma as the oracle's FP64 form,
    bit for bit;
  * end to end after the same iteration count: HPWL within 0.5 %, overflow
    within 0.005.
"""
import numpy as np
import pytest

from conftest import rel_l2
from designs import edge_design, small_synth, spread_positions

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def R(built):
    import reda_erplacer_gb300 as R
    return R


@pytest.fixture(scope="module")
def O(built):
    from oracle import erp_oracle as O
    return O


def make_pair(R, O, d, m, n, td=1.0, xy=None):
    o = O.Oracle(d, m, n, target_density=td, start_mode=O.START_DB, density_mode=O.DENSITY_FIXED,
                 reduce_fp64=1)
    g = R.Placement(d, (m, n), td, start_mode=1)
    if xy is not None:
        o.set_positions(*xy)
        g.set_positions(*xy)
    return o, g


DESIGNS = {
    "edge_32x16": (lambda: edge_design(), 32, 16),
    "edge_16x64": (lambda: edge_design(seed=9), 16, 64),
    "synth3k_64": (lambda: small_synth(3000, seed=11), 64, 64),
    "synth20k_256": (lambda: small_synth(20000, seed=1, macros=0, io=400), 256, 256),
    # four-warp transform paths from the fixed-point map (rows 512 / 2048, columns 1024)
    "synth60k_1024x512": (lambda: small_synth(60000, seed=3), 1024, 512),
    "synth20k_256x2048": (lambda: small_synth(20000, seed=4, macros=2, io=200), 256, 2048),
}


@pytest.fixture(scope="module", params=list(DESIGNS))
def case(request, R, O):
    mk, m, n = DESIGNS[request.param]
    d = mk()
    xy = spread_positions(d, seed=5, frac=0.6)
    o, g = make_pair(R, O, d, m, n, xy=xy)
    yield d, o, g, m, n
    g.close()
    o.close()


def test_initial_density_bit_exact(case):
    d, o, g, m, n = case
    assert np.array_equal(g.array("INITIAL"), o.get("initial_map"))


def test_wirelength(case):
    d, o, g, m, n = case
    for gamma in (0.5, 4.0, 40.0):
        ho = o.compute_hpwl(gamma)
        hg = g.compute_hpwl(gamma)
        assert abs(hg - ho) <= 1e-6 * abs(ho)
        assert rel_l2(g.array("PIN_GRAD_X"), o.get("pin_grad_x")) <= TOL
        assert rel_l2(g.array("PIN_GRAD_Y"), o.get("pin_grad_y")) <= TOL
        assert rel_l2(g.array("WL_GRAD_X"), o.get("wl_grad_x")) <= TOL
        assert rel_l2(g.array("WL_GRAD_Y"), o.get("wl_grad_y")) <= TOL
        assert np.allclose(g.array("NET_HPWL"), o.get("net_hpwl"), rtol=1e-6, atol=1e-6 * abs(ho))


def test_potential(case):
    d, o, g, m, n = case
    eo, ovo = o.compute_potential(0)
    eg, ovg = g.compute_potential(0)
    assert np.array_equal(g.array("DENSITY_I64"), o.get("density_i64"))
    assert np.array_equal(g.array("DENSITY"), o.get("density_map"))
    assert abs(ovg - ovo) <= 1e-6 * max(abs(ovo), 1e-12)
    assert rel_l2(g.array("FIELD_X"), o.get("field_x")) <= TOL
    assert rel_l2(g.array("FIELD_Y"), o.get("field_y")) <= TOL
    assert rel_l2(g.array("POTENTIAL"), o.get("potential")) <= TOL
    assert abs(eg - eo) <= 1e-5 * abs(eo)
    assert rel_l2(g.array("DENS_GRAD_X"), o.get("dens_grad_x")) <= TOL
    assert rel_l2(g.array("DENS_GRAD_Y"), o.get("dens_grad_y")) <= TOL


def test_scheduler_matches_the_fp64_form(R, O):
    """erp_scheduler_update on the device against the oracle's FP64 form: both
    evaluate b^e as exp(e ln b) in FP64 and cast to FP32, so a sequence of
    updates through every branch (the density-weight growth and decay powers,
    both clamps, the gamma coefficient and its clamps) gives the same bits."""
    d = small_synth(3000, seed=12)
    o, g = make_pair(R, O, d, 64, 64)
    with g:
        v, s = o.view(), g.scalars()
        assert s["density_weight"] == v.density_weight and s["gamma"] == v.gamma
        seq = [(1e6, 0.1), (5e5, 2.0), (6e5, 0.5), (4e5, 0.02), (4.5e5, 0.15), (3e5, 1.0)] + \
              [(3e5 - 97.0 * k, 0.3 + 0.001 * k) for k in range(1, 250)]
        for k, (hp, ov) in enumerate(seq):
            o.scheduler_update(hp, ov)
            g.scheduler_update(hp, ov)
            v, s = o.view(), g.scalars()
            assert s["iteration"] == v.iteration
            assert s["density_weight"] == v.density_weight, k
            assert s["gamma"] == v.gamma, k


def test_nesterov_and_scheduler(case):
    d, o, g, m, n = case
    NM = d.num_movable
    for it in (0, 1, 2):
        hp_o = o.compute_hpwl(o.view().gamma)
        hp_g = g.compute_hpwl(g.scalars()["gamma"])
        _, ov_o = o.compute_potential(it)
        _, ov_g = g.compute_potential(it)
        x0, y0 = g.positions()
        o.nesterov(it)
        g.step_adaptive(it)
        o.scheduler_update(hp_o, ov_o)
        g.scheduler_update(hp_g, ov_g)
        xg, yg = g.positions()
        xo, yo = o.get("x"), o.get("y")
        # compare the displacement of this step
        ex = rel_l2(xg[:NM] - x0[:NM], xo[:NM] - x0[:NM])
        ey = rel_l2(yg[:NM] - y0[:NM], yo[:NM] - y0[:NM])
        s = g.scalars()
        v = o.view()
        pairs = ((s["alpha"], v.alpha), (s["beta"], v.beta), (s["density_weight"], v.density_weight),
                 (s["gamma"], v.gamma))
        print(f"iteration {it}: displacement {ex:.2e} / {ey:.2e}; alpha, beta, density weight, gamma "
              f"{[abs(a - b) / abs(b) if b else abs(a) for a, b in pairs]}")
        # measured on the six designs: displacement <= 1.6e-6, scalars <= 1.1e-7
        assert ex <= 1e-5 and ey <= 1e-5
        assert s["iteration"] == v.iteration
        for a, b in pairs:
            assert abs(a - b) <= 1e-6 * abs(b) + 1e-12
        # keep both sides on identical positions for the next round
        o.set_positions(xg, yg)


def test_step_matches_stage_sequence(R, O):
    """erp_step (graph replay, on-device scheduler) == the stage entry points."""
    d = small_synth(2000, seed=21)
    a = R.Placement(d, (64, 64), 1.0, start_mode=1)
    b = R.Placement(d, (64, 64), 1.0, start_mode=1)
    for it in range(6):
        a.step()
        sa = a.last_stats
        s = b.scalars()
        hp = b.compute_hpwl(s["gamma"])
        _, ov = b.compute_potential(it, want_energy=False)
        b.step_adaptive(it)
        b.scheduler_update(hp, ov)
        assert abs(sa["hpwl"] - hp) <= 1e-6 * hp
        assert abs(sa["overflow"] - ov) <= 1e-6
    xa, ya = a.positions()
    xb, yb = b.positions()
    assert np.array_equal(xa, xb) and np.array_equal(ya, yb)


@pytest.mark.parametrize("steps", [16, 40])
def test_density_map_in_the_scatter_order(R, O, steps):
    """The scatter takes the cells in a spatial order recomputed every 16 steps;
    after `steps` steps (the order recomputed, then the cells moved on) the int64
    map of the current positions is still bit-exact against the oracle's."""
    d = small_synth(20000, seed=31, macros=2, io=200)
    g = R.Placement(d, (256, 128), 1.0, start_mode=1)
    o = O.Oracle(d, 256, 128, target_density=1.0, start_mode=O.START_DB, density_mode=O.DENSITY_FIXED,
                 reduce_fp64=1)
    try:
        for _ in range(steps):
            g.step(stats=False)
        x, y = g.positions()
        o.set_positions(x, y)
        _, ovo = o.compute_potential(0)
        _, ovg = g.compute_potential(0)
        assert np.array_equal(g.array("DENSITY_I64"), o.get("density_i64"))
        assert abs(ovg - ovo) <= 1e-6 * max(abs(ovo), 1e-12)
        assert rel_l2(g.array("FIELD_X"), o.get("field_x")) <= TOL
    finally:
        g.close()
        o.close()


def test_step_host_matches_step(R):
    d = small_synth(2000, seed=22)
    a = R.Placement(d, (64, 64), 1.0)
    b = R.Placement(d, (64, 64), 1.0)
    x, y = b.positions()
    for _ in range(4):
        a.step()
        b.step_host(x, y)
    xa, ya = a.positions()
    assert np.array_equal(xa, x) and np.array_equal(ya, y)


def test_step_host_pinned_buffers(R):
    """Registered (pinned) host buffers are read and written by the device
    directly; the positions are those of the device-resident step."""
    torch = pytest.importorskip("torch")
    d = small_synth(2000, seed=23)
    a = R.Placement(d, (64, 64), 1.0)
    b = R.Placement(d, (64, 64), 1.0)
    x0, y0 = b.positions()
    xp, yp = torch.from_numpy(x0.copy()).pin_memory(), torch.from_numpy(y0.copy()).pin_memory()
    x, y = xp.numpy(), yp.numpy()
    for _ in range(5):
        a.step()
        st = b.step_host(x, y)
    xa, ya = a.positions()
    assert np.array_equal(xa, x) and np.array_equal(ya, y)
    assert st["hpwl"] == a.last_stats["hpwl"]


@pytest.mark.parametrize("iters", [60, 100])
def test_end_to_end_small(R, O, iters):
    """Whole loop on the 20k-cell workload from its jittered start: after the same
    iteration count HPWL within 0.5 % and overflow within 0.005 of the oracle."""
    d, cfg = R.workload_small()
    o = O.Oracle(d, 256, 256, target_density=1.0, start_mode=O.START_DB,
                 density_mode=O.DENSITY_FIXED, reduce_fp64=1)
    g = R.Placement(d, (256, 256), 1.0, start_mode=1)
    rel = []
    for i in range(iters):
        so = o.step()
        g.step()
        sg = g.last_stats
        rel.append(abs(sg["hpwl"] - so["hpwl"]) / so["hpwl"])
    print(f"iters {iters}: hpwl gpu {sg['hpwl']:.1f} oracle {so['hpwl']:.1f}  overflow gpu "
          f"{sg['overflow']:.5f} oracle {so['overflow']:.5f}  median rel {np.median(rel):.2e}")
    assert rel[-1] <= 0.005
    assert abs(sg["overflow"] - so["overflow"]) <= 0.005
    assert float(np.median(rel)) <= 0.005


def test_reference_start_first_step(R, O):
    """From the reference's exact-centre start the first step's metrics agree."""
    d, cfg = R.workload_small()
    o = O.Oracle(d, 256, 256, target_density=1.0, density_mode=O.DENSITY_FIXED, reduce_fp64=1)
    g = R.Placement(d, (256, 256), 1.0)
    so = o.step()
    g.step()
    assert abs(g.last_stats["hpwl"] - so["hpwl"]) <= 1e-6 * so["hpwl"]
    assert abs(g.last_stats["overflow"] - so["overflow"]) <= 1e-6


def _piled(d, sigma_bins, bins, seed):
    """Movable cells around the die centre, Gaussian with sigma in bins."""
    rng = np.random.default_rng(seed)
    x, y = d.x.copy(), d.y.copy()
    NM = d.num_movable
    bw, bh = d.die_w / bins[0], d.die_h / bins[1]
    x[:NM] = (d.die_w / 2 - d.w[:NM] / 2 + rng.normal(0, sigma_bins * bw, NM)).astype(np.float32)
    y[:NM] = (d.die_h / 2 - d.h[:NM] / 2 + rng.normal(0, sigma_bins * bh, NM)).astype(np.float32)
    return x, y


def _with_wide_cells(d, cells, factor):
    """The same design with some movable cells widened (pin offsets stay inside)."""
    import copy
    e = copy.deepcopy(d)
    e.w = e.w.copy()
    e.w[cells] *= factor
    NM = e.num_movable
    mov = float(np.sum(e.w[:NM].astype(np.float64) * e.h[:NM]))
    fixed = float(np.sum(e.w[NM:].astype(np.float64) * e.h[NM:]))
    e.movable_area = mov
    e.cell_utilization = mov / (e.die_w * e.die_h - fixed)
    return e


@pytest.mark.parametrize("case", ["centre", "piled_0.3", "piled_2", "spread", "wide_cells_piled", "wide_cells_spread"])
def test_density_map_crowded_and_wide_cells_bit_exact(R, O, case):
    """The scatter's two paths against the oracle's fixed-point replay, bit for
    bit: warps whose cells all fall within 3 x 3 bins (one warp-summed atomic per
    bin and plane), and warps of spread cells or holding a cell that spans many
    bins (each lane its own bin loops)."""
    d = small_synth(20000, seed=61, macros=2, io=200)
    bins = (128, 128)
    if case.startswith("wide"):
        d = _with_wide_cells(d, np.arange(0, 20000, 97), 12.0)
    if case == "centre":
        xy = (d.x.copy(), d.y.copy())
        NM = d.num_movable
        xy[0][:NM] = (d.die_w / 2 - d.w[:NM] / 2).astype(np.float32)
        xy[1][:NM] = (d.die_h / 2 - d.h[:NM] / 2).astype(np.float32)
    elif case in ("piled_0.3", "wide_cells_piled"):
        xy = _piled(d, 0.3, bins, 5)
    elif case == "piled_2":
        xy = _piled(d, 2.0, bins, 6)
    else:
        xy = spread_positions(d, seed=7)
    o, g = make_pair(R, O, d, *bins, xy=xy)
    try:
        _, ovo = o.compute_potential(0)
        _, ovg = g.compute_potential(0)
        assert np.array_equal(g.array("DENSITY_I64"), o.get("density_i64"))
        assert abs(ovg - ovo) <= 1e-6 * max(abs(ovo), 1e-12)
    finally:
        g.close()
        o.close()


def test_run_retires_at_overflow(R):
    d = small_synth(3000, seed=23)
    g = R.Placement(d, (64, 64), 1.0)
    it, last = g.run(400, stop_overflow=0.3)
    assert last["overflow"] <= 0.3
    assert it == last["iteration"] + 1
    # a second run continues from there
    it2, last2 = g.run(3, 0.0)
    assert it2 == 3 and last2["iteration"] == last["iteration"] + 3


@pytest.mark.parametrize("m,n", [(32, 1024), (1024, 32), (2048, 64), (16, 256), (128, 128),
                                 (1024, 1024), (512, 2048), (2048, 512)])
def test_spectral_standalone_shapes(R, O, m, n):
    """Every transform-size path (four-warp FFT for sides 512..2048, one-warp FFT
    for 64..256, shared-memory radix-2 FFT otherwise) against the FP32 oracle
    pipeline."""
    import torch
    rng = np.random.default_rng(m * 7 + n)
    rho = (0.5 + rng.random((m, n))).astype(np.float32)
    bw, bh = 0.9, 1.7
    fxo, fyo, po = O.poisson(rho, bw, bh, dtype=np.float32)
    sol = R.SpectralSolver(m, n, bw, bh)
    r = torch.tensor(rho, device="cuda")
    out = [torch.empty_like(r) for _ in range(3)]
    sol.solve(r.data_ptr(), *[t.data_ptr() for t in out])
    torch.cuda.synchronize()
    for got, want in zip(out, (fxo, fyo, po)):
        assert rel_l2(got.cpu().numpy(), want) <= TOL
    sol.close()


def test_spectral_standalone_fp64_error(R, O):
    """Isolated Poisson solve at 512x512 against the FP64 solve (error reported)."""
    import torch
    rng = np.random.default_rng(3)
    m = n = 512
    rho = (0.7 + 0.3 * rng.random((m, n))).astype(np.float64)
    bw, bh = 1.3, 1.1
    fx64, fy64, p64 = O.poisson(rho, bw, bh, dtype=np.float64)
    sol = R.SpectralSolver(m, n, bw, bh)
    r = torch.tensor(rho.astype(np.float32), device="cuda")
    fx = torch.empty_like(r); fy = torch.empty_like(r); ps = torch.empty_like(r)
    sol.solve(r.data_ptr(), fx.data_ptr(), fy.data_ptr(), ps.data_ptr())
    torch.cuda.synchronize()
    ex = rel_l2(fx.cpu().numpy(), fx64)
    ey = rel_l2(fy.cpu().numpy(), fy64)
    ep = rel_l2(ps.cpu().numpy(), p64)
    print(f"FP32 FFT solve vs FP64: field_x {ex:.2e} field_y {ey:.2e} potential {ep:.2e}")
    assert max(ex, ey, ep) <= 1e-5


def test_batch_scatter_autotune(R):
    """erp_batch_create times the scatter's block shapes on all instances at once
    and keeps the fastest; a fixed shape (environment) gives the same results."""
    import os
    mix = R.workload_batch(count=6, seed=77, min_cells=2000, max_cells=30000)
    designs, bins = [d for d, _ in mix], [b for _, b in mix]
    bt = R.Batch(designs, bins, 1.0, start_mode=1)
    chosen, cand = bt.tuning()
    assert [c for c, _ in cand] == [0, 512, 1024, 2048] and all(t > 0 for _, t in cand)
    best = min(t for _, t in cand)
    fastest_few = max((c for c, t in cand if c > 0 and t <= 1.10 * best + 1e-6), default=None)
    assert chosen == (fastest_few if fastest_few is not None else min(cand, key=lambda ct: ct[1])[0])
    its, lasts = bt.run(200)
    assert bt.tuning() == (chosen, cand)
    xs = [bt.positions(i) for i in range(len(mix))]
    bt.close()
    for forced in ("0", "2048"):
        os.environ["ERP_BATCH_SCATTER_CELLS"] = forced
        try:
            b2 = R.Batch(designs, bins, 1.0, start_mode=1)
            assert b2.tuning() == (int(forced), [])
            its2, lasts2 = b2.run(200)
            assert its2 == its and [l["hpwl"] for l in lasts2] == [l["hpwl"] for l in lasts]
            for i in range(len(mix)):
                xa, ya = b2.positions(i)
                assert np.array_equal(xa, xs[i][0]) and np.array_equal(ya, xs[i][1])
            b2.close()
        finally:
            del os.environ["ERP_BATCH_SCATTER_CELLS"]


def test_batch_spectral_autotune(R):
    """erp_batch_create also times the FP32 spectral passes' sequences per block
    (fixed shape 0, then 2 and 8) on all instances at once and keeps the fastest;
    every fixed shape (environment) gives the same results bit for bit."""
    import os
    mix = R.workload_batch(count=6, seed=78, min_cells=2000, max_cells=30000)
    designs, bins = [d for d, _ in mix], [b for _, b in mix]
    assert any(64 <= min(b) <= 256 for b in bins)
    bt = R.Batch(designs, bins, 1.0, start_mode=1)
    chosen, cand = bt.spectral_tuning()
    assert [c for c, _ in cand] == [0, 2, 8] and all(t > 0 for _, t in cand)
    assert chosen == min(cand, key=lambda ct: ct[1])[0]
    its, lasts = bt.run(120)
    xs = [bt.positions(i) for i in range(len(mix))]
    bt.close()
    for forced in ("0", "2", "8"):
        os.environ["ERP_BATCH_SPECTRAL_SEQS"] = forced
        try:
            b2 = R.Batch(designs, bins, 1.0, start_mode=1)
            assert b2.spectral_tuning() == (int(forced), [])
            its2, lasts2 = b2.run(120)
            assert its2 == its and [l["hpwl"] for l in lasts2] == [l["hpwl"] for l in lasts]
            for i in range(len(mix)):
                xa, ya = b2.positions(i)
                assert np.array_equal(xa, xs[i][0]) and np.array_equal(ya, xs[i][1])
            b2.close()
        finally:
            del os.environ["ERP_BATCH_SPECTRAL_SEQS"]


def test_batch_packed_and_branch_forms_match(R):
    """The packed launches (small FP32 instances: one launch per stage over a
    table of all of them) and a graph branch per instance give the same bits;
    both equal the designs run alone (test_batch_matches_individual_runs runs
    the default form, the packed one)."""
    import os
    mix = R.workload_batch(count=8, seed=79, min_cells=2000, max_cells=60000)
    designs, bins = [d for d, _ in mix], [b for _, b in mix]
    res = {}
    for form in ("packed", "branches"):
        os.environ["ERP_BATCH_FORM"] = form
        try:
            bt = R.Batch(designs, bins, 1.0, start_mode=1)
        finally:
            del os.environ["ERP_BATCH_FORM"]
        packed = bt.packed_instances()
        its, lasts = bt.run(120, stop_overflow=0.6)
        res[form] = (packed, its, [(l["hpwl"], l["overflow"]) for l in lasts],
                     [bt.positions(i) for i in range(len(mix))])
        bt.close()
    small = sum(1 for d, b in mix if max(b) <= 256 and d.num_movable <= 100000)
    assert res["packed"][0] == small > 0 and res["branches"][0] == 0
    assert res["packed"][1] == res["branches"][1] and res["packed"][2] == res["branches"][2]
    for (xa, ya), (xb, yb) in zip(res["packed"][3], res["branches"][3]):
        assert np.array_equal(xa, xb) and np.array_equal(ya, yb)


def test_batch_matches_individual_runs(R):
    """Instances advanced together in one batched graph end bit-identical to the
    same designs run alone (each instance's kernels are the same; only their
    scheduling differs)."""
    mix = R.workload_batch(count=5, seed=77, min_cells=1500, max_cells=12000)
    designs = [d for d, _ in mix]
    bins = [b for _, b in mix]
    bt = R.Batch(designs, bins, 1.0, start_mode=1)
    its, lasts = bt.run(150, stop_overflow=0.6)
    for i, (d, b) in enumerate(mix):
        g = R.Placement(d, b, 1.0, start_mode=1)
        it, last = g.run(150, stop_overflow=0.6)
        assert it == its[i]
        assert last["hpwl"] == lasts[i]["hpwl"] and last["overflow"] == lasts[i]["overflow"]
        xa, ya = g.positions()
        xb, yb = bt.positions(i)
        assert np.array_equal(xa, xb) and np.array_equal(ya, yb)
        g.close()
    # retired instances stay retired; a second call continues all of them
    its2, _ = bt.run(3, 0.0)
    assert its2 == [3] * len(mix)
    bt.close()


@pytest.mark.parametrize("m,n", [(256, 256), (512, 1024), (1024, 512)])
@pytest.mark.parametrize("prec,bound", [(1, 3e-2), (2, 5e-3)])
def test_spectral_tensor_core_forms(R, O, m, n, prec, bound):
    """DCT/IDXST contractions on the tensor cores (TF32; BF16 hi/lo x3) against
    the FP64 solve on white-noise maps (the hardest case for a contraction: every
    output sums K terms of order one that cancel); without psi too.  Measured on
    these inputs: TF32 ~1e-2, BF16x3 ~2e-3; on the smooth isolated-solve maps
    2e-3 and 3e-5..6e-4 (reported by the benchmark)."""
    import torch
    rng = np.random.default_rng(m + 5 * n + prec)
    rho = (0.5 + rng.random((m, n))).astype(np.float32)
    bw, bh = 1.1, 0.8
    want = O.poisson(rho, bw, bh, dtype=np.float64)
    sol = R.SpectralSolver(m, n, bw, bh, precision=prec)
    r = torch.tensor(rho, device="cuda")
    out = [torch.empty_like(r) for _ in range(3)]
    sol.solve(r.data_ptr(), *[t.data_ptr() for t in out])
    torch.cuda.synchronize()
    for got, w in zip(out, want):
        assert rel_l2(got.cpu().numpy(), w) <= bound
    out2 = [torch.empty_like(r) for _ in range(2)]
    sol.solve(r.data_ptr(), out2[0].data_ptr(), out2[1].data_ptr(), None)
    torch.cuda.synchronize()
    assert torch.equal(out2[0], out[0]) and torch.equal(out2[1], out[1])
    sol.close()


def test_spectral_tensor_core_rejects_odd_sizes(R):
    with pytest.raises(R.ErpError):
        R.SpectralSolver(64, 256, 1.0, 1.0, precision=1)


@pytest.mark.parametrize("prec", [1, 2])
def test_step_mixed_precision_forms(R, O, prec):
    """Placement step with the tensor-core spectral solve: the fixed-point map and
    rho are the FP32 path's bit for bit, the fields stay within the form's error,
    and after 100 iterations overflow is within 0.005 and HPWL within 0.5 % of the
    plain FP32 run for BF16x3, the mixed form that batching and serving use.

    TF32 is held to 2 % HPWL: its operands keep 10 mantissa bits, the fields come
    out about 2e-3 off the FP64 solve (stated by the benchmark's isolated-solve
    section), and on this 20,000-cell design after 100 iterations from spread
    positions its HPWL is 0.8 % from the FP32 run's.  It is an opt-in form with a
    stated error, not one that meets the end-state bar here (on the 1M-cell
    workload it lands 0.06 % from the FP32 run at iteration 444)."""
    d = small_synth(20000, seed=1, macros=0, io=400)
    xy = spread_positions(d, seed=5, frac=0.6)
    a = R.Placement(d, (256, 256), 1.0, start_mode=1)
    b = R.Placement(d, (256, 256), 1.0, start_mode=1, precision=prec)
    for p in (a, b):
        p.set_positions(*xy)
    _, ova = a.compute_potential(0)
    _, ovb = b.compute_potential(0)
    assert np.array_equal(a.array("DENSITY_I64"), b.array("DENSITY_I64"))
    assert np.array_equal(a.array("DENSITY"), b.array("DENSITY"))
    assert abs(ova - ovb) <= 1e-6 * abs(ova)
    assert rel_l2(b.array("FIELD_X"), a.array("FIELD_X")) <= (3e-2 if prec == 1 else 5e-3)
    a.close()
    b.close()
    a = R.Placement(d, (256, 256), 1.0, start_mode=1)
    b = R.Placement(d, (256, 256), 1.0, start_mode=1, precision=prec)
    ia, la = a.run(100, 0.0)
    ib, lb = b.run(100, 0.0)
    assert ia == ib == 100
    assert abs(lb["hpwl"] - la["hpwl"]) <= (2e-2 if prec == 1 else 5e-3) * la["hpwl"]
    assert abs(lb["overflow"] - la["overflow"]) <= 5e-3
    a.close()
    b.close()


def test_step_mixed_precision_rejects_small_grids(R):
    d = small_synth(3000, seed=2)
    with pytest.raises(R.ErpError):
        R.Placement(d, (64, 64), 1.0, start_mode=1, precision=2)


def test_mixed_precision_batch_matches_individual_runs(R):
    """The mixed batched form (BF16x3 tensor-core solve where the grid allows,
    FP32 FFT on 64^2) ends bit-identical to each design run alone in its form."""
    mix = R.workload_batch(count=4, seed=78, min_cells=8000, max_cells=60000)
    designs = [d for d, _ in mix]
    bins = [b for _, b in mix]
    precs = [2 if b[0] >= 128 else 0 for b in bins]
    assert any(p == 2 for p in precs)
    bt = R.Batch(designs, bins, 1.0, start_mode=1, precision=precs)
    its, lasts = bt.run(120, stop_overflow=0.5)
    for i, (d, b) in enumerate(mix):
        g = R.Placement(d, b, 1.0, start_mode=1, precision=precs[i])
        it, last = g.run(120, stop_overflow=0.5)
        assert it == its[i]
        assert last["hpwl"] == lasts[i]["hpwl"] and last["overflow"] == lasts[i]["overflow"]
        xa, ya = g.positions()
        xb, yb = bt.positions(i)
        assert np.array_equal(xa, xb) and np.array_equal(ya, yb)
        g.close()
    bt.close()
