"""Headless snapshots against the reference's drawing rules restated in numpy
(bit-exact RGB), and checkpoint / resume (a restored run continues bit-identically;
foreign or damaged checkpoints are rejected)."""
import numpy as np
import pytest

from designs import small_synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R(built):
    import reda_erplacer_gb300 as R
    return R


def draw_placement_ref(d, x, y):
    """src/drawing.rs:7-60: white image ceil(die) pixels; instance i painted in
    index order (movable blue, fixed red) over [ceil x, +ceil w) x
    [H - ceil y - ceil h, +ceil h), clipped; zero-size instances skipped."""
    W, H = int(np.ceil(d.die_w)), int(np.ceil(d.die_h))
    img = np.full((H, W, 3), 255, np.uint8)
    for i in range(d.num_nodes):
        w, h = int(np.ceil(d.w[i])), int(np.ceil(d.h[i]))
        if w == 0 or h == 0:
            continue
        xi = int(np.ceil(x[i]))
        yi = H - int(np.ceil(y[i])) - h
        x0, x1 = max(xi, 0), min(xi + w, W)
        y0, y1 = max(yi, 0), min(yi + h, H)
        if x0 >= x1 or y0 >= y1:
            continue
        img[y0:y1, x0:x1] = (255, 0, 0) if i >= d.num_movable else (0, 0, 255)
    return img


def draw_density_ref(mp):
    """src/epotential.rs:199-223 with the map [m, n]: pixel (i, n-1-j)."""
    m, n = mp.shape
    lo, hi = np.float32(mp.min()), np.float32(mp.max())
    den = np.float32(np.float32(hi - lo) + np.float32(1e-12))
    v = np.clip(((mp - lo).astype(np.float32) / den).astype(np.float32), 0, 1).astype(np.float32)
    img = np.zeros((n, m, 3), np.uint8)
    r = (v * np.float32(255.0)).astype(np.float32).astype(np.uint8)
    b = ((np.float32(1.0) - v) * np.float32(255.0)).astype(np.float32).astype(np.uint8)
    img[::-1, :, 0] = r.T
    img[::-1, :, 2] = b.T
    return img


def test_snapshot_placement_matches_reference_rule(R, tmp_path):
    d = small_synth(3000, seed=21, macros=3, io=60)
    pl = R.Placement(d, (64, 64), 1.0, start_mode=1)
    pl.run(40, 0.0)
    x, y = pl.positions()
    got = pl.snapshot_placement(str(tmp_path / "p.ppm"))
    want = draw_placement_ref(d, x, y)
    assert got.shape == want.shape
    assert np.array_equal(got, want)
    raw = open(tmp_path / "p.ppm", "rb").read()
    assert raw.startswith(b"P6\n%d %d\n255\n" % (want.shape[1], want.shape[0]))
    pl.close()


def test_snapshot_density_matches_reference_rule(R):
    d = small_synth(3000, seed=22)
    pl = R.Placement(d, (64, 32), 1.0, start_mode=1)
    pl.run(25, 0.0)
    got = pl.snapshot_density()
    mp = pl.array("DENSITY").reshape(64, 32)   # the map snapshot_density just computed
    assert np.array_equal(got, draw_density_ref(mp))
    pl.close()


def test_checkpoint_resume_bit_identical(R):
    d = small_synth(5000, seed=23)
    a = R.Placement(d, (64, 64), 1.0, start_mode=1)
    a.run(30, 0.0)
    blob = a.checkpoint()
    ita, la = a.run(25, 0.0)
    xa, ya = a.positions()
    b = R.Placement(d, (64, 64), 1.0, start_mode=1)
    b.restore(blob)
    itb, lb = b.run(25, 0.0)
    xb, yb = b.positions()
    assert itb == ita and lb == la
    assert np.array_equal(xa, xb) and np.array_equal(ya, yb)
    assert b.scalars()["iteration"] == a.scalars()["iteration"] == 55
    # rejected: another bin grid, a damaged header, a truncated buffer
    c = R.Placement(d, (32, 64), 1.0, start_mode=1)
    with pytest.raises(R.ErpError):
        c.restore(blob)
    with pytest.raises(R.ErpError):
        b.restore(b"XX" + blob[2:])
    with pytest.raises(R.ErpError):
        b.restore(blob[: len(blob) // 2])
    for p in (a, b, c):
        p.close()
