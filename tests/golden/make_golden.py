"""Generate the golden fixtures that pin the oracle (run: python tests/golden/make_golden.py).

The reference's own known-answer files (tests/fft2/*, tests/density/* of the
Rust crate) are not shipped and the crate cannot be built here, so these
fixtures are computed independently of the oracle, in FP64, from closed-form
statements of what each reference function computes:

  spectral_golden.npz  DCT-II / IDCT / IDXST per axis via scipy.fft (dct type 2,
                       dct type 3, dst type 3), combined as the four 2-D
                       transforms of src/dct2d.rs, src/idct2.rs,
                       src/idct_idxst.rs, src/idxst_idct.rs, plus the full
                       Poisson solve of src/epotential.rs:284-343 with the
                       frequency weights of src/frequencies.rs.
  wa_golden.npz        analytic weighted-average wirelength gradient and HPWL
                       per net (the quantity src/hpwl.rs:139-343 evaluates).
  density_golden.npz   exact rectangle overlaps per bin with the reference's
                       bin ranges (src/density.rs:26-99, 174-237: the last bin
                       row and column receive nothing), movable cells stretched
                       to >= sqrt(2) bins with the area-preserving ratio
                       (src/epotential.rs:83-103), fixed cells x target density.
"""
import os

import numpy as np
from scipy import fft as sfft

HERE = os.path.dirname(os.path.abspath(__file__))


def dct2_axis(x, axis):          # (2/N) sum_i x[i] cos(pi k (2i+1) / 2N)
    return sfft.dct(x, type=2, axis=axis) / x.shape[axis]


def idct_axis(x, axis):          # sum_u c_u X[u] cos(pi u (2i+1) / 2N), c = (1, 2, 2, ...)
    return sfft.dct(x, type=3, axis=axis)


def idxst_axis(x, axis):         # sum_u c_u X[u] sin(pi u (2i+1) / 2N)
    x = np.moveaxis(x, axis, -1)
    shifted = np.concatenate([x[..., 1:], np.zeros_like(x[..., :1])], axis=-1)
    return np.moveaxis(sfft.dst(shifted, type=3, axis=-1), -1, axis)


def weights(m, n, bw, bh):
    wu = np.arange(m) * (2 * np.pi / m)
    wv = np.arange(n) * (2 * np.pi / n) * (bw / bh)
    s = wu[:, None] ** 2 + wv[None, :] ** 2
    s[0, 0] = 1.0
    inv = 1.0 / s
    inv[0, 0] = 0.0
    return wu[:, None] * inv * 0.5, wv[None, :] * inv * 0.5, inv


def spectral():
    rng = np.random.default_rng(2024)
    out = {}
    for (m, n) in [(16, 16), (16, 32), (64, 32)]:
        x = rng.uniform(-1, 1, (m, n))
        key = f"{m}x{n}"
        out[f"x_{key}"] = x
        out[f"dct2_{key}"] = dct2_axis(dct2_axis(x, 0), 1)
        out[f"idct2_{key}"] = idct_axis(idct_axis(x, 0), 1)
        out[f"idct_idxst_{key}"] = idxst_axis(idct_axis(x, 0), 1)
        out[f"idxst_idct_{key}"] = idct_axis(idxst_axis(x, 0), 1)
    m, n, bw, bh = 32, 64, 1.25, 0.75
    rho = rng.uniform(0.2, 1.2, (m, n))
    a = dct2_axis(dct2_axis(rho, 0), 1)
    wx, wy, inv = weights(m, n, bw, bh)
    out["poisson_rho"] = rho
    out["poisson_bins"] = np.array([bw, bh])
    out["poisson_fx"] = idct_axis(idxst_axis(a * wx, 0), 1)
    out["poisson_fy"] = idxst_axis(idct_axis(a * wy, 0), 1)
    out["poisson_psi"] = idct_axis(idct_axis(a * inv, 0), 1)
    np.savez_compressed(os.path.join(HERE, "spectral_golden.npz"), **out)


def wa():
    rng = np.random.default_rng(77)
    degs = [2, 2, 2, 3, 4, 7, 16, 33, 90]
    NM = 200
    die = 60.0
    x = rng.uniform(0, die - 5, NM).astype(np.float32)
    y = rng.uniform(0, die - 5, NM).astype(np.float32)
    w = np.full(NM, 1.0, np.float32)
    h = np.full(NM, 2.0, np.float32)
    pin_inst, pox, poy, nets = [], [], [], []
    for d in degs:
        cells = rng.choice(NM, d, replace=False)
        net = []
        for c in cells:
            pin_inst.append(int(c))
            pox.append(np.float32(rng.uniform(0, 1)))
            poy.append(np.float32(rng.uniform(0, 2)))
            net.append(len(pin_inst) - 1)
        nets.append(net)
    pin_inst = np.array(pin_inst, np.int32)
    pox = np.array(pox, np.float32)
    poy = np.array(poy, np.float32)
    px = x[pin_inst].astype(np.float64) + pox
    py = y[pin_inst].astype(np.float64) + poy
    res = {}
    for gamma in (0.7, 3.0, 20.0):
        gx = np.zeros(len(pin_inst))
        gy = np.zeros(len(pin_inst))
        hp = []
        for net in nets:
            for coord, g in ((px, gx), (py, gy)):
                v = coord[net]
                ep = np.exp((v - v.max()) / gamma)
                en = np.exp((v.min() - v) / gamma)
                wp = (v * ep).sum() / ep.sum()
                wn = (v * en).sum() / en.sum()
                g[net] = ep / ep.sum() * (1 + (v - wp) / gamma) - en / en.sum() * (1 - (v - wn) / gamma)
            hp.append(np.ptp(px[net]) + np.ptp(py[net]))
        res[f"grad_x_{gamma}"] = gx
        res[f"grad_y_{gamma}"] = gy
        res[f"hpwl_{gamma}"] = np.array(hp)
    net_ptr = np.concatenate([[0], np.cumsum([len(n_) for n_ in nets])]).astype(np.int32)
    np.savez_compressed(os.path.join(HERE, "wa_golden.npz"), x=x, y=y, w=w, h=h,
                        pin_inst=pin_inst, pin_ox=pox, pin_oy=poy, net_ptr=net_ptr,
                        net_pins=np.concatenate(nets).astype(np.int32), die=np.array([die, die]),
                        n_2nets=np.array([3]), gammas=np.array([0.7, 3.0, 20.0]), **res)


def overlap(lo, s, blo, bhi):
    return np.maximum(0.0, np.minimum(lo + s, bhi) - np.maximum(lo, blo))


def density():
    rng = np.random.default_rng(5)
    m, n = 16, 16
    die_w, die_h = 32.0, 24.0
    bw, bh = die_w / m, die_h / n
    NM = 60
    w = (rng.integers(1, 8, NM) * 0.5).astype(np.float32)
    h = np.full(NM, 1.5, np.float32)
    x = rng.uniform(0, die_w - w - 1).astype(np.float32)
    y = rng.uniform(0, die_h - h - 1).astype(np.float32)
    x[:3] = [0.0, die_w - w[1] - 1, 13.0]
    y[:3] = [0.0, die_h - h[1] - 1, 11.5]
    fx_ = np.array([4.0, 20.0], np.float32)
    fy_ = np.array([15.0, 3.0], np.float32)
    fw = np.array([6.0, 9.5], np.float32)
    fh = np.array([5.0, 4.0], np.float32)
    td = 0.9
    sq2 = np.float64(np.float32(np.sqrt(2.0)))
    cw = np.maximum(w.astype(np.float64), bw * sq2)
    ch = np.maximum(h.astype(np.float64), bh * sq2)
    ratio = w.astype(np.float64) * h / (cw * ch)
    ox = x + (w - cw) / 2
    oy = y + (h - ch) / 2
    rho = np.zeros((m, n))
    # movable: bins [floor, min(ceil+1, m-1)), clamped at 0
    for i in range(NM):
        xl = max(int(np.floor(ox[i] / bw)), 0)
        xh = min(int(np.ceil((ox[i] + cw[i]) / bw)) + 1, m - 1)
        yl = max(int(np.floor(oy[i] / bh)), 0)
        yh = min(int(np.ceil((oy[i] + ch[i]) / bh)) + 1, n - 1)
        for bx in range(xl, xh):
            px = overlap(ox[i], cw[i], bx * bw, (bx + 1) * bw)
            for by in range(yl, yh):
                rho[bx, by] += ratio[i] * px * overlap(oy[i], ch[i], by * bh, (by + 1) * bh)
    init = np.zeros((m, n))
    for i in range(len(fx_)):
        xl = max(int(np.floor(fx_[i] / bw)), 0)
        xh = min(int(np.ceil((fx_[i] + fw[i]) / bw)) + 1, m - 1)
        yl = max(int(np.floor(fy_[i] / bh)), 0)
        yh = min(int(np.ceil((fy_[i] + fh[i]) / bh)) + 1, n - 1)
        for bx in range(xl, xh):
            px = overlap(fx_[i], fw[i], bx * bw, (bx + 1) * bw)
            for by in range(yl, yh):
                init[bx, by] += px * overlap(fy_[i], fh[i], by * bh, (by + 1) * bh)
    init *= td
    dens = rho + init
    ovf = np.maximum(dens - td * bw * bh, 0).sum() / float(np.sum(w.astype(np.float64) * h))
    np.savez_compressed(os.path.join(HERE, "density_golden.npz"), x=x, y=y, w=w, h=h, fx=fx_, fy=fy_,
                        fw=fw, fh=fh, die=np.array([die_w, die_h]), bins=np.array([m, n]),
                        td=np.array([td]), initial=init, density_scaled=dens / (bw * bh),
                        overflow=np.array([ovf]))


if __name__ == "__main__":
    spectral()
    wa()
    density()
    print("fixtures written to", HERE)
