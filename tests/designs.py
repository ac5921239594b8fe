"""Test designs: a hand-built edge-case netlist and seeded synthetic ones."""
import numpy as np

from reda_erplacer_gb300.design import Design, synth


def build_design(x, y, w, h, num_movable, nets, pin_inst, pin_ox, pin_oy, die_w, die_h,
                 n_2nets, target_util=None, shuffle_pins_seed=None):
    """Assemble a Design from per-pin arrays and nets (lists of pin ids).  Optionally
    renumber the pins randomly so that the library's internal pin order differs
    from the caller's."""
    P = len(pin_inst)
    pin_inst = np.asarray(pin_inst, np.int32)
    pin_ox = np.asarray(pin_ox, np.float32)
    pin_oy = np.asarray(pin_oy, np.float32)
    if shuffle_pins_seed is not None:
        perm = np.random.default_rng(shuffle_pins_seed).permutation(P)   # new id of old pin
        inv = np.empty(P, np.int64)
        inv[perm] = np.arange(P)
        pin_inst, pin_ox, pin_oy = pin_inst[inv], pin_ox[inv], pin_oy[inv]
        nets = [[int(perm[p]) for p in net] for net in nets]
    N = len(x)
    net_ptr = np.zeros(len(nets) + 1, np.int32)
    for e, net in enumerate(nets):
        net_ptr[e + 1] = net_ptr[e] + len(net)
    net_pins = np.array([p for net in nets for p in net], np.int32)
    counts = np.bincount(pin_inst, minlength=N)
    inst_ptr = np.zeros(N + 1, np.int32)
    inst_ptr[1:] = np.cumsum(counts)
    inst_pins = np.argsort(pin_inst, kind="stable").astype(np.int32)
    w = np.asarray(w, np.float32)
    h = np.asarray(h, np.float32)
    mov_area = float(np.sum(w[:num_movable].astype(np.float64) * h[:num_movable]))
    fixed_area = float(np.sum(w[num_movable:].astype(np.float64) * h[num_movable:]))
    util = mov_area / (die_w * die_h - fixed_area) if target_util is None else target_util
    return Design(num_nodes=N, num_movable=num_movable, num_pins=P, num_nets=len(nets),
                  n_2nets=n_2nets, x=np.asarray(x, np.float32), y=np.asarray(y, np.float32), w=w, h=h,
                  num_pins_f=counts.astype(np.float32), pin_ox=pin_ox, pin_oy=pin_oy,
                  pin_inst=pin_inst, net_ptr=net_ptr, net_pins=net_pins, inst_pin_ptr=inst_ptr,
                  inst_pins=inst_pins, die_w=float(die_w), die_h=float(die_h),
                  cell_utilization=float(util), movable_area=mov_area)


def edge_design(seed=7):
    """Non-square die, movable cells touching every die edge, cells without pins,
    two macros, zero-size IO pins on the boundary (including the far corner),
    nets of degree 1, 2 (fast path and general path), 3..128, unconnected pins and
    a shuffled pin numbering."""
    rng = np.random.default_rng(seed)
    die_w, die_h = 100.0, 80.0
    NM = 320
    w = (rng.integers(2, 17, NM) * 0.2).astype(np.float32)
    h = np.full(NM, 2.0, np.float32)
    x = rng.uniform(0, die_w - w - 1).astype(np.float32)
    y = rng.uniform(0, die_h - h - 1).astype(np.float32)
    x[:4] = [0.0, die_w - w[1] - 1, 0.0, die_w - w[3] - 1]
    y[:4] = [0.0, 0.0, die_h - h[2] - 1, die_h - h[3] - 1]
    mx, my, mw, mh = [10.0, 60.0], [10.0, 40.0], [20.0, 25.0], [15.0, 30.0]
    io = [(0.0, 0.0), (die_w, die_h), (die_w, 13.0), (50.0, die_h), (0.0, 33.3)] + \
         [(float(t), 0.0) for t in np.linspace(5, 95, 15)]
    X = np.concatenate([x, mx, [p[0] for p in io]]).astype(np.float32)
    Y = np.concatenate([y, my, [p[1] for p in io]]).astype(np.float32)
    W = np.concatenate([w, mw, np.zeros(len(io))]).astype(np.float32)
    H = np.concatenate([h, mh, np.zeros(len(io))]).astype(np.float32)
    N = len(X)
    pin_inst, pin_ox, pin_oy = [], [], []

    def add_pin(inst):
        pin_inst.append(inst)
        pin_ox.append(float(rng.uniform(0, W[inst])) if W[inst] > 0 else 0.0)
        pin_oy.append(float(rng.uniform(0, H[inst])) if H[inst] > 0 else 0.0)
        return len(pin_inst) - 1

    nopin = set(range(300, 310))     # movable cells without pins
    pool = [i for i in range(NM) if i not in nopin]
    nets = []
    for _ in range(40):
        a, b = rng.choice(pool, 2, replace=False)
        nets.append([add_pin(int(a)), add_pin(int(b))])
    n_2nets = len(nets)
    degs = [1, 1, 1, 2, 2] + [3] * 20 + [4] * 10 + list(rng.integers(5, 9, 10)) + \
        list(rng.integers(9, 17, 8)) + list(rng.integers(17, 33, 5)) + [33, 33, 64, 128]
    for dg in degs:
        cells = rng.choice(pool, int(dg), replace=False)
        nets.append([add_pin(int(c)) for c in cells])
    for k in range(len(io)):          # IO pins join nets
        nets[n_2nets + 5 + k].append(add_pin(NM + 2 + k))
    for k in range(2):                # macro pins
        nets[n_2nets + 30 + k].append(add_pin(NM + k))
    for c in rng.choice(pool, 10, replace=False):   # unconnected pins
        add_pin(int(c))
    return build_design(X, Y, W, H, NM, nets, pin_inst, pin_ox, pin_oy, die_w, die_h, n_2nets,
                        shuffle_pins_seed=seed + 1)


def spread_positions(d, seed=3, frac=1.0):
    """Uniformly spread movable cells over the die (fixed cells unchanged)."""
    rng = np.random.default_rng(seed)
    x = d.x.copy()
    y = d.y.copy()
    NM = d.num_movable
    cx, cy = d.die_w / 2, d.die_h / 2
    ux = rng.uniform(0, d.die_w - d.w[:NM] - 1)
    uy = rng.uniform(0, d.die_h - d.h[:NM] - 1)
    x[:NM] = (cx + frac * (ux - cx)).astype(np.float32)
    y[:NM] = (cy + frac * (uy - cy)).astype(np.float32)
    return x, y


def small_synth(cells=3000, seed=11, macros=2, io=60, util=0.7):
    return synth(cells, int(round(1.05 * cells)), num_io=io, num_macros=macros, utilization=util,
                 seed=seed)
