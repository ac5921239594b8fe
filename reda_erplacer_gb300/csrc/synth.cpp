// Seeded synthetic netlist generator: the input source of the workloads in
// place of reda-db's read_db on ISPD LEF/DEF files (not shipped).  It produces
// the same database view the placement loop reads (include/erplacer.h:
// erp_design): movable standard cells first, then fixed macros, then fixed
// zero-size IO pins on the die boundary; nets with exactly two pins first.
//
// Generation rule (documented so that every consumer builds the same design):
//  * cells: one row high (row_h), width = uniform integer in [min_sites,
//    max_sites] times site_w;
//  * nets: degree classes by exact share — 2 pins 55 %, 3 pins 20 %, 4-8 pins
//    18 %, 9-32 pins 6 %, 33-128 pins 1 % (uniform inside a class, capped at the
//    cell count); pins sit on distinct, uniformly drawn movable cells with
//    offsets uniform inside the cell;
//  * IO pins: evenly spaced along the die perimeter, each joined to a random
//    net of three or more pins (so the two-pin share is kept);
//  * macros: each macro_area_frac of the die, aspect ratio uniform 0.5-2,
//    positions uniform without overlap (rejection sampling);
//  * die: square, area = cell area / (utilization * (1 - macro share)), its
//    side at least the largest cell width or height;
//  * start: die centre minus half the cell size plus Gaussian jitter
//    (sigma = jitter_frac * die width), clamped onto the die.
// Randomness: xoshiro256** seeded through splitmix64; only integer ops and
// IEEE double arithmetic, so x86 and Arm hosts produce the same design.
#include "erplacer.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

namespace {

struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t &x) {
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    explicit Rng(uint64_t seed) {
        for (auto &v : s) v = splitmix(seed);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    }
    // uniform double in [0, 1)
    double uni() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    // uniform integer in [lo, hi]
    int64_t range(int64_t lo, int64_t hi) {
        uint64_t span = (uint64_t)(hi - lo) + 1;
        unsigned __int128 m = (unsigned __int128)next() * span;
        return lo + (int64_t)(uint64_t)(m >> 64);
    }
    double normal() {
        double u1 = uni(), u2 = uni();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

}  // namespace

struct erp_synth {
    std::vector<float> x, y, w, h, npins, pox, poy;
    std::vector<int32_t> pin_inst, net_ptr, net_pins, inst_ptr, inst_pins;
    int32_t num_nodes = 0, num_movable = 0, num_pins = 0, num_nets = 0, n_2nets = 0;
    float die_w = 0, die_h = 0, util = 0, mov_area = 0;
};

namespace {
bool positive(float v) { return v > 0.0f && std::isfinite(v); }   // false for NaN
}  // namespace

static erp_status synth_fill(const erp_synth_params *p, erp_synth *s);

extern "C" erp_status erp_synth_create(const erp_synth_params *p, erp_synth **out) {
    if (!p || !out || p->num_cells < 2 || p->num_nets < 1 || p->num_io < 0 || p->num_macros < 0 ||
        !positive(p->utilization) || !positive(p->site_w) || !positive(p->row_h) || p->min_sites < 1 ||
        p->max_sites < p->min_sites || !(p->macro_area_frac >= 0.0f) || !std::isfinite(p->macro_area_frac) ||
        !std::isfinite(p->jitter_frac) || p->num_macros * (double)p->macro_area_frac >= 0.9)
        return ERP_EINVAL;
    // node ids are int32 in erp_design
    if ((int64_t)p->num_cells + p->num_macros + p->num_io >= INT32_MAX) return ERP_EINVAL;
    erp_synth *s = new (std::nothrow) erp_synth();
    if (!s) return ERP_ENOMEM;
    erp_status st;
    try {
        st = synth_fill(p, s);
    } catch (const std::bad_alloc &) {
        st = ERP_ENOMEM;
    }
    if (st != ERP_OK) {
        delete s;
        return st;
    }
    *out = s;
    return ERP_OK;
}

static erp_status synth_fill(const erp_synth_params *p, erp_synth *s) {
    Rng rng((uint64_t)p->seed);
    const int NC = p->num_cells, NMAC = p->num_macros, NIO = p->num_io, E = p->num_nets;
    const int N = NC + NMAC + NIO;
    s->num_nodes = N;
    s->num_movable = NC;
    s->x.assign(N, 0.f); s->y.assign(N, 0.f); s->w.assign(N, 0.f); s->h.assign(N, 0.f);
    s->npins.assign(N, 0.f);
    double cell_area = 0;
    for (int i = 0; i < NC; ++i) {
        int sites = (int)rng.range(p->min_sites, p->max_sites);
        s->w[i] = (float)(sites * (double)p->site_w);
        s->h[i] = p->row_h;
        cell_area += (double)s->w[i] * (double)s->h[i];
    }
    double macro_share = NMAC * (double)p->macro_area_frac;
    double die_area = cell_area / ((double)p->utilization * (1.0 - macro_share));
    double side = std::sqrt(die_area);
    double max_dim = 0;   // a die narrower than a cell is unplaceable (only tiny designs reach this)
    for (int i = 0; i < NC; ++i) max_dim = std::max(max_dim, (double)std::max(s->w[i], s->h[i]));
    if (side < max_dim) {
        side = max_dim;
        die_area = side * side;
    }
    s->die_w = s->die_h = (float)side;
    // macros
    std::vector<double> mx, my, mw, mh;
    for (int k = 0; k < NMAC; ++k) {
        double A = die_area * p->macro_area_frac;
        double a = 0.5 + 1.5 * rng.uni();
        double ww = std::sqrt(A * a), hh = std::sqrt(A / a);
        ww = std::min(ww, side * 0.95);
        hh = std::min(hh, side * 0.95);
        double px = 0, py = 0;
        for (int tries = 0; tries < 10000; ++tries) {
            px = rng.uni() * (side - ww);
            py = rng.uni() * (side - hh);
            bool ok = true;
            for (size_t j = 0; j < mx.size() && ok; ++j)
                ok = px + ww <= mx[j] || mx[j] + mw[j] <= px || py + hh <= my[j] || my[j] + mh[j] <= py;
            if (ok) break;
        }
        mx.push_back(px); my.push_back(py); mw.push_back(ww); mh.push_back(hh);
        int id = NC + k;
        s->x[id] = (float)px; s->y[id] = (float)py; s->w[id] = (float)ww; s->h[id] = (float)hh;
    }
    double macro_area = 0;
    for (int k = 0; k < NMAC; ++k) macro_area += (double)s->w[NC + k] * (double)s->h[NC + k];
    // IO pins on the perimeter
    for (int k = 0; k < NIO; ++k) {
        double t = (k + 0.5) * 4.0 * side / NIO, px, py;
        if (t < side) { px = t; py = 0; }
        else if (t < 2 * side) { px = side; py = t - side; }
        else if (t < 3 * side) { px = 3 * side - t; py = side; }
        else { px = 0; py = 4 * side - t; }
        s->x[NC + NMAC + k] = (float)px;
        s->y[NC + NMAC + k] = (float)py;
    }
    // movable start: centre + jitter
    double sigma = p->jitter_frac * side;
    for (int i = 0; i < NC; ++i) {
        double px = side / 2 - s->w[i] / 2.0 + sigma * rng.normal();
        double py = side / 2 - s->h[i] / 2.0 + sigma * rng.normal();
        px = std::min(std::max(px, 0.0), side - s->w[i]);
        py = std::min(std::max(py, 0.0), side - s->h[i]);
        s->x[i] = (float)px; s->y[i] = (float)py;
    }
    // net degrees by exact class share
    const double share[5] = {0.55, 0.20, 0.18, 0.06, 0.01};
    const int lo[5] = {2, 3, 4, 9, 33}, hi[5] = {2, 3, 8, 32, 128};
    std::vector<int> cnt(5);
    int assigned = 0;
    for (int c = 0; c < 5; ++c) { cnt[c] = (int)std::floor(share[c] * E + 0.5); assigned += cnt[c]; }
    cnt[0] += E - assigned;  // rounding remainder goes to the two-pin class
    if (cnt[0] < 0) { cnt[1] += cnt[0]; cnt[0] = 0; }
    std::vector<int> deg;
    deg.reserve(E);
    for (int c = 0; c < 5; ++c)
        for (int k = 0; k < cnt[c]; ++k) {
            int d = (int)rng.range(lo[c], hi[c]);
            deg.push_back(std::min(d, NC));
        }
    // IO attachments
    std::vector<int> extra(E, 0), big;
    for (int e = 0; e < E; ++e)
        if (deg[e] >= 3) big.push_back(e);
    std::vector<int> io_net(NIO, -1);
    if (!big.empty())
        for (int k = 0; k < NIO; ++k) { io_net[k] = big[(size_t)rng.range(0, (int64_t)big.size() - 1)]; extra[io_net[k]]++; }
    // build nets: two-pin nets are exactly the first cnt[0] (classes are emitted in order)
    s->num_nets = E;
    s->n_2nets = 0;
    for (int e = 0; e < E && deg[e] == 2 && extra[e] == 0; ++e) s->n_2nets++;
    int64_t P64 = 0;   // pin ids are int32 in erp_design
    for (int e = 0; e < E; ++e) P64 += deg[e] + extra[e];
    if (P64 >= INT32_MAX) return ERP_EINVAL;
    s->net_ptr.assign(E + 1, 0);
    for (int e = 0; e < E; ++e) s->net_ptr[e + 1] = s->net_ptr[e] + deg[e] + extra[e];
    const int P = s->net_ptr[E];
    s->num_pins = P;
    s->net_pins.resize(P);
    s->pin_inst.resize(P);
    s->pox.resize(P);
    s->poy.resize(P);
    std::vector<int> io_fill(E, 0);
    std::vector<int32_t> pick;
    for (int e = 0; e < E; ++e) {
        int base = s->net_ptr[e], d = deg[e];
        pick.clear();
        while ((int)pick.size() < d) {
            int c = (int)rng.range(0, NC - 1);
            if (std::find(pick.begin(), pick.end(), c) == pick.end()) pick.push_back(c);
        }
        for (int k = 0; k < d; ++k) {
            int pid = base + k, c = pick[k];
            s->net_pins[pid] = pid;
            s->pin_inst[pid] = c;
            s->pox[pid] = (float)(rng.uni() * s->w[c]);
            s->poy[pid] = (float)(rng.uni() * s->h[c]);
        }
    }
    for (int k = 0; k < NIO; ++k) {
        int e = io_net[k];
        if (e < 0) continue;
        int pid = s->net_ptr[e] + deg[e] + io_fill[e]++;
        s->net_pins[pid] = pid;
        s->pin_inst[pid] = NC + NMAC + k;
        s->pox[pid] = 0.f;
        s->poy[pid] = 0.f;
    }
    // per-instance pin lists (macro_2_pins), ascending pin id
    s->inst_ptr.assign(N + 1, 0);
    for (int pid = 0; pid < P; ++pid) s->inst_ptr[s->pin_inst[pid] + 1]++;
    for (int i = 0; i < N; ++i) s->inst_ptr[i + 1] += s->inst_ptr[i];
    s->inst_pins.resize(P);
    std::vector<int32_t> fill(s->inst_ptr.begin(), s->inst_ptr.end() - 1);
    for (int pid = 0; pid < P; ++pid) s->inst_pins[fill[s->pin_inst[pid]]++] = pid;
    for (int i = 0; i < N; ++i) s->npins[i] = (float)(s->inst_ptr[i + 1] - s->inst_ptr[i]);
    s->mov_area = (float)cell_area;
    s->util = (float)(cell_area / (die_area - macro_area));
    return ERP_OK;
}

extern "C" erp_status erp_synth_design(const erp_synth *s, erp_design *d) {
    if (!s || !d) return ERP_EINVAL;
    std::memset(d, 0, sizeof(*d));
    d->num_nodes = s->num_nodes;
    d->num_movable = s->num_movable;
    d->num_pins = s->num_pins;
    d->num_nets = s->num_nets;
    d->n_2nets = s->n_2nets;
    d->x = s->x.data(); d->y = s->y.data(); d->w = s->w.data(); d->h = s->h.data();
    d->num_pins_f = s->npins.data();
    d->pin_ox = s->pox.data(); d->pin_oy = s->poy.data();
    d->pin_inst = s->pin_inst.data();
    d->net_ptr = s->net_ptr.data(); d->net_pins = s->net_pins.data();
    d->inst_pin_ptr = s->inst_ptr.data(); d->inst_pins = s->inst_pins.data();
    d->die_w = s->die_w; d->die_h = s->die_h;
    d->cell_utilization = s->util;
    d->movable_area = s->mov_area;
    return ERP_OK;
}

extern "C" void erp_synth_destroy(erp_synth *s) { delete s; }
