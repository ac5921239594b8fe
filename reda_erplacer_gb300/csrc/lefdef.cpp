// LEF/DEF ingest, export and the placed-DEF hand-off: the stand-in for
// reda-db's read_db (src/main.rs:69) and the step after the loop that the
// reference leaves out (README.md:23, global placement only).
//
// Database semantics (reda-db is not shipped; restated from its use sites in
// src/placement.rs, src/hpwl.rs, src/nesterov.rs, src/epotential.rs):
//  * instances: movable components (not FIXED / COVER) first, in DEF order,
//    then fixed components, then the DEF PINS as zero-size fixed instances
//    (src/placement.rs:125);
//  * coordinates in microns, the die moved to the origin (src/nesterov.rs:131);
//    (x, y) is the lower-left corner of the placed, oriented footprint; the
//    footprint is the LEF SIZE with width and height swapped for E, W, FE, FW;
//  * a pin's offset is the centre of the bounding box of all its LEF port
//    shapes (RECT, POLYGON, PATH, VIA points), shifted by the macro ORIGIN and
//    carried through the component orientation, measured from the footprint's
//    lower-left corner (src/hpwl.rs:107); a pin with no shapes sits at the
//    macro centre; a DEF PIN's offset is the centre of its first LAYER / POLYGON
//    shape, rotated about its placement point;
//  * nets: every NETS entry with at least one connection, the nets of exactly
//    two pins first (stable), the rest in DEF order (src/hpwl.rs:159,173);
//    pin ids run net-major; wildcard "( * pin )" connections and MUSTJOIN
//    entries are skipped (counted in the statistics);
//  * num_pins_f: pins per instance; inst_pins ascending pin id (macro_2_pins);
//  * movable_area = sum of movable footprints; cell_utilization = movable_area /
//    (die area - fixed component area inside the die) (src/placement.rs:134,
//    src/epotential.rs:277).
// LEF geometry is snapped to the LEF database grid (UNITS DATABASE MICRONS, or
// the DEF's when the LEF has none) and kept as integers; the conversion to
// float happens once, in double, so x86 and Arm hosts build identical designs.
#include "erplacer.h"

#include <algorithm>
#include <cstdarg>
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <string_view>
#include <unordered_map>
#include <vector>

namespace {

thread_local std::string g_err;

struct Fail : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// Every coordinate and size in database units (DEF units, LEF grid units) is
// limited to |v| <= 2^40 (about 1.1e12 units, far beyond any die), so sums and
// differences of a few of them never overflow int64.
constexpr double kMaxUnits = 1099511627776.0;

// Open-addressing table from names to the indices of their owners (macros,
// macro pins, components, DEF pins).  It keeps only each key's hash and its
// owner's index and compares against the owner's name, so the owners'
// containers may reallocate.  insert keeps an existing entry (like emplace).
class NameTable {
  public:
    template <class NameOf>
    int find(std::string_view key, const NameOf &name_of) const {
        if (count_ == 0) return -1;
        const uint64_t h = hash(key);
        for (size_t s = h & mask_;; s = (s + 1) & mask_) {
            const int32_t i = idx_[s];
            if (i < 0) return -1;
            if (hash_[s] == h && name_of(i) == key) return i;
        }
    }
    template <class NameOf>
    bool insert(std::string_view key, int32_t owner, const NameOf &name_of) {
        if ((count_ + 1) * 2 > idx_.size()) grow();
        const uint64_t h = hash(key);
        for (size_t s = h & mask_;; s = (s + 1) & mask_) {
            const int32_t i = idx_[s];
            if (i < 0) {
                idx_[s] = owner;
                hash_[s] = h;
                ++count_;
                return true;
            }
            if (hash_[s] == h && name_of(i) == key) return false;
        }
    }
    bool empty() const { return count_ == 0; }

  private:
    static uint64_t hash(std::string_view k) {   // FNV-1a, then a 64-bit finaliser to spread the low bits
        uint64_t h = 1469598103934665603ull;
        for (unsigned char c : k) {
            h ^= c;
            h *= 1099511628211ull;
        }
        h ^= h >> 33;
        h *= 0xff51afd7ed558ccdull;
        h ^= h >> 33;
        return h;
    }
    void grow() {
        const size_t cap = idx_.empty() ? 64 : idx_.size() * 2;
        std::vector<int32_t> idx(cap, -1);
        std::vector<uint64_t> hs(cap, 0);
        for (size_t s = 0; s < idx_.size(); ++s) {
            if (idx_[s] < 0) continue;
            size_t t = hash_[s] & (cap - 1);
            while (idx[t] >= 0) t = (t + 1) & (cap - 1);
            idx[t] = idx_[s];
            hs[t] = hash_[s];
        }
        idx_.swap(idx);
        hash_.swap(hs);
        mask_ = cap - 1;
    }
    std::vector<int32_t> idx_;
    std::vector<uint64_t> hash_;
    size_t mask_ = 0, count_ = 0;
};

// llround(v) for a quantity in database units, or Fail.
int64_t to_units(double v, const char *what) {
    if (!std::isfinite(v) || std::fabs(v) > kMaxUnits) throw Fail(std::string(what) + " out of range");
    return (int64_t)std::llround(v);
}

enum Kind : uint8_t { kMovable = 0, kFixed = 1, kIo = 2 };
enum Orient : uint8_t { oN = 0, oW, oS, oE, oFN, oFW, oFS, oFE };
const char *const kOrientName[8] = {"N", "W", "S", "E", "FN", "FW", "FS", "FE"};

int orient_of(std::string_view t) {
    for (int o = 0; o < 8; ++o)
        if (t == kOrientName[o]) return o;
    return -1;
}
bool swaps(int o) { return o == oW || o == oE || o == oFW || o == oFE; }

// A point of a w x h footprint after orientation o, measured from the oriented
// footprint's lower-left corner (DEF component semantics).
void orient_in_box(int o, int64_t px, int64_t py, int64_t w, int64_t h, int64_t &qx, int64_t &qy) {
    switch (o) {
        default:
        case oN: qx = px; qy = py; break;
        case oS: qx = w - px; qy = h - py; break;
        case oW: qx = h - py; qy = px; break;
        case oE: qx = py; qy = w - px; break;
        case oFN: qx = w - px; qy = py; break;
        case oFS: qx = px; qy = h - py; break;
        case oFW: qx = py; qy = px; break;
        case oFE: qx = h - py; qy = w - px; break;
    }
}
// A point rotated about the placement point (DEF PINS shape semantics).
void orient_at_point(int o, int64_t px, int64_t py, int64_t &qx, int64_t &qy) {
    switch (o) {
        default:
        case oN: qx = px; qy = py; break;
        case oS: qx = -px; qy = -py; break;
        case oW: qx = -py; qy = px; break;
        case oE: qx = py; qy = -px; break;
        case oFN: qx = -px; qy = py; break;
        case oFS: qx = px; qy = -py; break;
        case oFW: qx = py; qy = px; break;
        case oFE: qx = -py; qy = -px; break;
    }
}

struct MacroPin {
    std::string name;
    double lx = 0, ly = 0, hx = 0, hy = 0;   // bbox of the shapes, microns, before ORIGIN
    bool has = false;
    int64_t c2x = 0, c2y = 0;                 // twice the centre, LEF grid units, after ORIGIN
    void add(double x, double y) {
        if (!has) { lx = hx = x; ly = hy = y; has = true; return; }
        lx = std::min(lx, x); hx = std::max(hx, x);
        ly = std::min(ly, y); hy = std::max(hy, y);
    }
};

struct Macro {
    std::string name;
    bool block = false;
    double w = 0, h = 0, ox = 0, oy = 0;      // microns
    int64_t W = 0, H = 0;                     // LEF grid units
    std::vector<MacroPin> pins;
    NameTable index;   // built when there are many pins; the first of equal names wins
    std::string_view pin_name(int k) const { return pins[k].name; }
    void index_pin(int k) {
        index.insert(pins[k].name, k, [this](int j) { return pin_name(j); });
    }
    int find_pin(std::string_view n) const {
        if (!index.empty()) return index.find(n, [this](int j) { return pin_name(j); });
        for (size_t k = 0; k < pins.size(); ++k)
            if (pins[k].name == n) return (int)k;
        return -1;
    }
};

struct Node {
    std::string name;
    uint8_t kind = kMovable;
    uint8_t orient = oN;
    bool placed = false;                      // has a PLACED / FIXED / COVER location
    int32_t master = -1;                      // macro (components)
    int64_t X = 0, Y = 0;                     // DEF units, absolute
    int64_t rlx = 0, rly = 0, rhx = 0, rhy = 0;   // DEF PIN shape (DEF units, unrotated)
    std::string status = "PLACED";            // DEF PIN placement keyword
    std::string net;                          // DEF PIN "+ NET" name
    size_t clause_off = 0, clause_len = 0;    // source bytes of the component's placement clause
    bool clause_insert = false;               // no clause: insert before clause_off (the ';')
};

struct Conn {
    int32_t node;   // parse-order node (components, then DEF PINS)
    int32_t pin;    // macro pin, -1 for a DEF PIN
};

}  // namespace

struct erp_netlist {
    std::string design_name = "design";
    int64_t lef_dbu = 0, def_dbu = 0, grid = 0;
    int64_t die[4] = {0, 0, 0, 0};
    bool have_die = false;
    std::vector<Macro> macros;
    NameTable macro_index;
    int32_t num_components = 0;
    std::vector<Node> nodes;                   // parse order
    std::vector<std::string> net_names;        // kept nets, in DEF order
    std::vector<int32_t> net_begin{0};
    std::vector<Conn> conns;
    std::string def_text;                      // the source DEF (placed-DEF splice)
    bool from_design = false;
    std::string site_name = "core";
    double site_w = 0, row_h = 0;
    erp_lefdef_stats st{};
    // erp_design view
    std::vector<int32_t> order;                // design index -> parse-order node
    std::vector<int32_t> net_order;            // design net -> kept net
    std::vector<float> x, y, w, h, npins, pox, poy;
    std::vector<int32_t> pin_inst, net_ptr, net_pins, inst_ptr, inst_pins;
    int32_t num_movable = 0, n_2nets = 0;
    float die_w = 0, die_h = 0, util = 0, mov_area = 0;
};

namespace {

bool read_file(const char *path, std::string &out) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    out.clear();
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, n);
    const bool ok = !std::ferror(f);
    std::fclose(f);
    return ok;
}

// Whitespace-separated tokens; "quoted strings" are one token; '#' at the start
// of a token comments out the rest of the line.
struct Lex {
    const char *b, *p, *e;
    std::string file;
    int line = 1;
    std::string_view t;
    size_t off = 0;
    int tline = 1;

    Lex(const std::string &text, const char *name) : b(text.data()), p(text.data()), e(text.data() + text.size()), file(name) {}

    bool next() {
        for (;;) {
            while (p < e && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n' || *p == '\f' || *p == '\v')) {
                if (*p == '\n') ++line;
                ++p;
            }
            if (p >= e) {
                t = {};
                return false;
            }
            if (*p == '#') {
                while (p < e && *p != '\n') ++p;
                continue;
            }
            break;
        }
        const char *s = p;
        tline = line;
        if (*p == '"') {
            ++p;
            while (p < e && *p != '"') {
                if (*p == '\n') ++line;
                ++p;
            }
            if (p < e) ++p;
        } else {
            while (p < e && !(*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n' || *p == '\f' || *p == '\v')) ++p;
        }
        t = std::string_view(s, (size_t)(p - s));
        off = (size_t)(s - b);
        return true;
    }
    [[noreturn]] void fail(const std::string &msg) const {
        throw Fail(file + ":" + std::to_string(tline) + ": " + msg);
    }
    std::string_view need() {
        if (!next()) fail("unexpected end of file");
        return t;
    }
    void expect(std::string_view want) {
        need();
        if (t != want) fail("expected '" + std::string(want) + "', found '" + std::string(t) + "'");
    }
    double num() {
        need();
        return as_num();
    }
    double as_num() const {
        double v = 0;
        const char *s = t.data(), *end = t.data() + t.size();
        if (s < end && *s == '+') ++s;
        auto r = std::from_chars(s, end, v);
        if (r.ec != std::errc() || r.ptr != end) fail("expected a number, found '" + std::string(t) + "'");
        return v;
    }
    bool is_num() const {
        double v;
        const char *s = t.data(), *end = t.data() + t.size();
        if (s < end && *s == '+') ++s;
        auto r = std::from_chars(s, end, v);
        return r.ec == std::errc() && r.ptr == end && s < end;
    }
    int64_t inum() {
        const double v = num();
        if (!std::isfinite(v) || std::fabs(v) > kMaxUnits) fail("number out of range");
        return (int64_t)std::llround(v);
    }
    void skip_statement() {   // to the next ';' token (inclusive)
        while (t != ";") need();
    }
    void skip_to_end(std::string_view name) {   // to "END name" (inclusive)
        for (;;) {
            need();
            if (t == "END") {
                need();
                if (t == name) return;
            }
        }
    }
    void skip_to(std::string_view word) {
        do need();
        while (t != word);
    }
};

// ---------------------------------------------------------------- LEF

void lef_port(Lex &L, MacroPin &pin) {
    for (;;) {
        L.need();
        if (L.t == "END") return;
        if (L.t == "RECT") {
            double v[4];
            int k = 0;
            for (;;) {
                L.need();
                if (L.t == ";") break;
                if (L.t == "MASK") { L.need(); continue; }
                if (L.t == "ITERATE") { L.skip_statement(); k = -1; break; }
                if (k < 4) v[k++] = L.as_num();
                else L.fail("RECT with more than four coordinates");
            }
            if (k == 4) { pin.add(v[0], v[1]); pin.add(v[2], v[3]); }
            else if (k >= 0) L.fail("RECT needs four coordinates");
        } else if (L.t == "POLYGON" || L.t == "PATH") {
            std::vector<double> v;
            for (;;) {
                L.need();
                if (L.t == ";") break;
                if (L.t == "MASK") { L.need(); continue; }
                if (L.t == "ITERATE") { L.skip_statement(); v.clear(); break; }
                v.push_back(L.as_num());
            }
            for (size_t k = 0; k + 1 < v.size(); k += 2) pin.add(v[k], v[k + 1]);
        } else if (L.t == "VIA") {
            std::vector<double> v;
            for (;;) {
                L.need();
                if (L.t == ";") break;
                if (L.t == "ITERATE") { L.skip_statement(); v.clear(); break; }
                if (L.is_num()) v.push_back(L.as_num());
            }
            if (v.size() >= 2) pin.add(v[0], v[1]);
        } else {
            L.skip_statement();   // LAYER, WIDTH, CLASS ...
        }
    }
}

void lef_pin(Lex &L, Macro &m) {
    MacroPin pin;
    pin.name = std::string(L.need());
    for (;;) {
        L.need();
        if (L.t == "END") {
            L.need();
            if (L.t != pin.name) L.fail("expected 'END " + pin.name + "'");
            break;
        }
        if (L.t == "PORT") lef_port(L, pin);
        else L.skip_statement();
    }
    if (m.find_pin(pin.name) >= 0) L.fail("duplicate pin '" + pin.name + "' in macro '" + m.name + "'");
    m.pins.push_back(std::move(pin));
    if (m.pins.size() == 16) {
        for (size_t k = 0; k < m.pins.size(); ++k) m.index_pin((int)k);
    } else if (m.pins.size() > 16) {
        m.index_pin((int)m.pins.size() - 1);
    }
}

void lef_macro(Lex &L, erp_netlist &nl) {
    Macro m;
    m.name = std::string(L.need());
    for (;;) {
        L.need();
        if (L.t == "END") {
            L.need();
            if (L.t != m.name) L.fail("expected 'END " + m.name + "'");
            break;
        }
        if (L.t == "SIZE") {
            m.w = L.num();
            L.expect("BY");
            m.h = L.num();
            L.expect(";");
        } else if (L.t == "ORIGIN") {
            m.ox = L.num();
            m.oy = L.num();
            L.expect(";");
        } else if (L.t == "CLASS") {
            L.need();
            m.block = L.t == "BLOCK" || L.t == "RING" || L.t == "PAD" || L.t == "COVER";
            L.skip_statement();
        } else if (L.t == "PIN") {
            lef_pin(L, m);
        } else if (L.t == "OBS" || L.t == "DENSITY") {
            L.skip_to("END");
        } else {
            L.skip_statement();   // FOREIGN, SYMMETRY, SITE, PROPERTY, EEQ, SOURCE ...
        }
    }
    auto macro_name = [&](int i) -> std::string_view { return nl.macros[i].name; };
    const int prev = nl.macro_index.find(m.name, macro_name);
    if (prev >= 0) {
        nl.macros[prev] = std::move(m);   // a later definition replaces an earlier one
    } else {
        nl.macro_index.insert(m.name, (int)nl.macros.size(), macro_name);
        nl.macros.push_back(std::move(m));
    }
}

void read_lef(const std::string &text, const char *path, erp_netlist &nl) {
    Lex L(text, path);
    while (L.next()) {
        const std::string_view k = L.t;
        if (k == "MACRO") {
            lef_macro(L, nl);
        } else if (k == "UNITS") {
            for (;;) {
                L.need();
                if (L.t == "END") { L.expect("UNITS"); break; }
                if (L.t == "DATABASE") {
                    L.expect("MICRONS");
                    const int64_t v = L.inum();
                    if (v <= 0) L.fail("DATABASE MICRONS must be positive");
                    nl.lef_dbu = v;
                    L.expect(";");
                } else {
                    L.skip_statement();
                }
            }
        } else if (k == "END") {
            L.need();
            if (L.t == "LIBRARY") break;
            L.fail("unexpected 'END " + std::string(L.t) + "'");
        } else if (k == "SITE" || k == "LAYER" || k == "VIA" || k == "VIARULE" || k == "NONDEFAULTRULE" ||
                   k == "ARRAY") {
            const std::string name(L.need());
            L.skip_to_end(name);
        } else if (k == "SPACING" || k == "PROPERTYDEFINITIONS" || k == "IRDROP" || k == "NOISETABLE" ||
                   k == "CORRECTIONTABLE") {
            const std::string name(k);
            L.skip_to_end(name);
        } else if (k == "BEGINEXT") {
            L.skip_to("ENDEXT");
        } else {
            L.skip_statement();   // VERSION, BUSBITCHARS, DIVIDERCHAR, MANUFACTURINGGRID ...
        }
    }
}

// ---------------------------------------------------------------- DEF

void def_point(Lex &L, int64_t &x, int64_t &y) {
    L.expect("(");
    x = L.inum();
    y = L.inum();
    L.expect(")");
}

bool is_section(std::string_view k) {
    return k == "VIAS" || k == "SPECIALNETS" || k == "BLOCKAGES" || k == "REGIONS" || k == "GROUPS" ||
           k == "NONDEFAULTRULES" || k == "FILLS" || k == "SCANCHAINS" || k == "STYLES" || k == "SLOTS" ||
           k == "PINPROPERTIES" || k == "PROPERTYDEFINITIONS";
}

struct DefState {
    NameTable comp_index, pin_index;   // component / DEF pin name -> node index
};

void def_components(Lex &L, erp_netlist &nl, DefState &S) {
    L.need();   // count
    L.expect(";");
    for (;;) {
        L.need();
        if (L.t == "END") { L.expect("COMPONENTS"); break; }
        if (L.t != "-") L.fail("expected '-' or 'END COMPONENTS', found '" + std::string(L.t) + "'");
        Node n;
        n.name = std::string(L.need());
        const std::string_view master = L.need();
        n.master = nl.macro_index.find(master, [&](int i) -> std::string_view { return nl.macros[i].name; });
        if (n.master < 0) L.fail("component '" + n.name + "' of unknown macro '" + std::string(master) + "'");
        bool clause = false;
        for (;;) {
            L.need();
            if (L.t == ";") break;
            if (L.t != "+") continue;   // the arguments of a skipped option
            L.need();
            if (L.t == "PLACED" || L.t == "FIXED" || L.t == "COVER") {
                n.clause_off = L.off;
                n.kind = L.t == "PLACED" ? kMovable : kFixed;
                def_point(L, n.X, n.Y);
                L.need();
                const int o = orient_of(L.t);
                if (o < 0) L.fail("bad orientation '" + std::string(L.t) + "'");
                n.orient = (uint8_t)o;
                n.placed = true;
                n.clause_len = L.off + L.t.size() - n.clause_off;
                clause = true;
            } else if (L.t == "UNPLACED") {
                n.clause_off = L.off;
                n.clause_len = L.t.size();
                n.kind = kMovable;
                n.placed = false;
                clause = true;
            }
        }
        if (!clause) {
            n.clause_off = L.off;   // the ';'
            n.clause_insert = true;
        }
        if (!S.comp_index.insert(n.name, (int)nl.nodes.size(), [&](int i) -> std::string_view { return nl.nodes[i].name; }))
            L.fail("duplicate component '" + n.name + "'");
        nl.nodes.push_back(std::move(n));
    }
    nl.num_components = (int32_t)nl.nodes.size();
}

void def_pins(Lex &L, erp_netlist &nl, DefState &S) {
    L.need();
    L.expect(";");
    for (;;) {
        L.need();
        if (L.t == "END") { L.expect("PINS"); break; }
        if (L.t != "-") L.fail("expected '-' or 'END PINS', found '" + std::string(L.t) + "'");
        Node n;
        n.kind = kIo;
        n.name = std::string(L.need());
        bool have_shape = false, pending = false;
        for (;;) {
            if (!pending) L.need();
            pending = false;
            if (L.t == ";") break;
            if (L.t != "+") continue;
            L.need();
            if (L.t == "NET") {
                n.net = std::string(L.need());
            } else if (L.t == "LAYER" && !have_shape) {
                L.skip_to("(");
                n.rlx = L.inum(); n.rly = L.inum();
                L.expect(")");
                def_point(L, n.rhx, n.rhy);
                have_shape = true;
            } else if (L.t == "POLYGON" && !have_shape) {
                L.skip_to("(");
                int64_t px = L.inum(), py = L.inum();
                L.expect(")");
                n.rlx = n.rhx = px; n.rly = n.rhy = py;
                for (;;) {
                    L.need();
                    if (L.t != "(") break;
                    px = L.inum(); py = L.inum();
                    L.expect(")");
                    n.rlx = std::min(n.rlx, px); n.rhx = std::max(n.rhx, px);
                    n.rly = std::min(n.rly, py); n.rhy = std::max(n.rhy, py);
                }
                have_shape = true;
                pending = true;   // the token after the points is the next '+' or the ';'
            } else if ((L.t == "PLACED" || L.t == "FIXED" || L.t == "COVER") && !n.placed) {
                n.status = std::string(L.t);
                def_point(L, n.X, n.Y);
                L.need();
                const int o = orient_of(L.t);
                if (o < 0) L.fail("bad orientation '" + std::string(L.t) + "'");
                n.orient = (uint8_t)o;
                n.placed = true;
            }
        }
        if (!n.placed) nl.st.num_unplaced_io++;
        if (!S.pin_index.insert(n.name, (int)nl.nodes.size(), [&](int i) -> std::string_view { return nl.nodes[i].name; }))
            L.fail("duplicate pin '" + n.name + "'");
        nl.nodes.push_back(std::move(n));
    }
}

void def_nets(Lex &L, erp_netlist &nl, DefState &S) {
    L.need();
    L.expect(";");
    auto node_name = [&](int i) -> std::string_view { return nl.nodes[i].name; };
    std::string_view a, b;   // views into the DEF text, which outlives the parse
    for (;;) {
        L.need();
        if (L.t == "END") { L.expect("NETS"); break; }
        if (L.t != "-") L.fail("expected '-' or 'END NETS', found '" + std::string(L.t) + "'");
        std::string name(L.need());
        if (name == "MUSTJOIN") {
            nl.st.num_skipped_conns++;
            L.skip_statement();
            continue;
        }
        const size_t first = nl.conns.size();
        bool in_options = false;
        for (;;) {
            L.need();
            if (L.t == ";") break;
            if (L.t == "+") in_options = true;
            if (in_options || L.t != "(") continue;
            a = L.need();
            b = L.need();
            // "( comp pin + SYNTHESIZED )"
            do L.need();
            while (L.t != ")");
            if (a == "*") {
                nl.st.num_skipped_conns++;
            } else if (a == "PIN") {
                const int node = S.pin_index.find(b, node_name);
                if (node < 0) L.fail("net '" + name + "' names unknown pin '" + std::string(b) + "'");
                nl.conns.push_back({node, -1});
            } else {
                const int node = S.comp_index.find(a, node_name);
                if (node < 0) L.fail("net '" + name + "' names unknown component '" + std::string(a) + "'");
                const Macro &m = nl.macros[nl.nodes[node].master];
                const int k = m.find_pin(b);
                if (k < 0) L.fail("net '" + name + "': macro '" + m.name + "' has no pin '" + std::string(b) + "'");
                nl.conns.push_back({node, k});
            }
        }
        if (nl.conns.size() == first) {
            nl.st.num_dropped_nets++;
            continue;
        }
        nl.net_names.push_back(std::move(name));
        nl.net_begin.push_back((int32_t)nl.conns.size());
        if (nl.conns.size() > (size_t)INT32_MAX) L.fail("too many net connections");
    }
}

void read_def(const std::string &text, const char *path, erp_netlist &nl) {
    Lex L(text, path);
    DefState S;
    bool have_components = false;
    while (L.next()) {
        const std::string_view k = L.t;
        if (k == "END") {
            L.need();
            if (L.t == "DESIGN") break;
            L.fail("unexpected 'END " + std::string(L.t) + "'");
        } else if (k == "DESIGN") {
            nl.design_name = std::string(L.need());
            L.skip_statement();
        } else if (k == "UNITS") {
            L.expect("DISTANCE");
            L.expect("MICRONS");
            const int64_t v = L.inum();
            if (v <= 0) L.fail("UNITS DISTANCE MICRONS must be positive");
            nl.def_dbu = v;
            L.expect(";");
        } else if (k == "DIEAREA") {
            int64_t px, py;
            def_point(L, px, py);
            nl.die[0] = nl.die[2] = px;
            nl.die[1] = nl.die[3] = py;
            for (;;) {
                L.need();
                if (L.t == ";") break;
                if (L.t != "(") L.fail("bad DIEAREA");
                px = L.inum(); py = L.inum();
                L.expect(")");
                nl.die[0] = std::min(nl.die[0], px); nl.die[2] = std::max(nl.die[2], px);
                nl.die[1] = std::min(nl.die[1], py); nl.die[3] = std::max(nl.die[3], py);
            }
            nl.have_die = true;
        } else if (k == "COMPONENTS") {
            if (have_components) L.fail("second COMPONENTS section");
            if (!nl.nodes.empty()) L.fail("COMPONENTS must come before PINS");
            def_components(L, nl, S);
            have_components = true;
        } else if (k == "PINS") {
            if (nl.num_components != (int32_t)nl.nodes.size()) L.fail("second PINS section");
            def_pins(L, nl, S);
        } else if (k == "NETS") {
            def_nets(L, nl, S);
        } else if (is_section(k)) {
            const std::string name(k);
            L.skip_to_end(name);
        } else if (k == "BEGINEXT") {
            L.skip_to("ENDEXT");
        } else {
            L.skip_statement();   // VERSION, DIVIDERCHAR, BUSBITCHARS, ROW, TRACKS, GCELLGRID, HISTORY ...
        }
    }
    if (!nl.have_die) throw Fail(std::string(path) + ": no DIEAREA");
    if (nl.die[2] <= nl.die[0] || nl.die[3] <= nl.die[1]) throw Fail(std::string(path) + ": empty DIEAREA");
}

// ---------------------------------------------------------------- the design view

void finalize(erp_netlist &nl) {
    const int64_t D = nl.def_dbu > 0 ? nl.def_dbu : (nl.lef_dbu > 0 ? nl.lef_dbu : 1000);
    nl.def_dbu = D;
    const int64_t G = nl.lef_dbu > 0 ? nl.lef_dbu : D;
    nl.grid = G;
    for (Macro &m : nl.macros) {
        m.W = to_units(m.w * (double)G, "macro size");
        m.H = to_units(m.h * (double)G, "macro size");
        for (MacroPin &p : m.pins) {
            if (p.has) {
                p.c2x = to_units((p.lx + p.hx + 2.0 * m.ox) * (double)G, "pin shape");
                p.c2y = to_units((p.ly + p.hy + 2.0 * m.oy) * (double)G, "pin shape");
            } else {
                p.c2x = m.W;
                p.c2y = m.H;
            }
        }
    }
    const int32_t NN = (int32_t)nl.nodes.size();
    nl.order.clear();
    nl.order.reserve(NN);
    for (int32_t i = 0; i < nl.num_components; ++i)
        if (nl.nodes[i].kind == kMovable) nl.order.push_back(i);
    nl.num_movable = (int32_t)nl.order.size();
    for (int32_t i = 0; i < nl.num_components; ++i)
        if (nl.nodes[i].kind == kFixed) nl.order.push_back(i);
    for (int32_t i = nl.num_components; i < NN; ++i) nl.order.push_back(i);
    std::vector<int32_t> design_of(NN);
    for (int32_t k = 0; k < NN; ++k) design_of[nl.order[k]] = k;

    // every conversion is one correctly rounded division (double), then a cast
    const double x0 = (double)nl.die[0], y0 = (double)nl.die[1];
    const double Dd = (double)D, Gd = (double)G;
    nl.x.assign(NN, 0.f); nl.y.assign(NN, 0.f); nl.w.assign(NN, 0.f); nl.h.assign(NN, 0.f);
    double mov_area = 0, fixed_area = 0;
    const double die_w = (double)(nl.die[2] - nl.die[0]) / Dd, die_h = (double)(nl.die[3] - nl.die[1]) / Dd;
    for (int32_t k = 0; k < NN; ++k) {
        const Node &n = nl.nodes[nl.order[k]];
        if (n.placed) {   // an unplaced instance sits at the die's lower-left corner
            nl.x[k] = (float)(((double)n.X - x0) / Dd);
            nl.y[k] = (float)(((double)n.Y - y0) / Dd);
        }
        if (n.kind != kIo) {
            const Macro &m = nl.macros[n.master];
            const int64_t ww = swaps(n.orient) ? m.H : m.W, hh = swaps(n.orient) ? m.W : m.H;
            nl.w[k] = (float)((double)ww / Gd);
            nl.h[k] = (float)((double)hh / Gd);
            const double a = (double)nl.w[k] * (double)nl.h[k];
            if (n.kind == kMovable) {
                mov_area += a;
            } else {
                const double lx = std::max(0.0, (double)nl.x[k]), hx = std::min(die_w, (double)nl.x[k] + nl.w[k]);
                const double ly = std::max(0.0, (double)nl.y[k]), hy = std::min(die_h, (double)nl.y[k] + nl.h[k]);
                if (hx > lx && hy > ly) fixed_area += (hx - lx) * (hy - ly);
            }
        }
    }
    // nets: two-pin nets first, stable
    const int32_t E = (int32_t)nl.net_names.size();
    nl.net_order.clear();
    nl.net_order.reserve(E);
    for (int32_t e = 0; e < E; ++e)
        if (nl.net_begin[e + 1] - nl.net_begin[e] == 2) nl.net_order.push_back(e);
    nl.n_2nets = (int32_t)nl.net_order.size();
    for (int32_t e = 0; e < E; ++e)
        if (nl.net_begin[e + 1] - nl.net_begin[e] != 2) nl.net_order.push_back(e);
    const int32_t P = (int32_t)nl.conns.size();
    nl.net_ptr.assign(E + 1, 0);
    nl.net_pins.resize(P);
    nl.pin_inst.resize(P);
    nl.pox.resize(P);
    nl.poy.resize(P);
    int32_t pid = 0;
    for (int32_t q = 0; q < E; ++q) {
        const int32_t e = nl.net_order[q];
        for (int32_t c = nl.net_begin[e]; c < nl.net_begin[e + 1]; ++c, ++pid) {
            const Conn &cn = nl.conns[c];
            const Node &n = nl.nodes[cn.node];
            nl.net_pins[pid] = pid;
            nl.pin_inst[pid] = design_of[cn.node];
            int64_t qx, qy;
            if (cn.pin >= 0) {
                const Macro &m = nl.macros[n.master];
                orient_in_box(n.orient, m.pins[cn.pin].c2x, m.pins[cn.pin].c2y, 2 * m.W, 2 * m.H, qx, qy);
                nl.pox[pid] = (float)((double)qx / (2.0 * Gd));
                nl.poy[pid] = (float)((double)qy / (2.0 * Gd));
            } else {
                orient_at_point(n.orient, n.rlx + n.rhx, n.rly + n.rhy, qx, qy);
                nl.pox[pid] = (float)((double)qx / (2.0 * Dd));
                nl.poy[pid] = (float)((double)qy / (2.0 * Dd));
            }
        }
        nl.net_ptr[q + 1] = pid;
    }
    nl.inst_ptr.assign(NN + 1, 0);
    for (int32_t p = 0; p < P; ++p) nl.inst_ptr[nl.pin_inst[p] + 1]++;
    for (int32_t i = 0; i < NN; ++i) nl.inst_ptr[i + 1] += nl.inst_ptr[i];
    nl.inst_pins.resize(P);
    std::vector<int32_t> fill(nl.inst_ptr.begin(), nl.inst_ptr.end() - 1);
    for (int32_t p = 0; p < P; ++p) nl.inst_pins[fill[nl.pin_inst[p]]++] = p;
    nl.npins.resize(NN);
    for (int32_t i = 0; i < NN; ++i) nl.npins[i] = (float)(nl.inst_ptr[i + 1] - nl.inst_ptr[i]);
    nl.die_w = (float)die_w;
    nl.die_h = (float)die_h;
    nl.mov_area = (float)mov_area;
    const double free_area = die_w * die_h - fixed_area;
    nl.util = (float)(free_area > 0 ? mov_area / free_area : mov_area / (die_w * die_h));

    erp_lefdef_stats &s = nl.st;
    s.num_nodes = NN;
    s.num_movable = nl.num_movable;
    s.num_fixed = nl.num_components - nl.num_movable;
    s.num_io = NN - nl.num_components;
    s.num_nets = E;
    s.num_pins = P;
    s.num_macros = (int32_t)nl.macros.size();
    s.def_dbu = (int32_t)D;
    s.lef_dbu = (int32_t)G;
    for (int k = 0; k < 4; ++k) s.die[k] = nl.die[k];
}

// ---------------------------------------------------------------- writing

struct Out {
    FILE *f;
    std::string buf;
    explicit Out(FILE *f_) : f(f_) { buf.reserve(1 << 20); }
    void put(const char *s, size_t n) {
        buf.append(s, n);
        if (buf.size() >= (1u << 20)) flush();
    }
    void put(std::string_view s) { put(s.data(), s.size()); }
    void printf(const char *fmt, ...) __attribute__((format(printf, 2, 3))) {
        char tmp[512];
        va_list ap;
        va_start(ap, fmt);
        const int n = std::vsnprintf(tmp, sizeof tmp, fmt, ap);
        va_end(ap);
        if (n < 0) throw Fail("format error");
        if ((size_t)n < sizeof tmp) {
            put(tmp, (size_t)n);
        } else {
            std::string big((size_t)n + 1, '\0');
            va_start(ap, fmt);
            std::vsnprintf(&big[0], big.size(), fmt, ap);
            va_end(ap);
            put(big.data(), (size_t)n);
        }
    }
    void flush() {
        if (!buf.empty() && std::fwrite(buf.data(), 1, buf.size(), f) != buf.size()) throw Fail("write failed");
        buf.clear();
    }
};

struct File {
    FILE *f = nullptr;
    std::string path;
    explicit File(const char *p) : path(p) {
        f = std::fopen(p, "wb");
        if (!f) throw Fail(std::string(p) + ": cannot open for writing");
    }
    void close() {
        if (f && std::fclose(f) != 0) { f = nullptr; throw Fail(path + ": write failed"); }
        f = nullptr;
    }
    ~File() { if (f) std::fclose(f); }
};

// microns of n / den (exact decimal for the usual 100 .. 10000 grids)
// n / den microns as "%.15g" prints the double n / den.  When den divides 10^6
// (every DEF / LEF grid of 100 ... 10000 units per micron does), n / den is a
// terminating decimal with at most six fraction digits; with at most 15
// significant digits and a magnitude of at least 1e-4 (below 1e15 by the
// bound on n), "%.15g" prints exactly that decimal with trailing zeros
// removed, which is formed here in integers.  Anything else goes through
// snprintf.
std::string um(int64_t n, int64_t den) {
    if (den > 0 && 1000000 % den == 0 && n > -100000000000000LL && n < 100000000000000LL) {
        const uint64_t scale = (uint64_t)(1000000 / den);   // n / den = n * scale / 10^6
        const bool neg = n < 0;
        const uint64_t an = neg ? (uint64_t)(-n) : (uint64_t)n;
        if (an <= UINT64_MAX / scale) {
            const uint64_t q = an * scale;
            if (q == 0) return "0";
            const uint64_t ip = q / 1000000;
            uint64_t fp = q % 1000000;
            int frac = 6;   // fraction digits after removing trailing zeros
            while (frac > 0 && fp % 10 == 0) {
                fp /= 10;
                --frac;
            }
            char idig[24];
            int nd = 0;
            for (uint64_t t = ip; t; t /= 10) idig[nd++] = (char)('0' + t % 10);
            int sig;
            if (ip > 0) {
                sig = nd + frac;
            } else {
                int lead = 0;   // zeros between the point and the first nonzero digit
                for (uint64_t t = q % 1000000; t < 100000; t *= 10) ++lead;
                sig = frac - lead;
                if (lead >= 4) sig = 99;   // below 1e-4: "%g" uses an exponent
            }
            if (sig <= 15) {
                std::string out;
                if (neg) out.push_back('-');
                if (nd == 0) out.push_back('0');
                while (nd) out.push_back(idig[--nd]);
                if (frac > 0) {
                    out.push_back('.');
                    char fd[8];
                    for (int k = frac - 1; k >= 0; --k) {
                        fd[k] = (char)('0' + fp % 10);
                        fp /= 10;
                    }
                    out.append(fd, (size_t)frac);
                }
                return out;
            }
        }
    }
    char b[64];
    std::snprintf(b, sizeof b, "%.15g", (double)n / (double)den);
    return b;
}

const int64_t kPinHalf = 50;   // written pin shapes: a square of +-kPinHalf grid units around the centre

void write_lef(const erp_netlist &nl, const char *path) {
    File F(path);
    Out o(F.f);
    const int64_t G = nl.grid;
    o.put("VERSION 5.8 ;\nBUSBITCHARS \"[]\" ;\nDIVIDERCHAR \"/\" ;\n\nUNITS\n");
    o.printf("  DATABASE MICRONS %lld ;\nEND UNITS\n\n", (long long)G);
    o.printf("MANUFACTURINGGRID %s ;\n\n", um(1, G).c_str());
    o.put("LAYER metal1\n  TYPE ROUTING ;\n  DIRECTION HORIZONTAL ;\nEND metal1\n\n");
    if (nl.site_w > 0 && nl.row_h > 0)
        o.printf("SITE %s\n  CLASS CORE ;\n  SYMMETRY Y ;\n  SIZE %s BY %s ;\nEND %s\n\n", nl.site_name.c_str(),
                 um(to_units(nl.site_w * (double)G, "site width"), G).c_str(),
                 um(to_units(nl.row_h * (double)G, "row height"), G).c_str(),
                 nl.site_name.c_str());
    for (const Macro &m : nl.macros) {
        o.printf("MACRO %s\n  CLASS %s ;\n  ORIGIN 0 0 ;\n  SIZE %s BY %s ;\n  SYMMETRY X Y ;\n", m.name.c_str(),
                 m.block ? "BLOCK" : "CORE", um(m.W, G).c_str(), um(m.H, G).c_str());
        if (!m.block && nl.site_w > 0 && nl.row_h > 0) o.printf("  SITE %s ;\n", nl.site_name.c_str());
        for (const MacroPin &p : m.pins) {
            // the centre (c2x, c2y) / 2 in grid units; the shape keeps the centre exactly
            o.printf("  PIN %s\n    DIRECTION INOUT ;\n    USE SIGNAL ;\n    PORT\n      LAYER metal1 ;\n"
                     "        RECT %s %s %s %s ;\n    END\n  END %s\n",
                     p.name.c_str(), um(p.c2x - 2 * kPinHalf, 2 * G).c_str(), um(p.c2y - 2 * kPinHalf, 2 * G).c_str(),
                     um(p.c2x + 2 * kPinHalf, 2 * G).c_str(), um(p.c2y + 2 * kPinHalf, 2 * G).c_str(), p.name.c_str());
        }
        o.printf("END %s\n\n", m.name.c_str());
    }
    o.put("END LIBRARY\n");
    o.flush();
    F.close();
}

void put_placement(Out &o, const char *kw, int64_t X, int64_t Y, int orient) {
    o.printf("%s ( %lld %lld ) %s", kw, (long long)X, (long long)Y, kOrientName[orient]);
}

// The DEF of a netlist; movable components at (xs, ys) microns when given.
void write_def(const erp_netlist &nl, const char *path, const int64_t *xs, const int64_t *ys) {
    File F(path);
    Out o(F.f);
    const int64_t D = nl.def_dbu;
    o.put("VERSION 5.8 ;\nDIVIDERCHAR \"/\" ;\nBUSBITCHARS \"[]\" ;\n");
    o.printf("DESIGN %s ;\nUNITS DISTANCE MICRONS %lld ;\n\n", nl.design_name.c_str(), (long long)D);
    o.printf("DIEAREA ( %lld %lld ) ( %lld %lld ) ;\n\n", (long long)nl.die[0], (long long)nl.die[1],
             (long long)nl.die[2], (long long)nl.die[3]);
    if (nl.site_w > 0 && nl.row_h > 0) {
        const int64_t step = to_units(nl.site_w * (double)D, "site width");
        const int64_t rh = to_units(nl.row_h * (double)D, "row height");
        if (step > 0 && rh > 0) {
            const int64_t sites = (nl.die[2] - nl.die[0]) / step, rows = (nl.die[3] - nl.die[1]) / rh;
            if (rows > (int64_t(1) << 24)) throw Fail("row height too small for the die: more than 2^24 rows");
            for (int64_t r = 0; r < rows; ++r)
                o.printf("ROW ROW_%lld %s %lld %lld %s DO %lld BY 1 STEP %lld 0 ;\n", (long long)r, nl.site_name.c_str(),
                         (long long)nl.die[0], (long long)(nl.die[1] + r * rh), (r & 1) ? "FS" : "N", (long long)sites,
                         (long long)step);
            o.put("\n");
        }
    }
    o.printf("COMPONENTS %d ;\n", (int)nl.num_components);
    for (int32_t i = 0; i < nl.num_components; ++i) {
        const Node &n = nl.nodes[i];
        o.printf("- %s %s + ", n.name.c_str(), nl.macros[n.master].name.c_str());
        if (n.kind == kFixed) put_placement(o, "FIXED", n.X, n.Y, n.orient);
        else if (xs) put_placement(o, "PLACED", xs[i], ys[i], n.orient);
        else if (n.placed) put_placement(o, "PLACED", n.X, n.Y, n.orient);
        else o.put("UNPLACED");
        o.put(" ;\n");
    }
    o.put("END COMPONENTS\n\n");
    const int32_t NN = (int32_t)nl.nodes.size();
    o.printf("PINS %d ;\n", (int)(NN - nl.num_components));
    for (int32_t i = nl.num_components; i < NN; ++i) {
        const Node &n = nl.nodes[i];
        o.printf("- %s + NET %s + DIRECTION INPUT + USE SIGNAL\n  + LAYER metal1 ( %lld %lld ) ( %lld %lld )\n", n.name.c_str(),
                 n.net.empty() ? n.name.c_str() : n.net.c_str(), (long long)n.rlx, (long long)n.rly, (long long)n.rhx,
                 (long long)n.rhy);
        if (n.placed) {
            o.put("  + ");
            put_placement(o, n.status.c_str(), n.X, n.Y, n.orient);
        }
        o.put(" ;\n");
    }
    o.put("END PINS\n\n");
    const int32_t E = (int32_t)nl.net_names.size();
    o.printf("NETS %d ;\n", (int)E);
    for (int32_t e = 0; e < E; ++e) {
        o.printf("- %s", nl.net_names[e].c_str());
        int k = 0;
        for (int32_t c = nl.net_begin[e]; c < nl.net_begin[e + 1]; ++c, ++k) {
            const Conn &cn = nl.conns[c];
            const Node &n = nl.nodes[cn.node];
            if (k && k % 8 == 0) o.put("\n ");
            if (cn.pin < 0) o.printf(" ( PIN %s )", n.name.c_str());
            else o.printf(" ( %s %s )", n.name.c_str(), nl.macros[n.master].pins[cn.pin].name.c_str());
        }
        o.put(" ;\n");
    }
    o.put("END NETS\n\nEND DESIGN\n");
    o.flush();
    F.close();
}

// The source DEF with the placement clause of every movable component replaced.
void splice_def(const erp_netlist &nl, const char *path, const int64_t *xs, const int64_t *ys) {
    File F(path);
    Out o(F.f);
    const std::string &src = nl.def_text;
    size_t at = 0;
    char tmp[160];
    for (int32_t i = 0; i < nl.num_components; ++i) {
        const Node &n = nl.nodes[i];
        if (n.kind != kMovable) continue;
        o.put(src.data() + at, n.clause_off - at);
        const int len = std::snprintf(tmp, sizeof tmp, "%sPLACED ( %lld %lld ) %s%s", n.clause_insert ? "+ " : "",
                                      (long long)xs[i], (long long)ys[i], kOrientName[n.placed ? (int)n.orient : (int)oN],
                                      n.clause_insert ? " " : "");
        o.put(tmp, (size_t)len);
        at = n.clause_off + (n.clause_insert ? 0 : n.clause_len);
    }
    o.put(src.data() + at, src.size() - at);
    o.flush();
    F.close();
}

erp_status fail_with(const std::string &msg, erp_status st = ERP_EINVAL) {
    g_err = msg;
    return st;
}

}  // namespace

extern "C" const char *erp_lefdef_last_error(void) { return g_err.c_str(); }

extern "C" erp_status erp_lefdef_read(const char *const *lef_paths, int32_t num_lef, const char *def_path,
                                      erp_netlist **out) {
    if (!out) return fail_with("out is NULL");
    *out = nullptr;
    if (!def_path || num_lef < 0 || (num_lef > 0 && !lef_paths)) return fail_with("bad arguments");
    try {
        std::unique_ptr<erp_netlist> nl(new erp_netlist());
        std::string text;
        for (int32_t k = 0; k < num_lef; ++k) {
            if (!lef_paths[k]) return fail_with("LEF path is NULL");
            if (!read_file(lef_paths[k], text)) return fail_with(std::string(lef_paths[k]) + ": cannot read");
            read_lef(text, lef_paths[k], *nl);
        }
        if (!read_file(def_path, nl->def_text)) return fail_with(std::string(def_path) + ": cannot read");
        read_def(nl->def_text, def_path, *nl);
        finalize(*nl);
        *out = nl.release();
        g_err.clear();
        return ERP_OK;
    } catch (const Fail &f) {
        return fail_with(f.what());
    } catch (const std::bad_alloc &) {
        return fail_with("out of host memory", ERP_ENOMEM);
    }
}

extern "C" erp_status erp_netlist_from_design(const erp_design *d, const erp_lefdef_params *p, erp_netlist **out) {
    if (!out) return fail_with("out is NULL");
    *out = nullptr;
    if (!d) return fail_with("design is NULL");
    const int64_t D = p && p->dbu > 0 ? p->dbu : 2000;
    const int32_t NN = d->num_nodes, P = d->num_pins, E = d->num_nets;
    if (NN < 0 || d->num_movable < 0 || d->num_movable > NN || P < 0 || E < 0) return fail_with("bad counts");
    if (!(d->die_w > 0) || !(d->die_h > 0)) return fail_with("die must have positive size");
    if (NN && (!d->x || !d->y || !d->w || !d->h)) return fail_with("instance arrays missing");
    if (P && (!d->pin_ox || !d->pin_oy || !d->pin_inst)) return fail_with("pin arrays missing");
    if (!d->net_ptr || !d->inst_pin_ptr || (P && (!d->net_pins || !d->inst_pins))) return fail_with("CSR arrays missing");
    try {
        std::unique_ptr<erp_netlist> nl(new erp_netlist());
        nl->from_design = true;
        nl->design_name = "synth";
        nl->lef_dbu = nl->def_dbu = D;
        nl->site_w = p && p->site_w > 0 ? p->site_w : 0;
        nl->row_h = p && p->row_h > 0 ? p->row_h : 0;
        nl->die[0] = nl->die[1] = 0;
        nl->die[2] = to_units((double)d->die_w * (double)D, "die size");
        nl->die[3] = to_units((double)d->die_h * (double)D, "die size");
        nl->have_die = true;
        auto q = [&](float v) -> int64_t {
            if (!std::isfinite(v)) throw Fail("non-finite coordinate in design");
            return to_units((double)v * (double)D, "coordinate");
        };
        // slot of each pin in its instance's list: the macro pin P<slot>
        std::vector<int32_t> slot(P, -1);
        for (int32_t i = 0; i < NN; ++i)
            for (int32_t k = d->inst_pin_ptr[i]; k < d->inst_pin_ptr[i + 1]; ++k) {
                const int32_t pid = d->inst_pins[k];
                if (pid < 0 || pid >= P || d->pin_inst[pid] != i || slot[pid] >= 0)
                    throw Fail("inst_pins does not match pin_inst");
                slot[pid] = k - d->inst_pin_ptr[i];
            }
        for (int32_t pid = 0; pid < P; ++pid)
            if (slot[pid] < 0) throw Fail("a pin is missing from inst_pins");
        // which fixed zero-size instances become DEF PINS: at most one pin
        std::vector<uint8_t> kind(NN);
        for (int32_t i = 0; i < NN; ++i) {
            const int32_t np = d->inst_pin_ptr[i + 1] - d->inst_pin_ptr[i];
            kind[i] = i < d->num_movable ? kMovable : (d->w[i] == 0.f && d->h[i] == 0.f && np <= 1 ? kIo : kFixed);
        }
        // components in design order (movable, then fixed), then DEF PINS
        std::vector<int32_t> parse_of(NN);
        std::unordered_map<std::string, int> dedupe;
        std::string key;
        int32_t ncomp = 0, nio = 0;
        for (int pass = 0; pass < 2; ++pass)
            for (int32_t i = 0; i < NN; ++i) {
                if ((pass == 0) != (kind[i] != kIo)) continue;
                Node n;
                n.kind = kind[i];
                n.placed = true;
                n.X = q(d->x[i]);
                n.Y = q(d->y[i]);
                n.status = "FIXED";
                if (n.kind == kIo) {
                    n.name = "p" + std::to_string(nio++);
                    if (d->inst_pin_ptr[i + 1] > d->inst_pin_ptr[i]) {
                        const int32_t pid = d->inst_pins[d->inst_pin_ptr[i]];
                        const int64_t cx = q(d->pin_ox[pid]), cy = q(d->pin_oy[pid]);
                        n.rlx = cx - kPinHalf; n.rhx = cx + kPinHalf;
                        n.rly = cy - kPinHalf; n.rhy = cy + kPinHalf;
                    } else {
                        n.rlx = n.rly = -kPinHalf;
                        n.rhx = n.rhy = kPinHalf;
                    }
                } else {
                    const bool block = n.kind == kFixed;
                    n.name = (block ? "m" : "c") + std::to_string(i);
                    const int64_t W = q(d->w[i]), H = q(d->h[i]);
                    key.assign(block ? "B" : "C");
                    auto app = [&](int64_t v) { key.append(reinterpret_cast<const char *>(&v), sizeof v); };
                    app(W);
                    app(H);
                    for (int32_t k = d->inst_pin_ptr[i]; k < d->inst_pin_ptr[i + 1]; ++k) {
                        const int32_t pid = d->inst_pins[k];
                        app(q(d->pin_ox[pid]));
                        app(q(d->pin_oy[pid]));
                    }
                    auto it = dedupe.find(key);
                    if (it == dedupe.end()) {
                        Macro m;
                        m.block = block;
                        m.name = (block ? "BLOCK" : "CELL") + std::to_string(nl->macros.size());
                        m.w = (double)W / (double)D;
                        m.h = (double)H / (double)D;
                        for (int32_t k = d->inst_pin_ptr[i]; k < d->inst_pin_ptr[i + 1]; ++k) {
                            const int32_t pid = d->inst_pins[k];
                            MacroPin mp;
                            mp.name = "P" + std::to_string(k - d->inst_pin_ptr[i]);
                            const int64_t cx = q(d->pin_ox[pid]), cy = q(d->pin_oy[pid]);
                            mp.add((double)(cx - kPinHalf) / (double)D, (double)(cy - kPinHalf) / (double)D);
                            mp.add((double)(cx + kPinHalf) / (double)D, (double)(cy + kPinHalf) / (double)D);
                            m.pins.push_back(std::move(mp));
                        }
                        if (m.pins.size() >= 16)
                            for (size_t k = 0; k < m.pins.size(); ++k) m.index_pin((int)k);
                        it = dedupe.emplace(key, (int)nl->macros.size()).first;
                        nl->macro_index.insert(m.name, (int)nl->macros.size(),
                                               [&](int j) -> std::string_view { return nl->macros[j].name; });
                        nl->macros.push_back(std::move(m));
                    }
                    n.master = it->second;
                    ++ncomp;
                }
                parse_of[i] = (int32_t)nl->nodes.size();
                nl->nodes.push_back(std::move(n));
            }
        nl->num_components = ncomp;
        // nets in design order, connections in net order
        nl->net_begin.assign(1, 0);
        for (int32_t e = 0; e < E; ++e) {
            const int32_t b = d->net_ptr[e], en = d->net_ptr[e + 1];
            if (b < 0 || en < b || en > P) throw Fail("bad net_ptr");
            if (en == b) continue;
            nl->net_names.push_back("n" + std::to_string(e));
            for (int32_t k = b; k < en; ++k) {
                const int32_t pid = d->net_pins[k];
                if (pid < 0 || pid >= P) throw Fail("net pin out of range");
                const int32_t i = d->pin_inst[pid];
                if (i < 0 || i >= NN) throw Fail("pin_inst out of range");
                Node &n = nl->nodes[parse_of[i]];
                if (n.kind == kIo) {
                    nl->conns.push_back({parse_of[i], -1});
                    n.net = nl->net_names.back();
                } else {
                    nl->conns.push_back({parse_of[i], slot[pid]});
                }
            }
            nl->net_begin.push_back((int32_t)nl->conns.size());
        }
        finalize(*nl);
        *out = nl.release();
        g_err.clear();
        return ERP_OK;
    } catch (const Fail &f) {
        return fail_with(f.what());
    } catch (const std::bad_alloc &) {
        return fail_with("out of host memory", ERP_ENOMEM);
    }
}

extern "C" erp_status erp_netlist_design(const erp_netlist *nl, erp_design *d) {
    if (!nl || !d) return fail_with("bad arguments");
    std::memset(d, 0, sizeof(*d));
    d->num_nodes = (int32_t)nl->order.size();
    d->num_movable = nl->num_movable;
    d->num_pins = (int32_t)nl->pin_inst.size();
    d->num_nets = (int32_t)nl->net_order.size();
    d->n_2nets = nl->n_2nets;
    d->x = nl->x.data(); d->y = nl->y.data(); d->w = nl->w.data(); d->h = nl->h.data();
    d->num_pins_f = nl->npins.data();
    d->pin_ox = nl->pox.data(); d->pin_oy = nl->poy.data();
    d->pin_inst = nl->pin_inst.data();
    d->net_ptr = nl->net_ptr.data(); d->net_pins = nl->net_pins.data();
    d->inst_pin_ptr = nl->inst_ptr.data(); d->inst_pins = nl->inst_pins.data();
    d->die_w = nl->die_w; d->die_h = nl->die_h;
    d->cell_utilization = nl->util;
    d->movable_area = nl->mov_area;
    return ERP_OK;
}

extern "C" erp_status erp_netlist_stats(const erp_netlist *nl, erp_lefdef_stats *s) {
    if (!nl || !s) return fail_with("bad arguments");
    *s = nl->st;
    return ERP_OK;
}

extern "C" const char *erp_netlist_node_name(const erp_netlist *nl, int32_t i) {
    if (!nl || i < 0 || i >= (int32_t)nl->order.size()) return nullptr;
    return nl->nodes[nl->order[i]].name.c_str();
}

extern "C" const char *erp_netlist_net_name(const erp_netlist *nl, int32_t e) {
    if (!nl || e < 0 || e >= (int32_t)nl->net_order.size()) return nullptr;
    return nl->net_names[nl->net_order[e]].c_str();
}

extern "C" erp_status erp_lefdef_write(const erp_netlist *nl, const char *lef_path, const char *def_path) {
    if (!nl || (!lef_path && !def_path)) return fail_with("bad arguments");
    try {
        if (lef_path) write_lef(*nl, lef_path);
        if (def_path) write_def(*nl, def_path, nullptr, nullptr);
        return ERP_OK;
    } catch (const Fail &f) {
        return fail_with(f.what());
    } catch (const std::bad_alloc &) {
        return fail_with("out of host memory", ERP_ENOMEM);
    }
}

extern "C" erp_status erp_def_write_placed(const erp_netlist *nl, const float *x, const float *y, const char *def_path) {
    if (!nl || !x || !y || !def_path) return fail_with("bad arguments");
    try {
        // movable positions (design order = the first num_movable of order) to DEF units
        std::vector<int64_t> xs(nl->num_components, 0), ys(nl->num_components, 0);
        const double D = (double)nl->def_dbu;
        for (int32_t k = 0; k < nl->num_movable; ++k) {
            if (!std::isfinite(x[k]) || !std::isfinite(y[k])) throw Fail("non-finite position of instance " + std::to_string(k));
            const int32_t i = nl->order[k];
            xs[i] = to_units((double)x[k] * D, "position") + nl->die[0];
            ys[i] = to_units((double)y[k] * D, "position") + nl->die[1];
        }
        if (nl->from_design) write_def(*nl, def_path, xs.data(), ys.data());
        else splice_def(*nl, def_path, xs.data(), ys.data());
        return ERP_OK;
    } catch (const Fail &f) {
        return fail_with(f.what());
    } catch (const std::bad_alloc &) {
        return fail_with("out of host memory", ERP_ENOMEM);
    }
}

extern "C" void erp_netlist_destroy(erp_netlist *nl) { delete nl; }
