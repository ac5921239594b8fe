// erplacer_gb300: the reference's command-line driver (src/main.rs:32-98) over
// the C ABI.  It reads the LEF/DEF pair, builds the placement on the GPU, runs
// the Nesterov loop, snapshots the placement and writes the placed DEF.
//
// Reference flags, same meaning: -d/--def FILE, -l/--lef FILE (repeatable:
// technology, then cells), --iterations N (default 1), -v/--verbose.
// Additions: --bins MxN (default 512x512, src/placement.rs:50),
// --target-density T (default -1: the design's cell utilisation,
// src/placement.rs:134), --stop-overflow O (0: run all iterations, like the
// reference), --precision fp32|tf32|bf16x3, --start center|db, --out FILE
// (placed DEF), --images DIR (default: ./images when it exists, as
// draw_placement expects), --device K.
// Snapshots are binary PPM files named solution_<iteration:07>.ppm, taken at
// iteration 0, every 50 iterations with --verbose, and at the end
// (src/main.rs:75-95, src/drawing.rs:56).
#include "erplacer.h"

#include <sys/stat.h>

#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;

double secs(Clock::time_point a) { return std::chrono::duration<double>(Clock::now() - a).count(); }

void usage(FILE *f) {
    std::fprintf(f,
                 "usage: erplacer_gb300 -d FILE -l FILE [-l FILE ...] [--iterations N] [-v]\n"
                 "                      [--bins MxN] [--target-density T] [--stop-overflow O]\n"
                 "                      [--precision fp32|tf32|bf16x3] [--start center|db]\n"
                 "                      [--out FILE] [--images DIR] [--device K]\n");
}

bool is_dir(const char *p) {
    struct stat s;
    return stat(p, &s) == 0 && S_ISDIR(s.st_mode);
}

bool write_ppm(const std::string &path, const std::vector<unsigned char> &rgb, int w, int h) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    std::fprintf(f, "P6\n%d %d\n255\n", w, h);
    const bool ok = std::fwrite(rgb.data(), 1, rgb.size(), f) == rgb.size();
    return std::fclose(f) == 0 && ok;
}

struct Args {
    std::string def;
    std::vector<std::string> lef;
    long iterations = 1;
    bool verbose = false;
    int m = 512, n = 512;
    float target_density = -1.0f;
    float stop_overflow = 0.0f;
    int precision = ERP_PREC_FP32;
    int start = ERP_START_CENTER;
    std::string out, images;
    int device = 0;
};

// a whole-token number, or exit 2 (strtol / strtof alone take "12abc" as 12
// and "abc" as 0)
long whole_int(const std::string &k, const char *v) {
    char *end = nullptr;
    errno = 0;
    const long r = std::strtol(v, &end, 10);
    if (end == v || *end || errno) {
        std::fprintf(stderr, "error: %s wants an integer, got '%s'\n", k.c_str(), v);
        std::exit(2);
    }
    return r;
}
float whole_float(const std::string &k, const char *v) {
    char *end = nullptr;
    const float r = std::strtof(v, &end);
    if (end == v || *end || !std::isfinite(r)) {
        std::fprintf(stderr, "error: %s wants a finite number, got '%s'\n", k.c_str(), v);
        std::exit(2);
    }
    return r;
}

int parse(int argc, char **argv, Args &a) {
    for (int i = 1; i < argc; ++i) {
        const std::string k = argv[i];
        auto val = [&](const char *what) -> const char * {
            if (i + 1 >= argc) {
                std::fprintf(stderr, "error: %s needs %s\n", k.c_str(), what);
                std::exit(2);
            }
            return argv[++i];
        };
        if (k == "-d" || k == "--def") a.def = val("a file");
        else if (k == "-l" || k == "--lef") a.lef.push_back(val("a file"));
        else if (k == "--iterations") a.iterations = whole_int(k, val("a count"));
        else if (k == "-v" || k == "--verbose") a.verbose = true;
        else if (k == "--bins") {
            const char *v = val("MxN");
            char tail = 0;
            if (std::sscanf(v, "%dx%d%c", &a.m, &a.n, &tail) != 2) {
                std::fprintf(stderr, "error: --bins wants MxN, got '%s'\n", v);
                return 2;
            }
        } else if (k == "--target-density") a.target_density = whole_float(k, val("a value"));
        else if (k == "--stop-overflow") a.stop_overflow = whole_float(k, val("a value"));
        else if (k == "--precision") {
            const std::string v = val("fp32|tf32|bf16x3");
            if (v == "fp32") a.precision = ERP_PREC_FP32;
            else if (v == "tf32") a.precision = ERP_PREC_TF32_GEMM;
            else if (v == "bf16x3") a.precision = ERP_PREC_BF16X3_GEMM;
            else {
                std::fprintf(stderr, "error: unknown precision '%s'\n", v.c_str());
                return 2;
            }
        } else if (k == "--start") {
            const std::string v = val("center|db");
            if (v == "center") a.start = ERP_START_CENTER;
            else if (v == "db") a.start = ERP_START_DB;
            else {
                std::fprintf(stderr, "error: unknown start '%s'\n", v.c_str());
                return 2;
            }
        } else if (k == "--out") a.out = val("a file");
        else if (k == "--images") a.images = val("a directory");
        else if (k == "--device") a.device = (int)whole_int(k, val("an index"));
        else if (k == "-h" || k == "--help") {
            usage(stdout);
            std::exit(0);
        } else {
            std::fprintf(stderr, "error: unknown argument '%s'\n", k.c_str());
            usage(stderr);
            return 2;
        }
    }
    if (a.def.empty() || a.lef.empty()) {
        usage(stderr);
        return 2;
    }
    if (a.iterations < 0) {
        std::fprintf(stderr, "error: --iterations must be >= 0\n");
        return 2;
    }
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    std::setvbuf(stdout, nullptr, _IOLBF, 0);   // a redirected log keeps the order of the INFO and error lines
    Args a;
    if (int rc = parse(argc, argv, a)) return rc;
    if (a.images.empty() && is_dir("images")) a.images = "images";

    auto t0 = Clock::now();
    std::vector<const char *> lefs;
    for (auto &s : a.lef) lefs.push_back(s.c_str());
    erp_netlist *nl = nullptr;
    erp_status st = erp_lefdef_read(lefs.data(), (int32_t)lefs.size(), a.def.c_str(), &nl);
    if (st != ERP_OK) {
        std::fprintf(stderr, "error: %s\n", erp_lefdef_last_error());
        return 1;
    }
    erp_lefdef_stats ls;
    erp_netlist_stats(nl, &ls);
    erp_design d;
    erp_netlist_design(nl, &d);
    std::printf("[INFO] Reading DB took %.3fs: %d instances (%d movable, %d fixed, %d IO pins), %d nets, %d pins; "
                "die %.3f x %.3f um; utilisation %.4f\n",
                secs(t0), ls.num_nodes, ls.num_movable, ls.num_fixed, ls.num_io, ls.num_nets, ls.num_pins, d.die_w,
                d.die_h, d.cell_utilization);
    if (ls.num_dropped_nets || ls.num_skipped_conns || ls.num_unplaced_io)
        std::printf("[INFO] skipped: %d nets without connections, %d wildcard/MUSTJOIN connections, %d unplaced IO pins\n",
                    ls.num_dropped_nets, ls.num_skipped_conns, ls.num_unplaced_io);

    t0 = Clock::now();
    erp_params p;
    std::memset(&p, 0, sizeof p);
    p.num_bins_x = a.m;
    p.num_bins_y = a.n;
    p.target_density = a.target_density;
    p.start_mode = a.start;
    p.precision = a.precision;
    p.device = a.device;
    erp_ctx *ctx = nullptr;
    st = erp_create(&d, &p, &ctx);
    if (st != ERP_OK) {
        std::fprintf(stderr, "error: %s: %s\n", erp_status_string(st), erp_last_error(ctx));
        erp_destroy(ctx);
        erp_netlist_destroy(nl);
        return 1;
    }
    erp_scalars sc;
    erp_get_scalars(ctx, &sc);
    std::printf("[INFO] Creating Placement took %.3fs\n[INFO] Bins: %g x %g (%d x %d)\n", secs(t0), sc.bin_w, sc.bin_h,
                sc.num_bins_x, sc.num_bins_y);

    std::vector<unsigned char> img;
    int iw = 0, ih = 0;
    auto snapshot = [&](long it) {
        if (a.images.empty()) return;
        if (img.empty()) {
            if (erp_snapshot_size(ctx, &iw, &ih) != ERP_OK) return;
            img.resize((size_t)iw * ih * 3);
        }
        char name[64];
        std::snprintf(name, sizeof name, "/solution_%07ld.ppm", it);
        if (erp_snapshot_placement(ctx, img.data(), img.size()) != ERP_OK ||
            !write_ppm(a.images + name, img, iw, ih))
            std::fprintf(stderr, "[WARN] snapshot %ld not written\n", it);
    };
    snapshot(0);

    const auto tp = Clock::now();
    erp_step_stats ss{};
    long ran = 0;
    for (long i = 0; i < a.iterations; ++i) {
        const auto ts = Clock::now();
        st = erp_step(ctx, &ss);
        if (st != ERP_OK) {
            std::fprintf(stderr, "error: step %ld: %s: %s\n", i, erp_status_string(st), erp_last_error(ctx));
            break;
        }
        ++ran;
        if (a.verbose) {
            std::printf("[DEBUG] Step %-5ld took %.3fms  hpwl %.6g  overflow %.5f  lambda %.4g\n", i,
                        1e3 * secs(ts), ss.hpwl, ss.overflow, ss.density_weight);
            if (i % 50 == 0) snapshot(i);
        }
        if (ss.should_stop) {
            std::printf("[INFO] Something is wrong!\n");
            if (a.verbose) snapshot(i);
        }
        if (a.stop_overflow > 0.f && ss.overflow <= a.stop_overflow) break;
    }
    std::printf("[INFO] Placement took %.3fs: %ld iterations, hpwl %.6g, overflow %.5f\n", secs(tp), ran, ss.hpwl,
                ss.overflow);
    snapshot(a.iterations);

    int rc = st == ERP_OK ? 0 : 1;
    if (rc == 0 && !a.out.empty()) {
        std::vector<float> x(d.num_nodes), y(d.num_nodes);
        st = erp_get_positions(ctx, x.data(), y.data());
        if (st == ERP_OK) st = erp_def_write_placed(nl, x.data(), y.data(), a.out.c_str());
        if (st != ERP_OK) {
            std::fprintf(stderr, "error: placed DEF: %s\n", erp_lefdef_last_error());
            rc = 1;
        } else {
            std::printf("[INFO] wrote %s\n", a.out.c_str());
        }
    }
    erp_destroy(ctx);
    erp_netlist_destroy(nl);
    return rc;
}
