// ref_placer.cpp -- extern "C" entry points onto the reference's own placer
// (vck5000/host/src/AIEplace.cpp, DataBase.cpp, Grid.cpp, Net.cpp, DCT.cpp)
// compiled for the CPU.
//
// TEST INFRASTRUCTURE ONLY.  Built by `make -C oracle refplacer REF=<checkout>`
// into _ref/libref_placer.so, with stand-ins for what the reference host
// links but this machine lacks:
//   * XRT (oracle/ref_stubs/experimental/): never called -- the placer runs
//     with use_aie false;
//   * cairo (oracle/ref_stubs/cairo/, no-op definitions below): the
//     visualiser is set up by Placer::Placer but draws only from run();
//   * the Limbo LEF/DEF parsers: LefParser::read / DefParser::read below hand
//     a netlist to the reference's own DataBase callbacks (add_def_component,
//     add_def_pin, add_def_net, DataBase.cpp:357-416) instead of parsing files;
//     MacroClass entries and the die box go into DataBase directly (the LEF
//     callback takes a LEF-library object, and DEF's die area is integer);
//   * the LEF library's lefi*::print / lefiMacro accessors, referenced by
//     Limbo's LefDataBase.cc defaults and DataBase::lef_macro_cbk, never
//     called (no LEF is parsed).
// Placer::Placer reads host/config_aieplace.json relative to the working
// directory (AIEplace.cpp:90-109): the harness writes one into a scratch
// directory and constructs the placer there.
//
// Entry points: build a placer on a CSR netlist, set positions, and run one of
// Placer::computeAllPartials_CPU (AIEplace.cpp:574-673), computeOverlaps
// (:937-967), the host's DCT field path compute_a_uv_DCT / compute_eField_DCT
// (:752-934), the CPU loop's naive field path computeElectricFields_CPU
// (:679-750) or nudgeAllNodes (:993-1046), each timed with a steady clock;
// and passes of the CPU loop itself (Placer::run's body, :55-76).
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <string>
#include <vector>

#include <cerrno>
#include <sys/stat.h>
#include <unistd.h>

#include "Common.h"
// the parser stand-ins fill DataBase's private maps (test-only access)
#define private public
#include "DataBase.h"
#undef private
#include "AIEplace.h"

using namespace AIEplace;

namespace {

struct Pending {
    int n = 0;
    const float *w = nullptr, *h = nullptr, *x = nullptr, *y = nullptr;
    const uint8_t *fixed = nullptr;
    int n_nets = 0;
    const int32_t *net_ptr = nullptr, *pin_node = nullptr;
    float die_w = 0.f, die_h = 0.f;
};
Pending g_pend;  // the netlist the parser stand-ins hand over (one placer built at a time)

bool is_pad(int i) { return g_pend.fixed[i] && g_pend.w[i] * g_pend.h[i] == 0.f; }
std::string comp_name(int i) { return "c" + std::to_string(i); }
std::string pin_name(int i) { return "p" + std::to_string(i); }

struct Handle {
    Placer *placer = nullptr;
    std::vector<Node *> nodes;  // node i of the caller's netlist
};

double seconds_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

// ---- Limbo parser entry points: the netlist instead of files --------------
namespace LefParser {
bool read(LefDataBase &ldb, const std::string &) {
    auto &db = dynamic_cast<DataBase &>(ldb);
    for (int i = 0; i < g_pend.n; ++i)
        if (!is_pad(i)) db.mm_macros["m" + std::to_string(i)] = new MacroClass("m" + std::to_string(i), g_pend.w[i], g_pend.h[i]);
    return true;
}
}  // namespace LefParser

namespace DefParser {
bool read(DefDataBase &ddb, const std::string &) {
    auto &db = dynamic_cast<DataBase &>(ddb);
    db.set_def_unit(1);
    db.set_def_design("synthetic");
    db.m_die_area = Box<position_type>(Position<position_type>(0.f, 0.f), Position<position_type>(g_pend.die_w, g_pend.die_h));
    for (int i = 0; i < g_pend.n; ++i) {
        if (is_pad(i)) {
            DefParser::Pin p;
            p.reset();
            p.pin_name = pin_name(i);
            p.direct = "INPUT";
            p.status = "FIXED";
            p.origin[0] = (int32_t)g_pend.x[i];
            p.origin[1] = (int32_t)g_pend.y[i];
            p.vBbox.push_back({0, 0, 0, 0});
            db.add_def_pin(p);
        } else {
            DefParser::Component c;
            c.reset();
            c.comp_name = comp_name(i);
            c.macro_name = "m" + std::to_string(i);
            c.status = g_pend.fixed[i] ? "FIXED" : "PLACED";
            c.origin[0] = (int32_t)g_pend.x[i];
            c.origin[1] = (int32_t)g_pend.y[i];
            db.add_def_component(c);
        }
    }
    for (int e = 0; e < g_pend.n_nets; ++e) {
        DefParser::Net net;
        net.reset();
        net.net_name = "n" + std::to_string(e);
        for (int q = g_pend.net_ptr[e]; q < g_pend.net_ptr[e + 1]; ++q) {
            const int i = g_pend.pin_node[q];
            if (is_pad(i))
                net.vNetPin.emplace_back("PIN", pin_name(i));
            else
                net.vNetPin.emplace_back(comp_name(i), "A");
        }
        db.add_def_net(net);
    }
    return true;
}
}  // namespace DefParser

// ---- LEF-library members referenced but never reached --------------------
namespace LefDefParser {
const char *lefiMacro::name() const { return ""; }
double lefiMacro::sizeX() const { return 0.0; }
double lefiMacro::sizeY() const { return 0.0; }
void lefiArray::print(FILE *) const {}
void lefiDensity::print(FILE *) const {}
void lefiIRDrop::print(FILE *) const {}
void lefiLayer::print(FILE *) const {}
void lefiMacro::print(FILE *) const {}
void lefiMaxStackVia::print(FILE *) const {}
void lefiMinFeature::print(FILE *) const {}
void lefiObstruction::print(FILE *) const {}
void lefiPin::print(FILE *) const {}
void lefiProp::print(FILE *) const {}
void lefiSite::print(FILE *) const {}
void lefiSpacing::print(FILE *) const {}
void lefiUnits::print(FILE *) const {}
void lefiUseMinSpacing::print(FILE *) const {}
void lefiVia::print(FILE *) const {}
void lefiViaRule::print(FILE *) const {}
}  // namespace LefDefParser

// ---- cairo: the visualiser's calls as no-ops -------------------------------
extern "C" {
cairo_surface_t *cairo_image_surface_create(cairo_format_t, int, int) { return nullptr; }
cairo_t *cairo_create(cairo_surface_t *) { return nullptr; }
void cairo_scale(cairo_t *, double, double) {}
void cairo_rectangle(cairo_t *, double, double, double, double) {}
void cairo_set_source_rgb(cairo_t *, double, double, double) {}
void cairo_paint(cairo_t *) {}
void cairo_set_line_width(cairo_t *, double) {}
void cairo_stroke(cairo_t *) {}
void cairo_fill(cairo_t *) {}
int cairo_surface_write_to_png(cairo_surface_t *, const char *) { return 0; }
}

extern "C" {

// The reference placer on a CSR netlist: components (area > 0 or not fixed)
// and IO pins (fixed, zero area), nets through the DEF callbacks, the die
// box, the config keys Placer::Placer reads.  workdir: a writable scratch
// directory.  Node positions are set from x, y as floats after construction.
void *ref_placer_create(int n, const float *w, const float *h, const float *x, const float *y, const uint8_t *fixed,
                        int n_nets, const int32_t *net_ptr, const int32_t *pin_node, float die_w, float die_h,
                        int bins, float gamma, float learning_rate, float global_lambda, const char *workdir) {
    const std::string wd(workdir);
    const std::string design = wd + "/design";
    for (const std::string &d : {wd, wd + "/host", design})
        if (mkdir(d.c_str(), 0755) != 0 && errno != EEXIST) return nullptr;
    {
        std::ofstream(design + "/cells.lef") << "";
        std::ofstream(design + "/floorplan.def") << "";
        std::ofstream cfg(wd + "/host/config_aieplace.json");
        cfg << "{\"params\": {\"gamma\": " << gamma << ", \"init_learning_rate\": " << learning_rate
            << ", \"init_global_lambda\": " << global_lambda << ", \"bins_per_row\": " << bins
            << ", \"input_filepath\": \"" << design << "\", \"use_aie\": false, \"wirelength_method\": \"HPWL\""
            << ", \"max_iterations\": 1}}\n";
    }
    g_pend = Pending{n, w, h, x, y, fixed, n_nets, net_ptr, pin_node, die_w, die_h};
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd) || chdir(wd.c_str()) != 0) return nullptr;
    Handle *hd = new Handle;
    hd->placer = new Placer("none");
    if (chdir(cwd) != 0) return nullptr;
    // the node classification of Placer::initializePlacement (AIEplace.cpp:200-216),
    // without its random positions
    Placer &p = *hd->placer;
    const float bin_area_16th = p.grid.getBinWidth() * p.grid.getBinHeight() / 16;
    hd->nodes.resize((size_t)n, nullptr);
    for (int i = 0; i < n; ++i) {
        if (is_pad(i)) {
            hd->nodes[(size_t)i] = p.db.mm_pins[pin_name(i)];
        } else {
            Component *c = p.db.mm_components[comp_name(i)];
            c->checkIfLarge(bin_area_16th);
            hd->nodes[(size_t)i] = c;
        }
        hd->nodes[(size_t)i]->setPosition(Position<position_type>(x[i], y[i]));
    }
    return hd;
}

void ref_placer_destroy(void *h) {
    Handle *hd = (Handle *)h;
    delete hd->placer;  // (the reference never frees its DataBase objects)
    delete hd;
}

int ref_placer_set_positions(void *h, const float *x, const float *y) {
    Handle *hd = (Handle *)h;
    for (size_t i = 0; i < hd->nodes.size(); ++i) hd->nodes[i]->setPosition(Position<position_type>(x[i], y[i]));
    return 0;
}

// Placer::iterationReset + computeAllPartials_CPU (nets of degree 2..8);
// each node's accumulated terms_cpu.partials.
int ref_placer_partials(void *h, float *gx, float *gy, double *seconds) {
    Handle *hd = (Handle *)h;
    hd->placer->iterationReset();
    const auto t0 = std::chrono::steady_clock::now();
    hd->placer->computeAllPartials_CPU();
    if (seconds) *seconds = seconds_since(t0);
    for (size_t i = 0; i < hd->nodes.size(); ++i) {
        gx[i] = hd->nodes[i]->terms_cpu.partials.x;
        gy[i] = hd->nodes[i]->terms_cpu.partials.y;
    }
    return 0;
}

// Placer::iterationReset + computeOverlaps; Grid::getRho (x-major M*M) and
// Grid::computeTotalOverflow.
int ref_placer_overlaps(void *h, float *rho, double *overflow, double *seconds) {
    Handle *hd = (Handle *)h;
    Placer &p = *hd->placer;
    p.iterationReset();
    const auto t0 = std::chrono::steady_clock::now();
    p.computeOverlaps();
    if (seconds) *seconds = seconds_since(t0);
    const std::vector<std::vector<float> > r = p.grid.getRho();
    const int M = p.grid.getBinsPerRow();
    for (int c = 0; c < M; ++c)
        for (int k = 0; k < M; ++k) rho[(size_t)c * M + k] = r[(size_t)c][(size_t)k];
    if (overflow) *overflow = p.grid.computeTotalOverflow();
    return 0;
}

// The host's DCT field path at the current positions: iterationReset,
// computeOverlaps, compute_a_uv_DCT, compute_eField_DCT; each bin's eField
// (x-major).  The seconds cover the two field functions only.
int ref_placer_fields_dct(void *h, float *ex, float *ey, double *seconds) {
    Handle *hd = (Handle *)h;
    Placer &p = *hd->placer;
    p.iterationReset();
    p.computeOverlaps();
    const auto t0 = std::chrono::steady_clock::now();
    p.compute_a_uv_DCT();
    p.compute_eField_DCT();
    if (seconds) *seconds = seconds_since(t0);
    const int M = p.grid.getBinsPerRow();
    for (int c = 0; c < M; ++c)
        for (int k = 0; k < M; ++k) {
            ex[(size_t)c * M + k] = p.grid.getBin(c, k).eField.x;
            ey[(size_t)c * M + k] = p.grid.getBin(c, k).eField.y;
        }
    return 0;
}

// Placer::nudgeNode for every component with the caller's bin fields (x-major)
// and wirelength partials (partials_aie, which nudgeNode reads), every bin's
// local weight 1: iterationReset and computeOverlaps at the current positions,
// then each component is moved from the origin, so that its new position is
// nudgeNode's move exactly: learning_rate min(W, H) (global_lambda F - partial),
// F = sum over its bins of overlap / bin area x eField.  Pins are not moved
// (AIEplace.cpp:996-999); their entries are zero.
int ref_placer_nudge(void *h, const float *ex, const float *ey, const float *px, const float *py, float *mx, float *my,
                     double *seconds) {
    Handle *hd = (Handle *)h;
    Placer &p = *hd->placer;
    p.iterationReset();
    p.computeOverlaps();
    const int M = p.grid.getBinsPerRow();
    for (int c = 0; c < M; ++c)
        for (int k = 0; k < M; ++k) {
            Bin &b = p.grid.getBin(c, k);
            b.eField.x = ex[(size_t)c * M + k];
            b.eField.y = ey[(size_t)c * M + k];
            b.lambda = 1.f;
        }
    std::vector<Position<position_type> > keep(hd->nodes.size());
    for (size_t i = 0; i < hd->nodes.size(); ++i) {
        keep[i] = Position<position_type>(hd->nodes[i]->getX(), hd->nodes[i]->getY());
        hd->nodes[i]->partials_aie.x = px[i];
        hd->nodes[i]->partials_aie.y = py[i];
        hd->nodes[i]->setPosition(Position<position_type>(0.f, 0.f));
    }
    const auto t0 = std::chrono::steady_clock::now();
    p.nudgeAllNodes();
    if (seconds) *seconds = seconds_since(t0);
    for (size_t i = 0; i < hd->nodes.size(); ++i) {
        mx[i] = hd->nodes[i]->getX();
        my[i] = hd->nodes[i]->getY();
        hd->nodes[i]->setPosition(keep[i]);
    }
    return 0;
}

// The reference CPU loop's own field solve, Placer::computeElectricFields_CPU
// (compute_a_uv_naive / compute_eField_naive, AIEplace.cpp:679-750): iterationReset
// and computeOverlaps at the current positions, then the two naive passes
// (O(M^4)); each bin's eField (x-major).  The seconds cover the two passes.
int ref_placer_fields_naive(void *h, float *ex, float *ey, double *seconds) {
    Handle *hd = (Handle *)h;
    Placer &p = *hd->placer;
    p.iterationReset();
    p.computeOverlaps();
    const auto t0 = std::chrono::steady_clock::now();
    p.computeElectricFields_CPU();
    if (seconds) *seconds = seconds_since(t0);
    const int M = p.grid.getBinsPerRow();
    for (int c = 0; c < M; ++c)
        for (int k = 0; k < M; ++k) {
            ex[(size_t)c * M + k] = p.grid.getBin(c, k).eField.x;
            ey[(size_t)c * M + k] = p.grid.getBin(c, k).eField.y;
        }
    return 0;
}

// `iters` passes of the loop body of Placer::run (AIEplace.cpp:55-76) from the
// current positions and iteration count: the learning-rate and lambda
// schedule, performIteration (:9-40, CPU branches: computeAllPartials_CPU,
// computeOverlaps, computeElectricFields_CPU, nudgeAllNodes,
// printIterationResults), iteration + 1.  Placer::run's random initial
// placement and final report are left out.
int ref_placer_iterate(void *h, int iters, double *seconds) {
    Placer &p = *((Handle *)h)->placer;
    const auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < iters; ++i) {
        if (p.iteration % 100 == 0) p.learning_rate *= 0.8;
        if (p.iteration % 10 == 0) p.global_lambda *= 1.01;
        p.performIteration();
        p.iteration++;
    }
    if (seconds) *seconds = seconds_since(t0);
    return 0;
}

int ref_placer_get_positions(void *h, float *x, float *y) {
    Handle *hd = (Handle *)h;
    for (size_t i = 0; i < hd->nodes.size(); ++i) {
        x[i] = hd->nodes[i]->getX();
        y[i] = hd->nodes[i]->getY();
    }
    return 0;
}

// DataBase::computeTotalWirelength("HPWL") at the current positions.
double ref_placer_hpwl(void *h) {
    Handle *hd = (Handle *)h;
    return hd->placer->db.computeTotalWirelength("HPWL");
}

}  // extern "C"
