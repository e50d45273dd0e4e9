// aieplace: the placer as a program.  Counterpart of the reference host's
// main (vck5000/host/src/main.cpp:3-40) and Placer::run (AIEplace.cpp:44-76)
// with its configuration file (host/config_aieplace.json, AIEplace.cpp:87-109)
// and the DEF write-back (DataBase::writeDEF, DataBase.cpp:538-655):
//
//   aieplace <config.json>
//
// reads the design directory the config names (*.lef + floorplan.def),
// places it on the GPU until the overflow target or max_iterations, writes
// <output_filepath>/<design>.def and prints one JSON line with the result.
// Built against include/aieplace.h only.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/aieplace.h"

static int fail(const char *what, int st) {
    const char *detail = ap_last_error();
    std::fprintf(stderr, "aieplace: %s: %s%s%s\n", what, ap_status_string(st), detail && *detail ? ": " : "",
                 detail ? detail : "");
    return 1;
}

int main(int argc, char **argv) {
    if (argc != 2 || !std::strcmp(argv[1], "-h") || !std::strcmp(argv[1], "--help")) {
        std::fprintf(stderr, "usage: aieplace <config.json>\n");
        return 2;
    }
    ap_params p;
    ap_run_config run;
    int st = ap_run_config_read(argv[1], &p, &run);
    if (st != AP_OK) return fail("config", st);
    if (!run.input_dir[0]) {
        std::fprintf(stderr, "aieplace: the config names no input_filepath\n");
        return 2;
    }
    ap_design *d = nullptr;
    if ((st = ap_design_read_dir(run.input_dir, run.size_mode, &d)) != AP_OK) return fail("design", st);
    ap_netlist nl;
    ap_design_netlist(d, &nl);
    ap_design_info info;
    ap_design_get_info(d, &info);
    if (run.filler_cells) p.filler_cells = 1;
    ap_handle *h = nullptr;
    if ((st = ap_create(&nl, &p, &h)) != AP_OK) return fail("ap_create", st);
    if (run.log_path[0] && (st = ap_set_log(h, run.log_path, 1 << 16)) != AP_OK) return fail("ap_set_log", st);
    const float bin_w = (info.die_xh - info.die_xl) / (float)p.bins_x;
    const float sigma = run.init_sigma > 0.f ? run.init_sigma : bin_w;
    if ((st = ap_init_seeded(h, run.seed, sigma)) != AP_OK) return fail("ap_init_seeded", st);
    int32_t iterations = 0;
    if ((st = ap_run(h, &iterations)) != AP_OK) return fail("ap_run", st);
    ap_stats s;
    if ((st = ap_get_stats(h, &s)) != AP_OK) return fail("ap_get_stats", st);
    std::vector<float> x((size_t)nl.num_nodes), y((size_t)nl.num_nodes);
    if ((st = ap_get_positions(h, x.data(), y.data())) != AP_OK) return fail("ap_get_positions", st);
    const std::string out = std::string(run.output_dir) + "/" + ap_design_name(d) + ".def";
    if ((st = ap_design_write_def(d, x.data(), y.data(), out.c_str())) != AP_OK) return fail("write DEF", st);
    std::printf("{\"design\": \"%s\", \"nodes\": %d, \"nets\": %d, \"iterations\": %d, \"evals\": %d, "
                "\"%s\": %.17g, \"overflow\": %.17g, \"overflow_abs\": %.17g, \"status\": %d, \"def\": \"%s\"}\n",
                ap_design_name(d), nl.num_nodes, nl.num_nets, iterations, s.evals,
                run.wirelength_method ? "wa_wirelength" : "hpwl", run.wirelength_method ? s.wa_wirelength : s.hpwl,
                s.overflow, s.overflow_abs, s.status, out.c_str());
    ap_destroy(h);
    ap_design_destroy(d);
    return 0;
}
