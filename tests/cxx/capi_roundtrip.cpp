// A C++ caller of the placement library through include/aieplace.h only: the
// sequence a host placer runs (netlist -> create -> initial placement ->
// host-buffer steps -> readout -> destroy).  tests/test_capi_cxx.py builds it
// with g++ against the header, links libaieplace_gb300.so, runs it and
// compares its results with the Python binding's.
//
//   capi_roundtrip <cells> <nets> <macros> <pads> <unit_cells> <degree_mix>
//                  <locality> <window> <target_density> <die_side> <seed>
//                  <bins> <solver 0|1> <init_seed> <steps> <out.bin>
//
// out.bin: the final x and y of every node (float32, netlist order); stdout:
// one line "hpwl overflow overflow_abs iteration status".
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "aieplace.h"

static int fail(const char *what, int st) {
    std::fprintf(stderr, "%s: %s (%d)\n", what, ap_status_string(st), st);
    return 1;
}

int main(int argc, char **argv) {
    if (argc != 17) {
        std::fprintf(stderr, "usage: see the header of capi_roundtrip.cpp\n");
        return 2;
    }
    if (ap_abi_version() != AP_ABI_VERSION) return fail("abi version", AP_ERR_UNSUPPORTED);
    ap_synth_config cfg{};
    cfg.num_cells = std::atoi(argv[1]);
    cfg.num_nets = std::atoi(argv[2]);
    cfg.num_macros = std::atoi(argv[3]);
    cfg.num_pads = std::atoi(argv[4]);
    cfg.unit_cells = std::atoi(argv[5]);
    cfg.degree_mix = std::atoi(argv[6]);
    cfg.locality = (float)std::atof(argv[7]);
    cfg.window = std::atoi(argv[8]);
    cfg.macro_area_min = 20.f;
    cfg.macro_area_max = 200.f;
    cfg.target_density = (float)std::atof(argv[9]);
    cfg.die_side = (float)std::atof(argv[10]);
    cfg.seed = std::strtoull(argv[11], nullptr, 10);
    const int bins = std::atoi(argv[12]), solver = std::atoi(argv[13]);
    const uint64_t init_seed = std::strtoull(argv[14], nullptr, 10);
    const int steps = std::atoi(argv[15]);

    int32_t nn = 0, ne = 0, np = 0;
    int st = ap_synth_counts(&cfg, &nn, &ne, &np);
    if (st != AP_OK) return fail("ap_synth_counts", st);
    std::vector<int32_t> net_ptr(ne + 1), pin_node(np > 0 ? np : 1);
    std::vector<float> w(nn), h(nn), x(nn), y(nn);
    std::vector<uint8_t> fixed(nn);
    float die[4];
    st = ap_synth_generate(&cfg, net_ptr.data(), pin_node.data(), w.data(), h.data(), x.data(), y.data(),
                           fixed.data(), die);
    if (st != AP_OK) return fail("ap_synth_generate", st);

    ap_netlist nl{nn, ne, np, net_ptr.data(), pin_node.data(), w.data(), h.data(), x.data(), y.data(),
                  fixed.data(), die[0], die[1], die[2], die[3]};
    ap_params p;
    ap_params_default(&p);
    p.bins_x = p.bins_y = bins;
    p.target_density = cfg.target_density;
    p.field_solver = solver;
    ap_handle *hd = nullptr;
    st = ap_create(&nl, &p, &hd);
    if (st != AP_OK) return fail("ap_create", st);
    st = ap_init_seeded(hd, init_seed, 1.0f);
    if (st != AP_OK) return fail("ap_init_seeded", st);
    // the host owns the positions, as the reference host does (Node::m_pos)
    st = ap_get_positions(hd, x.data(), y.data());
    if (st != AP_OK) return fail("ap_get_positions", st);
    ap_stats s{};
    for (int i = 0; i < steps; ++i) {
        st = ap_step_host(hd, x.data(), y.data(), x.data(), y.data(), &s);
        if (st != AP_OK) return fail("ap_step_host", st);
    }
    double hpwl = 0, ov = 0, ov_abs = 0;
    if ((st = ap_hpwl(hd, &hpwl)) != AP_OK) return fail("ap_hpwl", st);
    if ((st = ap_overflow(hd, &ov, &ov_abs)) != AP_OK) return fail("ap_overflow", st);
    std::vector<float> gx(nn), gy(nn);
    if ((st = ap_get_positions(hd, gx.data(), gy.data())) != AP_OK) return fail("ap_get_positions", st);
    for (int32_t i = 0; i < nn; ++i)
        if (gx[i] != x[i] || gy[i] != y[i]) return fail("positions of the last host step", AP_ERR_STATE);
    if ((st = ap_destroy(hd)) != AP_OK) return fail("ap_destroy", st);

    FILE *f = std::fopen(argv[16], "wb");
    if (!f) return fail("open output", AP_ERR_INVALID_ARG);
    std::fwrite(x.data(), sizeof(float), x.size(), f);
    std::fwrite(y.data(), sizeof(float), y.size(), f);
    std::fclose(f);
    std::printf("%.17g %.17g %.17g %d %d\n", hpwl, ov, ov_abs, s.iteration, s.status);
    return 0;
}
