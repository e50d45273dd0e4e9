// ref_shim.cpp -- extern "C" entry points onto the reference's own CPU code.
//
// TEST INFRASTRUCTURE ONLY.  Built by `make -C oracle ref` against the
// reference checkout; loaded by tests (and the CPU baseline when present) to
// pin the oracle restatement to the reference functions themselves:
//   Grid::computeBinOverlaps / getRho / computeTotalOverflow (Grid.cpp:38-151)
//   Net::computeWirelength_HPWL                            (Net.cpp:117-155)
//   DCT_naive / IDCT_naive / IDXST_naive                   (DCT.cpp:24-82)
//   replace::FFT::doFFT                                    (fft_replace/fft.cpp:204-299)
#include <cstdint>
#include <iostream>
#include <vector>

#include "Component.h"
#include "DCT.h"
#include "Grid.h"
#include "MacroClass.h"
#include "Net.h"
#include "fft.h"

using namespace AIEplace;

extern "C" {

// Density map of the given nodes through Grid::computeBinOverlaps, after the
// node classification Placer::initializePlacement does (AIEplace.cpp:200-216).
// rho is x-major M*M (Grid::getRho()[col][row]); returns computeTotalOverflow.
int ref_density(int n, const float *x, const float *y, const float *w, const float *h,
                float die_w, float die_h, int M, float *rho, double *overflow) {
    Grid grid(Box<position_type>(0.f, 0.f, die_w, die_h), M, M);
    grid.iterationReset();  // Bin::overlap starts uninitialised (Bin.h:65)
    std::vector<MacroClass> macros;
    macros.reserve((size_t)n);
    std::vector<Component *> comps((size_t)n, nullptr);
    const float bin_area_16th = grid.getBinWidth() * grid.getBinHeight() / 16;
    for (int i = 0; i < n; ++i) {
        macros.emplace_back("m", w[i], h[i]);
        comps[(size_t)i] = new Component("c");
        comps[(size_t)i]->setMacroClass(&macros.back());
        comps[(size_t)i]->setPosition(Position<position_type>(x[i], y[i]));
        comps[(size_t)i]->checkIfLarge(bin_area_16th);
    }
    for (int i = 0; i < n; ++i) grid.computeBinOverlaps(comps[(size_t)i]);
    std::vector<std::vector<float> > r = grid.getRho();
    for (int c = 0; c < M; ++c)
        for (int k = 0; k < M; ++k) rho[(size_t)c * M + k] = r[(size_t)c][(size_t)k];
    if (overflow) *overflow = grid.computeTotalOverflow();
    for (Component *cp : comps) delete cp;
    return 0;
}

// DataBase::computeTotalWirelength("HPWL") over a CSR netlist (DataBase.cpp:143-149).
double ref_hpwl(int n_nodes, int n_nets, const int32_t *net_ptr, const int32_t *pin_node,
                const float *x, const float *y) {
    std::vector<Node> nodes;
    nodes.reserve((size_t)n_nodes);
    for (int i = 0; i < n_nodes; ++i) {
        nodes.emplace_back("n");
        nodes.back().setPosition(Position<position_type>(x[i], y[i]));
    }
    double total = 0;
    for (int e = 0; e < n_nets; ++e) {
        if (net_ptr[e + 1] <= net_ptr[e]) continue;
        Net net("e");
        for (int p = net_ptr[e]; p < net_ptr[e + 1]; ++p) net.addNode(&nodes[(size_t)pin_node[p]]);
        total += net.computeWirelength("HPWL");
    }
    return total;
}

static void run_1d(std::vector<float> (*f)(std::vector<float>), int n, const float *in, float *out) {
    std::vector<float> v(in, in + n);
    std::vector<float> r = f(v);
    for (int i = 0; i < n; ++i) out[i] = r[(size_t)i];
}

void ref_dct(int n, const float *in, float *out) { run_1d(DCT_naive, n, in, out); }
void ref_idct(int n, const float *in, float *out) { run_1d(IDCT_naive, n, in, out); }
void ref_idxst(int n, const float *in, float *out) { run_1d(IDXST_naive, n, in, out); }

// replace::FFT::doFFT on an x-major M*M density map; its debug printing is
// muted by putting std::cout into a failed state for the call.
int ref_replace_field(int M, const float *density, float *phi, float *ex, float *ey) {
    replace::FFT fft(M, M, 1, 1);
    for (int x = 0; x < M; ++x)
        for (int y = 0; y < M; ++y) fft.updateDensity(x, y, density[(size_t)x * M + y]);
    std::ios_base::iostate st = std::cout.rdstate();
    std::cout.setstate(std::ios_base::badbit);
    fft.doFFT();
    std::cout.clear(st);
    for (int x = 0; x < M; ++x)
        for (int y = 0; y < M; ++y) {
            size_t k = (size_t)x * M + y;
            if (phi) phi[k] = fft.getElectroPhi(x, y);
            std::pair<float, float> e = fft.getElectroForce(x, y);
            ex[k] = e.first;
            ey[k] = e.second;
        }
    return 0;
}
}
