// Seeded synthetic netlists standing in for the LEF/DEF designs the reference
// host reads through Limbo (vck5000/host/src/DataBase.cpp:42-96).  The
// generator is deterministic across hosts: its PRNG is xoshiro256** seeded by
// splitmix64 and every draw is built from raw 64-bit outputs, so no
// implementation-defined std:: distribution is involved.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "../../include/aieplace.h"

namespace {

struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t z = seed;
        for (int i = 0; i < 4; ++i) {
            z += 0x9E3779B97F4A7C15ull;
            uint64_t t = z;
            t = (t ^ (t >> 30)) * 0xBF58476D1CE4E5B9ull;
            t = (t ^ (t >> 27)) * 0x94D049BB133111EBull;
            s[i] = t ^ (t >> 31);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        uint64_t r = rotl(s[1] * 5, 7) * 9;
        uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    // integer in [0, n)
    int64_t below(int64_t n) { return (int64_t)(uniform() * (double)n); }
    double normal() {
        double u1 = uniform();
        double u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

int draw_degree(Rng &r, int mix) {
    double u = r.uniform();
    if (mix == 0) {
        if (u < 0.70) return 2;
        if (u < 0.90) return 3;
        return 4;
    }
    if (u < 0.65) return 2;
    if (u < 0.85) return 3;
    if (u < 0.95) return 4 + (int)r.below(7);   // U[4,10]
    return 11 + (int)r.below(54);               // U[11,64]
}

bool valid(const ap_synth_config *c) {
    return c && c->num_cells > 0 && c->num_nets >= 0 && c->num_macros >= 0 &&
           c->num_pads >= 0 && c->window > 0 && c->locality >= 0.f && c->locality <= 1.f &&
           c->target_density > 0.f && c->macro_area_min >= 0.f &&
           c->macro_area_max >= c->macro_area_min;
}

// Degrees are drawn from a stream of their own so that counting pins does not
// require generating the whole netlist.
uint64_t degree_seed(uint64_t seed) { return seed ^ 0xD1B54A32D192ED03ull; }

}  // namespace

extern "C" int ap_synth_counts(const ap_synth_config *cfg, int32_t *num_nodes,
                               int32_t *num_nets, int32_t *num_pins) {
    if (!valid(cfg) || !num_nodes || !num_nets || !num_pins) return AP_ERR_INVALID_ARG;
    int64_t nodes = (int64_t)cfg->num_cells + cfg->num_macros + cfg->num_pads;
    if (nodes > INT32_MAX) return AP_ERR_INVALID_ARG;
    Rng rd(degree_seed(cfg->seed));
    int64_t pins = 0;
    for (int32_t e = 0; e < cfg->num_nets; ++e) {
        int d = draw_degree(rd, cfg->degree_mix);
        pins += std::min<int64_t>(d, nodes);
    }
    if (pins > INT32_MAX) return AP_ERR_INVALID_ARG;
    *num_nodes = (int32_t)nodes;
    *num_nets = cfg->num_nets;
    *num_pins = (int32_t)pins;
    return AP_OK;
}

extern "C" int ap_synth_generate(const ap_synth_config *cfg, int32_t *net_ptr, int32_t *pin_node,
                                 float *node_w, float *node_h, float *node_x, float *node_y,
                                 uint8_t *node_fixed, float *die) {
    int32_t n_nodes, n_nets, n_pins;
    int st = ap_synth_counts(cfg, &n_nodes, &n_nets, &n_pins);
    if (st != AP_OK) return st;
    if (!net_ptr || !pin_node || !node_w || !node_h || !node_x || !node_y || !node_fixed || !die)
        return AP_ERR_INVALID_ARG;

    const int32_t C = cfg->num_cells, F = cfg->num_macros, P = cfg->num_pads;
    Rng rs(cfg->seed);                    // sizes
    Rng rm(cfg->seed ^ 0x5851F42D4C957F2Dull);  // macro placement
    Rng rp(cfg->seed ^ 0x2545F4914F6CDD1Dull);  // pins
    Rng ri(cfg->seed ^ 0x9FB21C651E98DF25ull);  // initial positions
    Rng rd(degree_seed(cfg->seed));

    // ---- sizes
    double cell_area = 0.0, macro_area = 0.0;
    for (int32_t i = 0; i < C; ++i) {
        float w = 1.0f, h = 1.0f;
        if (!cfg->unit_cells) w = (float)std::exp(std::log(2.0) + 0.5 * rs.normal());
        node_w[i] = w;
        node_h[i] = h;
        node_fixed[i] = 0;
        cell_area += (double)w * (double)h;
    }
    for (int32_t j = 0; j < F; ++j) {
        double area = cfg->macro_area_min + (cfg->macro_area_max - cfg->macro_area_min) * rs.uniform();
        double aspect = 0.5 + 1.5 * rs.uniform();  // w/h in [0.5, 2]
        double w = std::sqrt(area * aspect);
        double h = area / w;
        node_w[C + j] = (float)w;
        node_h[C + j] = (float)h;
        node_fixed[C + j] = 1;
        macro_area += (double)node_w[C + j] * (double)node_h[C + j];
    }
    for (int32_t k = 0; k < P; ++k) {
        node_w[C + F + k] = 0.f;
        node_h[C + F + k] = 0.f;
        node_fixed[C + F + k] = 1;
    }

    // ---- die
    double side = cfg->die_side > 0.f ? (double)cfg->die_side
                                       : std::sqrt(cell_area / cfg->target_density + macro_area);
    float W = (float)std::ceil(side), H = W;
    die[0] = 0.f;
    die[1] = 0.f;
    die[2] = W;
    die[3] = H;

    // ---- macros: rejection sampling against a uniform hash of placed boxes
    {
        const double cell = 32.0;
        const int gx = std::max(1, (int)std::ceil(W / cell)), gy = std::max(1, (int)std::ceil(H / cell));
        std::vector<std::vector<int32_t>> hash((size_t)gx * gy);
        for (int32_t j = 0; j < F; ++j) {
            const int32_t id = C + j;
            const double w = node_w[id], h = node_h[id];
            double x = 0, y = 0;
            bool placed = false;
            for (int attempt = 0; attempt < 4096 && !placed; ++attempt) {
                x = std::floor(rm.uniform() * std::max(0.0, W - w));
                y = std::floor(rm.uniform() * std::max(0.0, H - h));
                int cx0 = std::max(0, (int)(x / cell) - 1), cx1 = std::min(gx - 1, (int)((x + w) / cell) + 1);
                int cy0 = std::max(0, (int)(y / cell) - 1), cy1 = std::min(gy - 1, (int)((y + h) / cell) + 1);
                bool clash = false;
                for (int cx = cx0; cx <= cx1 && !clash; ++cx)
                    for (int cy = cy0; cy <= cy1 && !clash; ++cy)
                        for (int32_t o : hash[(size_t)cx * gy + cy]) {
                            if (x < node_x[o] + node_w[o] && node_x[o] < x + w && y < node_y[o] + node_h[o] &&
                                node_y[o] < y + h) {
                                clash = true;
                                break;
                            }
                        }
                placed = !clash;
            }
            // a macro that found no free spot after 4096 draws keeps its last
            // draw; the die is sized so this does not happen at the shipped presets
            node_x[id] = (float)x;
            node_y[id] = (float)y;
            int cx = std::min(gx - 1, (int)(x / cell)), cy = std::min(gy - 1, (int)(y / cell));
            hash[(size_t)cx * gy + cy].push_back(id);
        }
    }

    // ---- IO pads evenly on the boundary, counter-clockwise from (0,0)
    for (int32_t k = 0; k < P; ++k) {
        double t = (k + 0.5) / P * 2.0 * ((double)W + H);
        double x, y;
        if (t < W) { x = t; y = 0; }
        else if (t < (double)W + H) { x = W; y = t - W; }
        else if (t < 2.0 * W + H) { x = W - (t - W - H); y = H; }
        else { x = 0; y = H - (t - 2.0 * W - H); }
        node_x[C + F + k] = (float)x;
        node_y[C + F + k] = (float)y;
    }

    // ---- movable initial positions: die centre + N(0, 1 site)
    for (int32_t i = 0; i < C; ++i) {
        node_x[i] = (float)(0.5 * W + ri.normal());
        node_y[i] = (float)(0.5 * H + ri.normal());
    }

    // ---- nets: anchor uniform, each pin local (window) with prob `locality`
    int64_t p = 0;
    net_ptr[0] = 0;
    std::vector<int32_t> cur;
    for (int32_t e = 0; e < n_nets; ++e) {
        int d = (int)std::min<int64_t>(draw_degree(rd, cfg->degree_mix), n_nodes);
        int64_t anchor = rp.below(n_nodes);
        cur.clear();
        for (int q = 0; q < d; ++q) {
            int32_t node = -1;
            for (int attempt = 0; attempt < 64; ++attempt) {
                int64_t cand;
                if (rp.uniform() < cfg->locality) {
                    cand = anchor - cfg->window / 2 + rp.below(cfg->window);
                    if (cand < 0) cand += n_nodes;
                    if (cand >= n_nodes) cand -= n_nodes;
                    if (cand < 0 || cand >= n_nodes) cand = rp.below(n_nodes);
                } else {
                    cand = rp.below(n_nodes);
                }
                if (std::find(cur.begin(), cur.end(), (int32_t)cand) == cur.end()) {
                    node = (int32_t)cand;
                    break;
                }
            }
            if (node < 0) {  // dense duplicates: take the next unused index
                int64_t cand = anchor;
                while (std::find(cur.begin(), cur.end(), (int32_t)cand) != cur.end())
                    cand = (cand + 1) % n_nodes;
                node = (int32_t)cand;
            }
            cur.push_back(node);
        }
        for (int32_t v : cur) pin_node[p++] = v;
        net_ptr[e + 1] = (int32_t)p;
    }
    return p == n_pins ? AP_OK : AP_ERR_INVALID_ARG;
}
