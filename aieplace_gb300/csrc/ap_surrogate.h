// Learned density-to-field surrogate: shared definitions (see k_surrogate.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "ap_kernels.h"

namespace ap {

constexpr int kMaxCh = 32;     // channel limit of the conv kernels (registers per pixel)
constexpr int kTile = 16;      // weight-gradient tile (kTile x kTile output pixels)
constexpr int kSurrLayers = 4;

struct SurrLayer {
    int cin, cout, k, relu;
    size_t w_off, b_off;  // into the flat parameter vector
};

// Network description and training state (one per ap_surrogate).
struct SurrNet {
    int f;          // pooling factor: coarse grid R = M / f
    int cin0, cout;  // f^2 + 2 inputs, 2 f^2 outputs
    int width;      // hidden channels
    SurrLayer L[kSurrLayers];
    int n_params;
    float *d_params = nullptr, *d_grad = nullptr, *d_m = nullptr, *d_v = nullptr;
    int adam_t = 0;
};

// Per-handle inference buffers of an attached surrogate.
struct SurrState {
    int R = 0, M = 0;
    FieldSolver coarse{};
    float *d_pool = nullptr, *d_cex = nullptr, *d_cey = nullptr;  // R x R
    // tcgen05 coarse solve (R a multiple of 128): pooled density as BF16 hi/lo
    int tc = 0;
    __nv_bfloat16 *d_phi = nullptr, *d_plo = nullptr;
    float *d_scale = nullptr;                                     // [1]
    float *d_x0 = nullptr, *d_act[2] = {nullptr, nullptr}, *d_y = nullptr;
    float *d_sex = nullptr, *d_sey = nullptr;  // M x M: the surrogate field of a judged trial
    float *d_part = nullptr;
    unsigned int *d_cnt = nullptr;  // [4] last-block counters
    int use_net = 1;
};

// Host helpers (k_surrogate.cu).  Each enqueues work on `st`; gate/mask as
// for the field solvers (null gate: always run).
int surr_state_init(SurrState &ss, const SurrNet &net, int M, float bin_ratio);
void surr_state_free(SurrState &ss);
// pool -> coarse solve -> scale -> network input (ss.d_x0)
void surr_enqueue_input(const SurrNet &net, SurrState &ss, const float *d_f32, const __nv_bfloat16 *d_hi,
                        const __nv_bfloat16 *d_lo, const int *gate, int mask, cudaStream_t st,
                        bool with_net_input = true);
// full surrogate field into (ex, ey), or into ss.d_sex/d_sey on judged trials
void surr_enqueue_field(const SurrNet &net, SurrState &ss, const float *d_f32, const __nv_bfloat16 *d_hi,
                        const __nv_bfloat16 *d_lo, float *ex, float *ey, const int *gate, cudaStream_t st);
// judged trials: relative error of ss.d_sex/d_sey against (ex, ey) -> sc
void surr_enqueue_judge(SurrState &ss, const float *ex, const float *ey, DevScalars *sc, const int *gate,
                        cudaStream_t st);
// target of the current exact field + per-sample scale and norm into slot `slot`
void surr_enqueue_sample(const SurrNet &net, SurrState &ss, float *X, float *T, float *s_slot, float *e2_slot,
                         const float *ex, const float *ey, cudaStream_t st);


}  // namespace ap

// Opaque handle of the C ABI: network, sample store, training scratch.
struct ap_surrogate {
    ap::SurrNet net;
    int R = 0, cap = 0, n = 0;          // sample resolution, capacity, count
    float *d_X = nullptr, *d_T = nullptr;  // [cap][cin0][R][R], [cap][cout][R][R]
    float *d_s = nullptr, *d_e2 = nullptr;  // per sample: field scale, sum of exact E^2
    // training / host-call scratch, sized for tB maps of tR x tR
    int tB = 0, tR = 0;
    float *d_a[ap::kSurrLayers + 1] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    float *d_g[2] = {nullptr, nullptr};
    float *d_tb = nullptr, *d_wpart = nullptr, *d_lpart = nullptr, *d_loss = nullptr;
    float *d_w = nullptr;  // per-map weights of the relative training loss
    int *d_sel = nullptr;
    unsigned int *d_cnt = nullptr;
};
