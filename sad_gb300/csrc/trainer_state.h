// trainer_state.h -- the state of one fit on the device (sad_trainer of the C ABI),
// shared by the single-image trainer (trainer.cu) and the lockstep batch of fits
// (batch.cu), which drives many trainers' buffers with batched launches.
#pragma once

#include <chrono>
#include <vector>

#include "common.cuh"
#include "host_common.h"
#include "kernels.h"
#include "tuner.h"

namespace sad {

struct IterPlan {
    uint8_t upd, dens, prune;
    uint32_t split_k, prune_k;
};

}  // namespace sad

struct sad_trainer {
    sad_train_config_t cfg;
    int w = 0, h = 0, cw = 0, ch = 0, ds = 1;
    float inv_s2 = 0.0f;
    float prune_pct = 0.0f, densify_pct = 0.0f;
    uint32_t cap = 0, n = 0;
    int active = 0;
    int iter = 0;
    int passes = 1;
    int cur = 0;
    bool hilbert_ready = false;
    uint32_t hilbert_count = 0;
    bool have_mask = false;
    float mask_sum = 0.0f;
    uint32_t pow2 = 1, stages = 0;
    std::vector<sad::IterPlan> plan;

    float* target = nullptr;
    float* mask = nullptr;
    sad::Site* sites = nullptr;
    sad::SiteGeom* geom = nullptr;
    sad::SiteColor* color = nullptr;
    sad::SiteGeom* vgeom = nullptr;
    float* adam = nullptr;
    // [cap][12] 64-bit fixed-point records: 10 gradients, removal delta, sentinel count
    long long* grads = nullptr;
    float removal_mul = 1.0f;
    float* tau_a = nullptr;
    float* tau_b = nullptr;
    uint32_t* tau_nbr = nullptr;  // [cap][8] neighbour lists of the tau passes
    float* tau_raw = nullptr;
    // stream compaction of the active set: ascending active slots (state->n_alive of them),
    // walked by the per-site kernels; rebuilt after init, densify and every prune
    uint32_t* alive = nullptr;
    uint32_t* alive_blocks = nullptr;
    uint32_t alive_hint = 0;  // thread count of the per-site kernels' grids
    uint32_t* pairs = nullptr;
    void* sort_temp = nullptr;
    uint32_t* idx = nullptr;
    uint32_t* cand0[3] = {nullptr, nullptr, nullptr};
    uint32_t* cand1[3] = {nullptr, nullptr, nullptr};
    uint32_t* tmap_mem[3] = {nullptr, nullptr, nullptr};
    sad::TileMap tmap[3] = {};  // tile registration of each candidate field
    uint32_t* horder = nullptr;
    uint32_t* hpos = nullptr;
    uint32_t* hpairs = nullptr;
    uint32_t hpadded = 0;
    float* stats = nullptr;         // 8 x cap
    long long* stats_fix = nullptr;  // 8 x cap, zero between densify steps
    float* render = nullptr;
    uint32_t* packed = nullptr;   // [cap][4] 16-byte inference sites
    float* packed_quant = nullptr;  // sad_packed_quant_t
    long long* metric = nullptr;  // fixed-point squared-error sum (reproducible PSNR)
    uint32_t* count = nullptr;
    sad::DevState* state = nullptr;
    uint32_t* prune_k = nullptr;
    void* init_temp = nullptr;
    void* slab = nullptr;       // device memory of every buffer above
    size_t slab_bytes = 0;
    bool owns_slab = false;

    cudaStream_t st = nullptr, side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaGraphExec_t graphs[2][2][3] = {};
    uint64_t graph_kernels[2][2][3] = {};  // kernel launches one replay runs
    // a whole refresh window (a refresh iteration and the iterations up to the next one, no
    // densify or prune step) per start field: one replay, and programmatic dependent launch
    // across its iteration boundaries
    cudaGraphExec_t wgraphs[3] = {};
    uint64_t wgraph_kernels[3] = {};
    bool timing = false;
    std::vector<cudaEvent_t> tev;
    size_t tev_used = 0;
    double grad_ms = 0.0;
    int grad_launches = 0;
    sad::ShapeTuner tuner;  // tile-table shape rule, tuned while the fit runs
    std::chrono::steady_clock::time_point t0;
};

namespace sad {
// The field a candidate refresh of `passes` VPT passes from field src ends in, the Hilbert
// order build and the VPT parameters of a trainer.
int refresh_target_field(int passes, int src);
sad_status_t trainer_build_hilbert(sad_trainer* t, cudaStream_t s);
VptParams trainer_vpt_params(sad_trainer* t);
}  // namespace sad
