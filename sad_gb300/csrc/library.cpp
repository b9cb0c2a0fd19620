// library.cpp -- error state, version and launch accounting of libsad_gb300, plus the
// host-side schedule rules (bpp -> site count, capacity plan, render defaults).
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <algorithm>

#include "host_common.h"

namespace sad {

static thread_local char g_err[512];
static std::atomic<uint64_t> g_launches{0};

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

void clear_error() { g_err[0] = '\0'; }

void note_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
void unnote_launches(uint64_t n) { g_launches.fetch_sub(n, std::memory_order_relaxed); }

}  // namespace sad

using namespace sad;

extern "C" const char* sad_last_error(void) { return g_err; }
extern "C" const char* sad_version(void) { return "sad_gb300 1.0 (sm_103a)"; }
extern "C" int sad_abi_version(void) { return SAD_GB300_ABI_VERSION; }
extern "C" uint64_t sad_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

// ---------------------------------------------------------------------------
// bpp rule: simulateFinalSites / solveTargetBpp, backends/cuda/src/sad_cuda.cu:904-1066
// ---------------------------------------------------------------------------
extern "C" int sad_simulate_final_sites(int init_sites, int max_sites, int iters,
                                        int densify_enabled, int densify_start, int densify_end,
                                        int densify_freq, float densify_pct,
                                        int prune_during_densify, int prune_start, int prune_end,
                                        int prune_freq, float prune_pct, int max_split) {
    int actual = init_sites, active = init_sites;
    int maxc = std::max(max_sites, init_sites);
    int eff_prune_start = prune_start;
    if (densify_enabled && !prune_during_densify && prune_start < densify_end)
        eff_prune_start = densify_end;
    if (iters <= 0) return active;
    for (int it = 0; it < iters; ++it) {
        if (densify_enabled && densify_pct > 0.0f && it >= densify_start && it <= densify_end &&
            it % std::max(1, densify_freq) == 0 && actual < maxc) {
            int desired = static_cast<int>(active * densify_pct);
            int k = std::min(desired, std::min(maxc - actual, max_split));
            if (k > 0) {
                actual += k;
                active += k;
            }
        }
        if (prune_pct > 0.0f && it >= eff_prune_start && it < prune_end &&
            it % std::max(1, prune_freq) == 0) {
            int k = std::min(static_cast<int>(active * prune_pct), max_split);
            if (k > 0) active = std::max(0, active - k);
        }
    }
    return active;
}

extern "C" sad_status_t sad_solve_target_bpp(float target_bpp, int width, int height,
                                             int init_sites, int max_sites, int iters,
                                             int densify_enabled, int densify_start,
                                             int densify_end, int densify_freq,
                                             float base_densify, int prune_during_densify,
                                             int prune_start, int prune_end, int prune_freq,
                                             float base_prune, int max_split,
                                             sad_bpp_solution_t* out) {
    clear_error();
    SAD_REQUIRE(out, "sad_solve_target_bpp: null output");
    SAD_REQUIRE(width > 0 && height > 0, "sad_solve_target_bpp: invalid image size");
    const float bits_per_site = 16.0f * 8.0f;
    int target = std::max(1, static_cast<int>(std::round(target_bpp * static_cast<float>(width * height) / bits_per_site)));
    float max_base = std::max(base_densify, base_prune);
    auto sim = [&](float d, float p) {
        return sad_simulate_final_sites(init_sites, max_sites, iters, densify_enabled,
                                        densify_start, densify_end, densify_freq, d,
                                        prune_during_densify, prune_start, prune_end, prune_freq,
                                        p, max_split);
    };
    if (max_base <= 0.0f) {
        int fs = sim(0.0f, 0.0f);
        *out = {0.0f, 0.0f, fs, static_cast<float>(fs) * bits_per_site / static_cast<float>(width * height)};
        return SAD_OK;
    }
    const float max_pct = 0.95f;
    float smax = std::min(max_pct / max_base, 50.0f);
    auto eval = [&](float s) {
        float d = densify_enabled ? std::min(max_pct, base_densify * s) : 0.0f;
        float p = std::min(max_pct, base_prune * s);
        return sim(d, p);
    };
    float best_scale = 0.0f;
    int best_sites = eval(0.0f);
    int best_err = std::abs(best_sites - target);
    const int samples = 80;
    for (int i = 0; i <= samples; ++i) {
        float s = smax * static_cast<float>(i) / static_cast<float>(samples);
        int st = eval(s);
        int err = std::abs(st - target);
        if (err < best_err) {
            best_err = err;
            best_scale = s;
            best_sites = st;
        }
    }
    float step = smax / static_cast<float>(samples);
    for (int i = 0; i < 20; ++i) {
        bool improved = false;
        float s0 = best_scale - step, s1 = best_scale + step;
        if (s0 >= 0.0f) {
            int st = eval(s0);
            int err = std::abs(st - target);
            if (err < best_err) {
                best_err = err;
                best_scale = s0;
                best_sites = st;
                improved = true;
            }
        }
        if (s1 <= smax) {
            int st = eval(s1);
            int err = std::abs(st - target);
            if (err < best_err) {
                best_err = err;
                best_scale = s1;
                best_sites = st;
                improved = true;
            }
        }
        if (!improved) step *= 0.5f;
    }
    out->densify_percentile = densify_enabled ? std::min(max_pct, base_densify * best_scale) : 0.0f;
    out->prune_percentile = std::min(max_pct, base_prune * best_scale);
    out->final_sites = best_sites;
    out->achieved_bpp = static_cast<float>(best_sites) * bits_per_site / static_cast<float>(width * height);
    return SAD_OK;
}

// training_config.json of the reference (DEFAULT_SITES ... MAX_DIM) and the CLI defaults
// of backends/cuda/src/sad_cuda.cu:580-640
extern "C" void sad_train_config_default(sad_train_config_t* c) {
    if (!c) return;
    c->n_sites = 128000;
    c->max_sites = 128000;
    c->iterations = 4000;
    c->target_bpp = 1.0f;
    c->prune_percentile = 0.033f;
    c->prune_during_densify = 1;
    c->prune_start = 100;
    c->prune_freq = 40;
    c->prune_end = 3000;
    c->densify = 1;
    c->densify_start = 20;
    c->densify_freq = 20;
    c->densify_end = 3000;
    c->densify_percentile = 0.01f;
    c->densify_score_alpha = 0.7f;
    c->cand_update_freq = 8;
    c->cand_update_passes = 1;
    c->cand_downscale = 1;
    c->cand_radius_scale = 64.0f;
    c->cand_radius_probes = 0;
    c->cand_inject_count = 4;
    c->cand_hilbert_window = 32;
    c->cand_hilbert_probes = 1;
    c->lr_pos = 0.025f;
    c->lr_tau = 0.01f;
    c->lr_radius = 0.01f;
    c->lr_color = 0.01f;
    c->lr_dir = 0.0025f;
    c->lr_aniso = 0.025f;
    c->lr_scale = 1.0f;
    c->init_log_tau = 5.0f;
    c->init_radius = 4.0f;
    c->init_gradient_alpha = 1.0f;
    c->beta1 = 0.9f;
    c->beta2 = 0.999f;
    c->eps = 1e-8f;
    c->ssim_weight = 0.0f;
    c->log_freq = 1000;
    c->use_graphs = 1;
    c->init_per_pixel = 0;
    c->autotune = 0;
}

// RenderOptions defaults, backends/cuda/src/sad_cuda.cu:618-637 / 656-670
extern "C" void sad_render_config_default(sad_render_config_t* c) {
    if (!c) return;
    c->candidate_passes = 16;
    c->use_jfa = 1;
    c->jfa_rounds = 1;
    c->cand_downscale = 1;
    c->cand_radius_scale = 64.0f;
    c->cand_radius_probes = 0;
    c->cand_inject_count = 4;
    c->cand_hilbert_window = 32;
    c->cand_hilbert_probes = 1;
}
