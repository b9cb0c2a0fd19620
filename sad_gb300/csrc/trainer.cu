// trainer.cu -- the whole fit of one image on the device.
//
// Iteration schedule: backends/cuda/src/sad_cuda.cu:2158-2479 (trainVoronoi).  Per
// iteration it = 0 .. iters-1:
//   1. every cand_update_freq iterations: f16-round the sites and run the VPT pass(es)
//      from the current candidate field into a spare one, on a side stream (the
//      gradient step of this iteration still reads the old field);
//   2. on densify iterations (never at the default config, whose buffer starts full):
//      site statistics, score, sort, split -- run eagerly, the candidate refresh then
//      runs synchronously first, as in the reference;
//   3. fused gradients (+ removal delta on prune iterations);
//   4. join the side stream; 4 Jacobi passes of log-tau diffusion on the new field;
//   5. Adam (t = it + 1) fused with the gradient clear and the refresh of the per-site
//      records the pixel kernels gather;
//   6. on prune iterations: score, radix sort, prune the planned count.
//
// Everything the host decides (which iterations refresh, densify or prune, and how
// many sites they touch) depends only on the configuration, so the plan is computed
// once at init and the per-iteration scalars the kernels need (Adam's t, the diffusion
// lambda, the VPT step, the prune count) are read from device memory.  Each iteration
// kind (refresh? prune? which candidate buffer is current?) is captured once as a CUDA
// graph and replayed: the fit is ~4000 graph launches with no host synchronisation
// except on log iterations.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "accum.cuh"
#include "common.cuh"
#include "host_common.h"
#include "kernels.h"

#include "trainer_state.h"

namespace sad {

// Every device buffer of a fit lives in one slab: offsets are planned once (base null)
// to size it, then assigned from the slab's base.  One allocation per fit, or none when
// the caller provides the memory (sad_trainer_create_in).
struct SlabCarver {
    char* base;
    size_t off = 0;
    template <class T>
    void take(T*& p, size_t count) {
        p = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += (std::max<size_t>(count * sizeof(T), 16) + 255) & ~size_t(255);
    }
};

static void drop_graphs(sad_trainer* t) {
    for (auto& a : t->graphs)
        for (auto& b : a)
            for (auto& g : b)
                if (g) {
                    cudaGraphExecDestroy(g);
                    g = nullptr;
                }
    for (auto& g : t->wgraphs)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

// Host plan of the whole schedule (the same decisions the reference makes at run time).
static void make_plan(sad_trainer* t) {
    const sad_train_config_t& c = t->cfg;
    t->plan.assign(std::max(0, c.iterations), IterPlan{});
    int eff_prune_start = c.prune_start;
    if (c.densify && !c.prune_during_densify && c.prune_start < c.densify_end)
        eff_prune_start = c.densify_end;
    int eff_prune_end = c.prune_end > 0 ? c.prune_end : c.iterations - 1;
    int active = t->active;
    uint32_t n = t->n;
    for (int it = 0; it < c.iterations; ++it) {
        IterPlan& p = t->plan[it];
        p.upd = c.cand_update_freq > 0 && it % c.cand_update_freq == 0;
        int desired = std::max(0, static_cast<int>(active * t->densify_pct));
        bool dens = c.densify && it >= c.densify_start && it <= c.densify_end &&
                    it % std::max(1, c.densify_freq) == 0 && n < t->cap && desired > 0;
        if (dens) {
            int avail = static_cast<int>(t->cap - n);
            int k = std::min(desired, std::min(avail, SAD_MAX_SPLIT_INDICES));
            if (k > 0) {
                p.dens = 1;
                p.split_k = static_cast<uint32_t>(k);
                n += k;
                active += k;
            }
        }
        bool prune = t->prune_pct > 0.0f && it >= eff_prune_start && it < eff_prune_end &&
                     it % std::max(1, c.prune_freq) == 0;
        if (prune) {
            p.prune = 1;
            int k = std::min(std::max(0, static_cast<int>(active * t->prune_pct)), SAD_MAX_SPLIT_INDICES);
            p.prune_k = static_cast<uint32_t>(k);
            active = std::max(0, active - k);
        }
    }
}

static sad_status_t build_hilbert(sad_trainer* t, cudaStream_t s) {
    int bits = sad_hilbert_bits_for_size(t->w, t->h);
    uint32_t padded = (t->n + 1023u) / 1024u * 1024u;
    padded = std::min(padded, std::max(1u, t->hpadded));
    launch_hilbert_pairs(t->sites, t->hpairs, t->n, padded, t->w, t->h, bits, s);
    uint32_t maxk = bits >= 16 ? 0xFFFFFFFFu : (1u << (2 * bits));
    launch_radix_sort(t->hpairs, padded, maxk, t->sort_temp, s);
    launch_hilbert_order(t->hpairs, t->horder, t->hpos, t->n, s);
    t->hilbert_ready = true;
    t->hilbert_count = t->n;
    return check_launch("trainer hilbert order");
}

static VptParams vpt_params(sad_trainer* t) {
    VptParams p{};
    const sad_train_config_t& c = t->cfg;
    bool use_h = c.cand_hilbert_probes > 0 && c.cand_hilbert_window > 0;
    p.site_count = t->n;
    p.inv_scale_sq = t->inv_s2;
    p.radius_scale = c.cand_radius_scale;
    p.radius_probes = c.cand_radius_probes;
    p.inject_count = t->n == 0 ? 0u : c.cand_inject_count;
    p.hilbert_order = use_h ? t->horder : nullptr;
    p.hilbert_pos = use_h ? t->hpos : nullptr;
    p.hilbert_probes = use_h ? c.cand_hilbert_probes : 0u;
    p.hilbert_window = use_h ? c.cand_hilbert_window : 0u;
    p.cand_downscale = t->ds;
    p.target_width = t->w;
    p.target_height = t->h;
    p.width = t->cw;
    p.height = t->ch;
    p.state = t->state;
    p.pow2 = t->pow2;
    p.stages = t->stages;
    return p;
}

// Thread count of the per-site kernels' grids: the buffer's site count (the kernels loop
// over the compacted list, so the grid only has to be large enough for the first
// iterations; later blocks beyond the list return at once), so the captured graphs serve
// the whole fit.
static uint32_t alive_grid_hint(const sad_trainer* t) { return std::max<uint32_t>(1u, t->n); }

static uint32_t* n_alive_ptr(sad_trainer* t) { return &t->state->n_alive; }

static void launch_compact(sad_trainer* t, cudaStream_t s) {
    launch_compact_active(t->geom, t->n, t->alive_blocks, t->alive, n_alive_ptr(t), s);
}

// VPT passes from field `src` into the spare fields; returns the final field index.
static int launch_refresh(sad_trainer* t, int src, cudaStream_t s) {
    launch_pack_geom_alive(t->sites, t->vgeom, t->alive, t->state, t->alive_hint, s);
    int o[2], k = 0;
    for (int b = 0; b < 3; ++b)
        if (b != src) o[k++] = b;
    VptParams p = vpt_params(t);
    int in = src;
    for (int pass = 0; pass < t->passes; ++pass) {
        int out = o[pass & 1];
        p.in0 = t->cand0[in];
        p.in1 = t->cand1[in];
        p.out0 = t->cand0[out];
        p.out1 = t->cand1[out];
        p.pass_offset = static_cast<uint32_t>(pass);
        launch_vpt_geom(p, t->vgeom, s);
        in = out;
    }
    // the new field's tile registration (a separate pass measured faster than registering
    // inside the VPT kernel, whose 32x8 blocks suit the gathers better)
    if (t->passes > 0)
        launch_register_tiles(t->cand0[in], t->cand1[in], t->n, t->w, t->h, t->cw, t->ch, t->tmap[in], s);
    return in;
}

int refresh_target_field(int passes, int src) {
    int o[2], k = 0;
    for (int b = 0; b < 3; ++b)
        if (b != src) o[k++] = b;
    return o[(passes - 1) & 1];
}

static int refresh_target(sad_trainer* t, int src) { return refresh_target_field(t->passes, src); }

// For the lockstep batch (batch.cu): the Hilbert order of a trainer's sites and its VPT
// parameters.
sad_status_t trainer_build_hilbert(sad_trainer* t, cudaStream_t s) { return build_hilbert(t, s); }
VptParams trainer_vpt_params(sad_trainer* t) { return vpt_params(t); }

static void launch_gradients_step(sad_trainer* t, int field, bool prune, cudaStream_t s) {
    GradParams g{};
    g.cand0 = t->cand0[field];
    g.cand1 = t->cand1[field];
    g.target = t->target;
    g.rendered = t->render;
    g.mask = t->have_mask ? t->mask : nullptr;
    g.inv_scale_sq = t->inv_s2;
    g.site_count = t->n;
    g.ssim_weight = t->cfg.ssim_weight;
    g.width = t->w;
    g.height = t->h;
    g.cand_width = t->cw;
    g.cand_height = t->ch;
    g.fix12 = t->grads;
    g.slot_map = t->tmap[field].slot_map;
    g.tile_keys = t->tmap[field].tile_keys;
    g.tile_count = t->tmap[field].tile_count;
    g.removal_fix_mul = t->removal_mul;
    g.compute_removal = prune ? 1 : 0;
    launch_gradients_prepared(g, t->geom, t->color, s);
}

// Steps 3-6 of one iteration (and the fork/join of step 1 when `upd`), then the counter
// advance.  `field` is the current candidate field; returns the field current after it.
static int iteration_body(sad_trainer* t, bool upd, bool prune, int field, int adv_passes,
                          cudaStream_t s) {
    int next = field;
    if (upd) {
        NvtxRange r("candidate refresh (VPT, tile registration)");
        cudaEventRecord(t->ev_fork, s);
        cudaStreamWaitEvent(t->side, t->ev_fork, 0);
        next = launch_refresh(t, field, t->side);
        cudaEventRecord(t->ev_join, t->side);
    }
    if (t->cfg.ssim_weight > 0.0f)
        launch_render_prepared(t->cand0[field], t->cand1[field], t->render, t->geom, t->color,
                               t->inv_s2, t->n, t->w, t->h, t->cw, t->ch, s);
    bool timed = t->timing && t->tev_used + 2 <= t->tev.size();
    if (timed) cudaEventRecord(t->tev[t->tev_used], s);
    {
        NvtxRange r_grad("gradients");
        launch_gradients_step(t, field, prune, s);
    }
    if (timed) {
        cudaEventRecord(t->tev[t->tev_used + 1], s);
        t->tev_used += 2;
    }
    if (upd) cudaStreamWaitEvent(s, t->ev_join, 0);
    // 4 Jacobi passes: grads slot 2 -> A -> B -> A -> (inside Adam), over the active list
    const uint32_t hint = t->alive_hint;
    {
        NvtxRange r_site("tau diffusion and Adam");
        launch_tau_first_pass(t->cand0[next], t->cand1[next], t->geom, t->grads, t->tau_nbr, t->tau_raw,
                              t->alive, t->tau_a, t->n, hint, t->state, t->cfg.iterations, t->cw, t->ch,
                              t->ds, s);
        launch_tau_list_pass(t->tau_nbr, t->tau_raw, t->alive, t->tau_a, t->tau_b, hint, t->state,
                             t->cfg.iterations, s);
        launch_tau_list_pass(t->tau_nbr, t->tau_raw, t->alive, t->tau_b, t->tau_a, hint, t->state,
                             t->cfg.iterations, s);
        AdamHyper hp{t->cfg.lr_pos * t->cfg.lr_scale, t->cfg.lr_tau * t->cfg.lr_scale,
                     t->cfg.lr_radius * t->cfg.lr_scale, t->cfg.lr_color * t->cfg.lr_scale,
                     t->cfg.lr_dir * t->cfg.lr_scale, t->cfg.lr_aniso * t->cfg.lr_scale,
                     t->cfg.beta1, t->cfg.beta2, t->cfg.eps};
        launch_adam_train(t->sites, t->adam, t->grads, t->tau_nbr, t->tau_raw, t->alive, t->tau_a,
                          t->geom, t->color, hp, t->state, t->cfg.iterations, hint, t->w, t->h, s);
    }
    if (prune) {
        // score, sort and prune the active list (the same sorted prefix as over every slot:
        // inactive slots key last), then compact the list again
        NvtxRange r("prune (score, sort, mark, compact)");
        float delta_norm = 1.0f / std::max(1.0f, t->mask_sum);
        launch_prune_pairs_alive(t->grads, t->removal_mul, t->pairs, t->alive, t->state, hint, delta_norm, s);
        launch_radix_sort_dev(t->pairs, t->n, n_alive_ptr(t), 0xFFFFFFFFu, t->sort_temp, s);
        launch_prune_sorted_train(t->sites, t->geom, t->vgeom, t->pairs, t->prune_k, t->state,
                                  SAD_MAX_SPLIT_INDICES, s);
        launch_compact(t, s);
    }
    launch_advance_state(t->state, static_cast<uint32_t>(adv_passes), t->cfg.beta1, t->cfg.beta2, s);
    return next;
}

static sad_status_t run_densify(sad_trainer* t, const IterPlan& p, cudaStream_t s) {
    NvtxRange r("densify (statistics, score, sort, split, compact)");
    // site statistics on the current field, score, sort, split (sad_cuda.cu:2232-2292)
    float* st[8];
    for (int k = 0; k < 8; ++k) st[k] = t->stats + static_cast<size_t>(k) * t->cap;
    launch_site_stats_fixed(t->cand0[t->cur], t->cand1[t->cur], t->target,
                            t->have_mask ? t->mask : nullptr, t->sites, t->inv_s2, t->n,
                            t->stats_fix, t->cap, st, t->w, t->h, t->cw, t->ch, s);
    launch_densify_pairs(t->sites, st[0], st[1], t->pairs, t->n, 1.0f, t->cfg.densify_score_alpha,
                         t->cap, s);
    launch_radix_sort(t->pairs, t->cap, 0xFFFFFFFFu, t->sort_temp, s);
    launch_write_indices(t->pairs, t->idx, p.split_k, s);
    const float* sp[7] = {st[0], st[2], st[3], st[4], st[5], st[6], st[7]};
    launch_split(t->sites, t->adam, t->idx, p.split_k, sp, t->n, t->target, t->w, t->h, s);
    t->n += p.split_k;
    t->active += static_cast<int>(p.split_k);
    launch_prepare_sites(t->sites, t->geom, t->color, t->n, s);
    launch_compact(t, s);
    t->alive_hint = alive_grid_hint(t);
    drop_graphs(t);  // site count changed
    return check_launch("trainer densify");
}

static sad_status_t capture_variant(sad_trainer* t, bool upd, bool prune, int field,
                                    cudaGraphExec_t* out, uint64_t* kernels) {
    cudaGraph_t graph = nullptr;
    SAD_TRY(check_cuda(cudaStreamBeginCapture(t->st, cudaStreamCaptureModeThreadLocal),
                       "trainer graph capture"));
    const uint64_t before = sad_launch_count();
    iteration_body(t, upd, prune, field, upd ? t->passes : 0, t->st);
    *kernels = sad_launch_count() - before;
    unnote_launches(*kernels);  // captured, not run; each replay counts them
    cudaError_t e = cudaStreamEndCapture(t->st, &graph);
    if (e != cudaSuccess) return check_cuda(e, "trainer graph capture end");
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    return check_cuda(e, "trainer graph instantiate");
}

// A refresh window of cand_update_freq iterations from field `field`, captured whole.
static sad_status_t capture_window(sad_trainer* t, int field, cudaGraphExec_t* out, uint64_t* kernels) {
    cudaGraph_t graph = nullptr;
    SAD_TRY(check_cuda(cudaStreamBeginCapture(t->st, cudaStreamCaptureModeThreadLocal),
                       "trainer graph capture"));
    const uint64_t before = sad_launch_count();
    int f = field;
    for (int k = 0; k < t->cfg.cand_update_freq; ++k)
        f = iteration_body(t, k == 0, false, f, k == 0 ? t->passes : 0, t->st);
    *kernels = sad_launch_count() - before;
    unnote_launches(*kernels);
    cudaError_t e = cudaStreamEndCapture(t->st, &graph);
    if (e != cudaSuccess) return check_cuda(e, "trainer graph capture end");
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    return check_cuda(e, "trainer graph instantiate");
}

// Whether iterations [it, it + cand_update_freq) form a window that one captured replay
// can run: a refresh first, then only plain iterations, all inside this run call, with no
// log line due and the autotuner (which acts between iterations) off.
static bool window_at(const sad_trainer* t, int it, int end) {
    const sad_train_config_t& c = t->cfg;
    const int len = c.cand_update_freq;
    if (len < 2 || it + len > end || c.autotune) return false;
    for (int k = 0; k < len; ++k) {
        const IterPlan& p = t->plan[it + k];
        if ((k == 0) != (p.upd != 0) || p.dens || p.prune) return false;
        if (c.log_freq > 0 && ((it + k) % c.log_freq == 0 || it + k == c.iterations - 1)) return false;
    }
    return true;
}

static sad_status_t log_iteration(sad_trainer* t, int it) {
    float psnr = 0.0f;
    SAD_TRY(sad_trainer_render(t, nullptr, &psnr));
    uint32_t active = 0;
    SAD_TRY(check_cuda(cudaMemsetAsync(t->count, 0, 4, t->st), "trainer count"));
    launch_count_active(t->sites, t->count, t->n, t->st);
    SAD_TRY(check_cuda(cudaMemcpyAsync(&active, t->count, 4, cudaMemcpyDeviceToHost, t->st),
                       "trainer count copy"));
    SAD_TRY(check_cuda(cudaStreamSynchronize(t->st), "trainer log sync"));
    double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t->t0).count();
    double its = el > 0 ? (it + 1) / el : 0.0;
    printf("Iter %4d | PSNR: %.2f dB | Active: %u/%u | %.1f it/s | %.1fs\n", it, psnr, active, t->n,
           its, el);
    fflush(stdout);
    return SAD_OK;
}

}  // namespace sad

using namespace sad;

// Sizes and schedule constants of a fit (no device work).
static sad_status_t plan_trainer(sad_trainer* t, const sad_train_config_t* cfg, int width, int height) {
    SAD_REQUIRE(cfg, "sad_trainer_create: null argument");
    SAD_REQUIRE(image_size_ok(width, height), "sad_trainer_create: invalid image size");
    SAD_REQUIRE(cfg->iterations >= 0, "sad_trainer_create: negative iterations");
    SAD_REQUIRE(cfg->n_sites > 0, "sad_trainer_create: n_sites must be positive");
    SAD_REQUIRE(cfg->cand_update_passes >= 0, "sad_trainer_create: negative candidate passes");
    t->cfg = *cfg;
    t->w = width;
    t->h = height;
    t->ds = std::max(1, cfg->cand_downscale);
    t->cw = std::max(1, (width + t->ds - 1) / t->ds);
    t->ch = std::max(1, (height + t->ds - 1) / t->ds);
    float md = static_cast<float>(std::max(width, height));
    t->inv_s2 = 1.0f / (md * md);
    t->passes = std::max(1, cfg->cand_update_passes);
    jump_schedule_constants(t->cw, t->ch, &t->pow2, &t->stages);
    int num_pixels = width * height;
    // planSiteCapacity (sad_cuda.cu:1079-1101)
    int max_cap = cfg->max_sites > 0 ? cfg->max_sites
                  : cfg->densify  ? std::min(num_pixels * 2, std::max(cfg->n_sites * 8, 8192))
                                  : num_pixels * 2;
    int requested = cfg->densify ? max_cap : cfg->n_sites;
    t->cap = static_cast<uint32_t>(std::max(cfg->n_sites, requested));
    t->prune_pct = cfg->prune_percentile;
    t->densify_pct = cfg->densify_percentile;
    if (cfg->target_bpp > 0.0f) {
        int prune_end = cfg->prune_end > 0 ? cfg->prune_end : cfg->iterations - 1;
        sad_bpp_solution_t sol{};
        SAD_TRY(sad_solve_target_bpp(
            cfg->target_bpp, width, height, cfg->n_sites, max_cap, cfg->iterations, cfg->densify,
            cfg->densify_start, cfg->densify_end, std::max(1, cfg->densify_freq),
            cfg->densify_percentile, cfg->prune_during_densify, cfg->prune_start, prune_end,
            std::max(1, cfg->prune_freq), cfg->prune_percentile, SAD_MAX_SPLIT_INDICES, &sol));
        t->densify_pct = sol.densify_percentile;
        t->prune_pct = sol.prune_percentile;
    }
    t->hpadded = (t->cap + 1023u) / 1024u * 1024u;
    t->removal_mul = removal_fix_mul(width, height);
    return SAD_OK;
}

// Assigns every buffer from base (or only sizes them when base is null); returns the
// slab size, including 256 bytes of alignment slack.
static size_t carve_trainer(sad_trainer* t, void* base) {
    uintptr_t aligned = (reinterpret_cast<uintptr_t>(base) + 255) & ~uintptr_t(255);
    SlabCarver c{base ? reinterpret_cast<char*>(aligned) : nullptr};
    size_t np = static_cast<size_t>(t->w) * t->h;
    size_t nc = static_cast<size_t>(t->cw) * t->ch * 4;
    size_t cap = t->cap;
    c.take(t->target, np * 3);
    c.take(t->mask, np);
    c.take(t->sites, cap);
    c.take(t->geom, cap);
    c.take(t->color, cap);
    c.take(t->vgeom, cap);
    c.take(t->adam, cap * 20);
    c.take(t->grads, cap * 12);
    c.take(t->tau_a, cap);
    c.take(t->tau_b, cap);
    c.take(t->tau_nbr, cap * 8);
    c.take(t->tau_raw, cap);
    c.take(t->alive, cap);
    c.take(t->alive_blocks, std::max<uint32_t>(1u, compact_blocks(t->cap)));
    c.take(t->pairs, cap * 2);
    c.take(t->idx, SAD_MAX_SPLIT_INDICES);
    for (int b = 0; b < 3; ++b) {
        c.take(t->cand0[b], nc);
        c.take(t->cand1[b], nc);
        c.take(t->tmap_mem[b], tile_map_words(t->w, t->h));
        if (base) t->tmap[b] = tile_map_at(t->tmap_mem[b], t->w, t->h);
    }
    c.take(t->horder, cap);
    c.take(t->hpos, cap);
    c.take(t->hpairs, static_cast<size_t>(t->hpadded) * 2);
    c.take(t->stats, cap * 8);
    c.take(t->stats_fix, cap * 8);
    c.take(t->render, np * 3);
    c.take(t->packed, cap * 4);
    c.take(t->packed_quant, 16);
    c.take(t->metric, 1);
    c.take(t->count, 4);
    c.take(t->state, 1);
    if (base)
        for (int b = 0; b < 3; ++b) t->tmap[b].wide_far_refs = &t->state->wide_far_refs;
    c.take(t->prune_k, static_cast<size_t>(std::max(1, t->cfg.iterations)));
    char* sort_temp = nullptr;
    c.take(sort_temp, radix_sort_temp_bytes(std::max<uint32_t>(t->cap, t->hpadded)));
    t->sort_temp = sort_temp;
    char* init_temp = nullptr;
    c.take(init_temp, init_temp_bytes(static_cast<uint32_t>(t->cfg.n_sites)));
    t->init_temp = init_temp;
    return c.off + 256;
}

// Streams, events and kernel attributes once the buffers are in place.
static sad_status_t finish_create(sad_trainer* t) {
    sad_status_t s = check_cuda(prepare_gradient_kernels(), "trainer kernel attributes");
    if (s == SAD_OK)
        s = check_cuda(cudaStreamCreateWithFlags(&t->st, cudaStreamNonBlocking), "trainer stream");
    if (s == SAD_OK)
        s = check_cuda(cudaStreamCreateWithFlags(&t->side, cudaStreamNonBlocking), "trainer stream");
    if (s == SAD_OK)
        s = check_cuda(cudaEventCreateWithFlags(&t->ev_fork, cudaEventDisableTiming), "trainer event");
    if (s == SAD_OK)
        s = check_cuda(cudaEventCreateWithFlags(&t->ev_join, cudaEventDisableTiming), "trainer event");
    return s;
}

static sad_status_t create_common(const sad_train_config_t* cfg, int width, int height, void* memory,
                                  size_t bytes, sad_trainer_t** out) {
    clear_error();
    SAD_REQUIRE(out, "sad_trainer_create: null argument");
    *out = nullptr;
    sad_trainer* t = new sad_trainer();
    sad_status_t s = plan_trainer(t, cfg, width, height);
    if (s != SAD_OK) {
        delete t;
        return s;
    }
    size_t need = carve_trainer(t, nullptr);
    if (memory) {
        if (bytes < need) {
            delete t;
            set_error("sad_trainer_create_in: %zu bytes given, %zu needed (sad_trainer_memory_bytes)", bytes, need);
            return SAD_ERR_INVALID_ARGUMENT;
        }
        t->slab = memory;
    } else {
        cudaError_t e = cudaMalloc(&t->slab, need);
        if (e != cudaSuccess) {
            delete t;
            set_error("trainer allocation of %zu bytes: %s", need, cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? SAD_ERR_OUT_OF_MEMORY : SAD_ERR_CUDA;
        }
        t->owns_slab = true;
    }
    t->slab_bytes = need;
    carve_trainer(t, t->slab);
    s = finish_create(t);
    if (s != SAD_OK) {
        std::string msg = sad_last_error();
        sad_trainer_destroy(t);
        set_error("%s", msg.c_str());
        return s;
    }
    *out = t;
    return SAD_OK;
}

extern "C" size_t sad_trainer_memory_bytes(const sad_train_config_t* cfg, int width, int height) {
    sad_trainer t;
    if (plan_trainer(&t, cfg, width, height) != SAD_OK) return 0;
    return carve_trainer(&t, nullptr);
}

extern "C" sad_status_t sad_trainer_create(const sad_train_config_t* cfg, int width, int height,
                                           sad_trainer_t** out) {
    return create_common(cfg, width, height, nullptr, 0, out);
}

extern "C" sad_status_t sad_trainer_create_in(const sad_train_config_t* cfg, int width, int height,
                                              void* device_memory, size_t bytes, sad_trainer_t** out) {
    SAD_REQUIRE(device_memory, "sad_trainer_create_in: null memory");
    return create_common(cfg, width, height, device_memory, bytes, out);
}

extern "C" sad_status_t sad_trainer_destroy(sad_trainer_t* t) {
    if (!t) return SAD_OK;
    if (t->st) cudaStreamSynchronize(t->st);
    if (t->side) cudaStreamSynchronize(t->side);
    drop_graphs(t);
    for (cudaEvent_t e : t->tev) cudaEventDestroy(e);
    if (t->ev_fork) cudaEventDestroy(t->ev_fork);
    if (t->ev_join) cudaEventDestroy(t->ev_join);
    if (t->st) cudaStreamDestroy(t->st);
    if (t->side) cudaStreamDestroy(t->side);
    if (t->owns_slab && t->slab) cudaFree(t->slab);
    delete t;
    return SAD_OK;
}

extern "C" sad_stream_t sad_trainer_stream(sad_trainer_t* t) {
    return t ? reinterpret_cast<sad_stream_t>(t->st) : nullptr;
}

static sad_status_t set_mask_common(sad_trainer* t, bool have_mask) {
    t->have_mask = have_mask;
    if (!have_mask) {
        t->mask_sum = static_cast<float>(static_cast<size_t>(t->w) * t->h);
        return SAD_OK;
    }
    // the mask sum normalises the removal delta and the PSNR (read back once per target)
    std::vector<float> host(static_cast<size_t>(t->w) * t->h);
    SAD_TRY(check_cuda(cudaMemcpyAsync(host.data(), t->mask, host.size() * 4, cudaMemcpyDeviceToHost, t->st),
                       "trainer mask readback"));
    SAD_TRY(check_cuda(cudaStreamSynchronize(t->st), "trainer mask sync"));
    // the reference counts the pixels with mask > 0 (backends/cuda/src/sad_cuda.cu:208-213)
    size_t live = 0;
    for (float v : host) live += v > 0.0f;
    t->mask_sum = static_cast<float>(live);
    return SAD_OK;
}

extern "C" sad_status_t sad_trainer_set_target_device(sad_trainer_t* t, const float* target,
                                                      const float* mask) {
    clear_error();
    SAD_REQUIRE(t && target, "sad_trainer_set_target_device: null argument");
    size_t np = static_cast<size_t>(t->w) * t->h;
    SAD_TRY(check_cuda(cudaMemcpyAsync(t->target, target, np * 12, cudaMemcpyDeviceToDevice, t->st),
                       "trainer target copy"));
    if (mask)
        SAD_TRY(check_cuda(cudaMemcpyAsync(t->mask, mask, np * 4, cudaMemcpyDeviceToDevice, t->st),
                           "trainer mask copy"));
    return set_mask_common(t, mask != nullptr);
}

extern "C" sad_status_t sad_trainer_set_target_host(sad_trainer_t* t, const float* target_host,
                                                    const float* mask_host) {
    clear_error();
    SAD_REQUIRE(t && target_host, "sad_trainer_set_target_host: null argument");
    size_t np = static_cast<size_t>(t->w) * t->h;
    SAD_TRY(check_cuda(cudaMemcpyAsync(t->target, target_host, np * 12, cudaMemcpyHostToDevice, t->st),
                       "trainer target upload"));
    if (mask_host)
        SAD_TRY(check_cuda(cudaMemcpyAsync(t->mask, mask_host, np * 4, cudaMemcpyHostToDevice, t->st),
                           "trainer mask upload"));
    return set_mask_common(t, mask_host != nullptr);
}

__global__ void fill_inactive_kernel(sad::Site* sites, uint32_t from, uint32_t to) {
    uint32_t i = from + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= to) return;
    sad::Site s{};
    s.px = -1.0f;
    s.py = -1.0f;
    s.dx = 1.0f;
    sites[i] = s;
}

extern "C" sad_status_t sad_trainer_init(sad_trainer_t* t, const float* sites_host, int n) {
    clear_error();
    SAD_REQUIRE(t, "sad_trainer_init: null trainer");
    NvtxRange r_init("fit init (sites, candidates, plan)");
    cudaStream_t s = t->st;
    uint32_t n0;
    int active;
    if (sites_host) {
        SAD_REQUIRE(n > 0 && static_cast<uint32_t>(n) <= t->cap, "sad_trainer_init: site count exceeds capacity");
        n0 = static_cast<uint32_t>(n);
        SAD_TRY(check_cuda(cudaMemcpyAsync(t->sites, sites_host, static_cast<size_t>(n) * 40,
                                           cudaMemcpyHostToDevice, s),
                           "trainer sites upload"));
        active = 0;
        for (int i = 0; i < n; ++i) active += sites_host[static_cast<size_t>(i) * 10] >= 0.0f;
    } else {
        n0 = static_cast<uint32_t>(t->cfg.n_sites);
        SAD_REQUIRE(n0 <= t->cap, "sad_trainer_init: n_sites exceeds capacity");
        float thr = 0.01f * t->cfg.init_gradient_alpha;
        SAD_TRY(check_cuda(run_init_gradient_weighted(t->sites, n0, t->target,
                                                      t->have_mask ? t->mask : nullptr, thr, 256,
                                                      t->cfg.init_log_tau, t->cfg.init_radius,
                                                      t->w, t->h, t->init_temp, s),
                           "trainer gradient-weighted init"));
        active = static_cast<int>(n0);  // the reference counts its (zeroed) host sites here
    }
    if (n0 < t->cap) {
        fill_inactive_kernel<<<blocks_for(t->cap - n0, 256), 256, 0, s>>>(t->sites, n0, t->cap);
        note_launches(1);
    }
    launch_prepare_sites(t->sites, t->geom, t->color, t->cap, s);
    SAD_TRY(check_cuda(cudaMemsetAsync(t->adam, 0, static_cast<size_t>(t->cap) * 80, s), "trainer adam clear"));
    SAD_TRY(check_cuda(cudaMemsetAsync(t->grads, 0, static_cast<size_t>(t->cap) * 12 * sizeof(long long), s),
                       "trainer grad clear"));
    SAD_TRY(check_cuda(cudaMemsetAsync(t->stats_fix, 0, static_cast<size_t>(t->cap) * 8 * sizeof(long long), s),
                       "trainer stats clear"));
    launch_reset_state(t->state, t->cfg.beta1, t->cfg.beta2, s);
    t->tuner.reset(t->cfg.autotune != 0, t->cfg.cand_update_freq);
    t->n = n0;
    t->active = active;
    t->iter = 0;
    t->cur = 0;
    t->hilbert_ready = false;
    // the VPT geometry of every slot once (inactive slots stay marked; refreshes repack the
    // active list) and the first active list
    launch_pack_geom(t->sites, t->vgeom, n0, s);
    launch_compact(t, s);
    t->alive_hint = alive_grid_hint(t);
    launch_init_candidates(t->cand0[0], t->cand1[0], n0, 0u, t->cfg.init_per_pixel ? 1 : 0, t->cw, t->ch, s);
    launch_jfa_seed(t->cand0[0], t->sites, n0, t->cw, t->ch, t->ds, s);
    launch_register_tiles(t->cand0[0], t->cand1[0], n0, t->w, t->h, t->cw, t->ch, t->tmap[0], s);
    make_plan(t);
    std::vector<uint32_t> pk(std::max(1, t->cfg.iterations), 0u);
    for (size_t i = 0; i < t->plan.size(); ++i) pk[i] = t->plan[i].prune_k;
    SAD_TRY(check_cuda(cudaMemcpyAsync(t->prune_k, pk.data(), pk.size() * 4, cudaMemcpyHostToDevice, s),
                       "trainer plan upload"));
    SAD_TRY(check_cuda(cudaStreamSynchronize(s), "trainer init sync"));
    drop_graphs(t);
    t->grad_ms = 0.0;
    t->grad_launches = 0;
    t->t0 = std::chrono::steady_clock::now();
    return check_launch("sad_trainer_init");
}

extern "C" sad_status_t sad_trainer_enable_timing(sad_trainer_t* t, int enable) {
    clear_error();
    SAD_REQUIRE(t, "sad_trainer_enable_timing: null trainer");
    t->timing = enable != 0;
    if (t->timing && t->tev.empty()) {
        t->tev.resize(2 * static_cast<size_t>(std::max(1, t->cfg.iterations)));
        for (auto& e : t->tev) SAD_TRY(check_cuda(cudaEventCreate(&e), "trainer timing events"));
    }
    return SAD_OK;
}

extern "C" sad_status_t sad_trainer_run(sad_trainer_t* t, int end) {
    clear_error();
    SAD_REQUIRE(t, "sad_trainer_run: null trainer");
    SAD_REQUIRE(end >= t->iter && end <= t->cfg.iterations, "sad_trainer_run: end out of range");
    const sad_train_config_t& c = t->cfg;
    bool use_h = c.cand_hilbert_probes > 0 && c.cand_hilbert_window > 0;
    bool eager = !c.use_graphs || t->timing;
    t->tev_used = 0;
    NvtxRange r_run(eager ? "fit iterations (eager)" : "fit iterations (graph replays)");
    struct EndRun {  // the autotuner drops windows that did not close in this call
        ShapeTuner& tuner;
        ~EndRun() { tuner.end_run(); }
    } end_run{t->tuner};
    for (int it = t->iter; it < end; ++it) {
        const IterPlan& p = t->plan[it];
        if (!eager && window_at(t, it, end)) {
            if (use_h && (!t->hilbert_ready || t->hilbert_count != t->n)) SAD_TRY(build_hilbert(t, t->st));
            cudaGraphExec_t& g = t->wgraphs[t->cur];
            uint64_t& nk = t->wgraph_kernels[t->cur];
            if (!g) SAD_TRY(capture_window(t, t->cur, &g, &nk));
            SAD_TRY(check_cuda(cudaGraphLaunch(g, t->st), "trainer graph launch"));
            note_launches(nk);
            t->cur = refresh_target(t, t->cur);
            SAD_TRY(check_launch("sad_trainer_run"));
            it += c.cand_update_freq - 1;
            t->iter = it + 1;
            continue;
        }
        SAD_TRY(check_cuda(t->tuner.before_iteration(t->plan, t->state, it, end, t->st), "trainer autotuner"));
        if (p.upd && use_h && (!t->hilbert_ready || t->hilbert_count != t->n))
            SAD_TRY(build_hilbert(t, t->st));
        if (p.dens) {
            bool upd = p.upd;
            if (upd) t->cur = launch_refresh(t, t->cur, t->st);  // synchronous refresh
            SAD_TRY(run_densify(t, p, t->st));
            t->cur = iteration_body(t, false, p.prune, t->cur, upd ? t->passes : 0, t->st);
        } else if (eager) {
            t->cur = iteration_body(t, p.upd, p.prune, t->cur, p.upd ? t->passes : 0, t->st);
        } else {
            cudaGraphExec_t& g = t->graphs[p.upd][p.prune][t->cur];
            uint64_t& nk = t->graph_kernels[p.upd][p.prune][t->cur];
            if (!g) SAD_TRY(capture_variant(t, p.upd, p.prune, t->cur, &g, &nk));
            SAD_TRY(check_cuda(cudaGraphLaunch(g, t->st), "trainer graph launch"));
            note_launches(nk);
            if (p.upd) t->cur = refresh_target(t, t->cur);
        }
        SAD_TRY(check_launch("sad_trainer_run"));
        if (p.prune) t->active = std::max(0, t->active - static_cast<int>(p.prune_k));
        t->iter = it + 1;
        if (c.log_freq > 0 && (it % c.log_freq == 0 || it == c.iterations - 1))
            SAD_TRY(log_iteration(t, it));
    }
    if (t->timing && t->tev_used > 0) {
        SAD_TRY(check_cuda(cudaStreamSynchronize(t->st), "trainer timing sync"));
        for (size_t i = 0; i + 1 < t->tev_used; i += 2) {
            float ms = 0.0f;
            SAD_TRY(check_cuda(cudaEventElapsedTime(&ms, t->tev[i], t->tev[i + 1]), "trainer timing"));
            t->grad_ms += ms;
            t->grad_launches += 1;
        }
    }
    return SAD_OK;
}

// Copy-out and PSNR of the image in t->render (shared by the two render entry points).
static sad_status_t finish_render(sad_trainer* t, float* rgb_out, float* psnr_out) {
    if (rgb_out)
        SAD_TRY(check_cuda(cudaMemcpyAsync(rgb_out, t->render, static_cast<size_t>(t->w) * t->h * 12,
                                           cudaMemcpyDeviceToDevice, t->st),
                           "trainer render copy"));
    if (psnr_out) {
        long long fsum = 0;
        SAD_TRY(check_cuda(cudaMemsetAsync(t->metric, 0, sizeof(long long), t->st), "trainer metric clear"));
        launch_mse_fixed(t->render, t->target, t->have_mask ? t->mask : nullptr, t->metric, t->w, t->h,
                         t->st);
        SAD_TRY(check_cuda(cudaMemcpyAsync(&fsum, t->metric, sizeof(long long), cudaMemcpyDeviceToHost, t->st),
                           "trainer metric copy"));
        SAD_TRY(check_cuda(cudaStreamSynchronize(t->st), "trainer render sync"));
        float sum = static_cast<float>(static_cast<double>(fsum) * (1.0 / (1 << kFixFracBits)));
        float mse = sum / (std::max(1.0f, t->mask_sum) * 3.0f);
        *psnr_out = mse > 0.0f ? 20.0f * log10f(1.0f / sqrtf(mse)) : 100.0f;
    }
    return SAD_OK;
}

extern "C" sad_status_t sad_trainer_render(sad_trainer_t* t, float* rgb_out, float* psnr_out) {
    clear_error();
    SAD_REQUIRE(t, "sad_trainer_render: null trainer");
    launch_render_prepared(t->cand0[t->cur], t->cand1[t->cur], t->render, t->geom, t->color,
                           t->inv_s2, t->n, t->w, t->h, t->cw, t->ch, t->st);
    SAD_TRY(finish_render(t, rgb_out, psnr_out));
    return check_launch("sad_trainer_render");
}

extern "C" sad_status_t sad_trainer_render_packed(sad_trainer_t* t, float* rgb_out, float* psnr_out,
                                                  sad_packed_quant_t* quant_out) {
    clear_error();
    SAD_REQUIRE(t, "sad_trainer_render_packed: null trainer");
    SAD_REQUIRE(t->w <= 32768 && t->h <= 32768, "sad_trainer_render_packed: image side above 32768");
    launch_pack_inference(t->sites, t->n, t->w, t->h, t->packed_quant, t->packed, t->st);
    launch_render_packed(t->cand0[t->cur], t->cand1[t->cur], t->render, t->packed, t->packed_quant, t->inv_s2,
                         t->n, t->w, t->h, t->cw, t->ch, t->st);
    if (quant_out) {
        SAD_TRY(check_cuda(cudaMemcpyAsync(quant_out, t->packed_quant, sizeof(sad_packed_quant_t),
                                           cudaMemcpyDeviceToHost, t->st),
                           "trainer packed ranges copy"));
        SAD_TRY(check_cuda(cudaStreamSynchronize(t->st), "trainer packed sync"));
    }
    SAD_TRY(finish_render(t, rgb_out, psnr_out));
    return check_launch("sad_trainer_render_packed");
}

extern "C" sad_status_t sad_trainer_get_sites(sad_trainer_t* t, float* sites_host, int capacity,
                                              int active_only, int* written) {
    clear_error();
    SAD_REQUIRE(t && sites_host && written, "sad_trainer_get_sites: null argument");
    std::vector<float> all(static_cast<size_t>(t->n) * 10);
    SAD_TRY(check_cuda(cudaMemcpyAsync(all.data(), t->sites, all.size() * 4, cudaMemcpyDeviceToHost, t->st),
                       "trainer sites download"));
    SAD_TRY(check_cuda(cudaStreamSynchronize(t->st), "trainer sites sync"));
    int k = 0;
    for (uint32_t i = 0; i < t->n && k < capacity; ++i) {
        const float* s = all.data() + static_cast<size_t>(i) * 10;
        if (active_only && !(s[0] >= 0.0f)) continue;
        std::memcpy(sites_host + static_cast<size_t>(k) * 10, s, 40);
        ++k;
    }
    *written = k;
    return SAD_OK;
}

extern "C" sad_status_t sad_trainer_info(sad_trainer_t* t, sad_trainer_info_t* info) {
    clear_error();
    SAD_REQUIRE(t && info, "sad_trainer_info: null argument");
    info->width = t->w;
    info->height = t->h;
    info->iteration = t->iter;
    info->site_buffer = static_cast<int>(t->n);
    info->active_estimate = t->active;
    info->capacity = static_cast<int>(t->cap);
    info->prune_percentile = t->prune_pct;
    info->densify_percentile = t->densify_pct;
    info->gpu_ms_gradients = t->grad_ms;
    info->gradient_launches = t->grad_launches;
    info->kernel_launches = sad_launch_count();
    info->wide_far_refs = t->tuner.rule();
    info->tune_rounds = t->tuner.rounds();
    return SAD_OK;
}

extern "C" sad_status_t sad_trainer_fit_host(sad_trainer_t* t, const float* target_host,
                                             const float* mask_host, float* sites_host,
                                             int capacity, int* written, float* psnr_out) {
    clear_error();
    SAD_REQUIRE(t && target_host, "sad_trainer_fit_host: null argument");
    SAD_TRY(sad_trainer_set_target_host(t, target_host, mask_host));
    SAD_TRY(sad_trainer_init(t, nullptr, 0));
    SAD_TRY(sad_trainer_run(t, t->cfg.iterations));
    SAD_TRY(sad_trainer_render(t, nullptr, psnr_out));
    if (sites_host) {
        SAD_REQUIRE(written, "sad_trainer_fit_host: null written");
        SAD_TRY(sad_trainer_get_sites(t, sites_host, capacity, 1, written));
    }
    return SAD_OK;
}
