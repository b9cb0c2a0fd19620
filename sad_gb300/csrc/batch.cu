// batch.cu -- many fits in lockstep: every image of a batch advances one iteration at a
// time, and each stage of the iteration is one launch over all images -- a per-image tile
// work list for the per-pixel kernels (gradients, tile registration, VPT) and one flat
// list over every image's compacted active sites for the per-site kernels (tau passes,
// Adam, f16 refresh, prune scoring) -- captured once per iteration kind as a CUDA graph.
//
// Each image keeps its own fit state (a sad_trainer: slab, plan, per-image prune counts,
// device counters), so per image the arithmetic is exactly that of a single fit: a batch
// gives every image the sites its own sad_trainer fit would give, bit for bit.  The
// schedule must be common to the batch (the same training_config.json cadence; the bpp
// rule's prune percentage may differ per image), with one VPT pass per refresh and no
// densify step firing (the default configuration starts with a full buffer) -- other
// configurations are rejected at sad_batch_init with SAD_ERR_UNSUPPORTED.
//
// The reference fits one image per process (run.sh batch mode, run.sh:262-373); this is
// the batched-fitting workload with a per-image work list.
#include <algorithm>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "trainer_state.h"

using namespace sad;

struct sad_batch {
    sad_train_config_t cfg;
    std::vector<sad_trainer*> tr;
    uint32_t count = 0;
    bool ready = false;
    int iter = 0;
    int cur = 0;
    bool timing = false;
    double grad_ms = 0.0;
    int grad_launches = 0;
    uint32_t site_grid = 0;    // thread count of the per-site grids (grid-stride)
    uint32_t total_tiles = 0;  // 16x16 tiles of every image
    uint32_t total_vpt = 0;    // 32x8 VPT blocks of every image
    uint32_t max_compact = 0;  // largest per-image compaction grid
    uint32_t max_prune_k = 0;  // largest planned prune count
    // device tables, one allocation
    void* tables = nullptr;
    SiteBatchItem* site_items = nullptr;
    // the per-pixel kernels' images and block prefixes stay on the host: those kernels take
    // them as kernel parameters (BatchArgs; captured by value, and the graphs are dropped
    // whenever the tables change)
    std::vector<GradBatchItem> grad_items[3];
    std::vector<RegisterBatchItem> reg_items[3];
    std::vector<VptBatchItem> vpt_items[3];
    std::vector<uint32_t> tile_prefix, vpt_prefix;
    uint32_t* site_prefix = nullptr;
    cudaStream_t st = nullptr, side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_done = nullptr;
    cudaGraphExec_t graphs[2][2][3] = {};
    uint64_t graph_kernels[2][2][3] = {};  // kernel launches one replay runs
    cudaGraphExec_t wgraphs[3] = {};  // a whole refresh window per start field (as the trainer's)
    uint64_t wgraph_kernels[3] = {};
    std::vector<cudaEvent_t> tev;
    size_t tev_used = 0;
};

namespace {

void drop_batch_graphs(sad_batch* b) {
    for (auto& x : b->graphs)
        for (auto& y : x)
            for (auto& g : y)
                if (g) {
                    cudaGraphExecDestroy(g);
                    g = nullptr;
                }
    for (auto& g : b->wgraphs)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

uint32_t tiles_of(const sad_trainer* t) { return static_cast<uint32_t>(((t->w + 15) / 16) * ((t->h + 15) / 16)); }
uint32_t vpt_blocks_of(const sad_trainer* t) { return static_cast<uint32_t>(((t->cw + 31) / 32) * ((t->ch + 7) / 8)); }

// Host images of the device tables, then one upload.
sad_status_t build_tables(sad_batch* b) {
    const uint32_t B = b->count;
    std::vector<SiteBatchItem> site(B);
    std::vector<GradBatchItem> grad[3];
    std::vector<RegisterBatchItem> reg[3];
    std::vector<VptBatchItem> vpt[3];
    std::vector<uint32_t> tile_prefix(B + 1), vpt_prefix(B + 1);
    uint64_t sum_n = 0;
    b->total_tiles = b->total_vpt = b->max_compact = b->max_prune_k = 0;
    for (int f = 0; f < 3; ++f) {
        grad[f].resize(B);
        reg[f].resize(B);
        vpt[f].resize(B);
    }
    for (uint32_t i = 0; i < B; ++i) {
        sad_trainer* t = b->tr[i];
        tile_prefix[i] = b->total_tiles;
        vpt_prefix[i] = b->total_vpt;
        b->total_tiles += tiles_of(t);
        b->total_vpt += vpt_blocks_of(t);
        b->max_compact = std::max(b->max_compact, std::max(1u, compact_blocks(t->n)));
        for (const IterPlan& p : t->plan) b->max_prune_k = std::max(b->max_prune_k, p.prune_k);
        sum_n += t->n;
        SiteBatchItem& s = site[i];
        s.sites = t->sites;
        s.geom = t->geom;
        s.color = t->color;
        s.vgeom = t->vgeom;
        s.adam = t->adam;
        s.grads = t->grads;
        s.tau_a = t->tau_a;
        s.tau_b = t->tau_b;
        s.tau_nbr = t->tau_nbr;
        s.tau_raw = t->tau_raw;
        s.alive = t->alive;
        s.alive_blocks = t->alive_blocks;
        s.state = t->state;
        for (int f = 0; f < 3; ++f) {
            s.cand0[f] = t->cand0[f];
            s.cand1[f] = t->cand1[f];
        }
        s.pairs = t->pairs;
        s.prune_k = t->prune_k;
        s.n = t->n;
        s.w = t->w;
        s.h = t->h;
        s.cw = t->cw;
        s.ch = t->ch;
        s.ds = t->ds;
        s.removal_inv_mul = 1.0f / t->removal_mul;
        s.delta_norm = 1.0f / std::max(1.0f, t->mask_sum);
        const VptParams base = trainer_vpt_params(t);
        for (int f = 0; f < 3; ++f) {
            GradBatchItem& g = grad[f][i];
            g = GradBatchItem{};
            g.p.cand0 = t->cand0[f];
            g.p.cand1 = t->cand1[f];
            g.p.target = t->target;
            g.p.rendered = t->render;
            g.p.mask = t->have_mask ? t->mask : nullptr;
            g.p.inv_scale_sq = t->inv_s2;
            g.p.site_count = t->n;
            g.p.ssim_weight = t->cfg.ssim_weight;
            g.p.width = t->w;
            g.p.height = t->h;
            g.p.cand_width = t->cw;
            g.p.cand_height = t->ch;
            g.p.fix12 = t->grads;
            g.p.removal_fix_mul = t->removal_mul;
            g.p.slot_map = t->tmap[f].slot_map;
            g.p.tile_keys = t->tmap[f].tile_keys;
            g.p.tile_count = t->tmap[f].tile_count;
            g.geom = t->geom;
            g.color = t->color;
            g.tiles_x = (t->w + 15) / 16;
            RegisterBatchItem& r = reg[f][i];
            r.c0 = t->cand0[f];
            r.c1 = t->cand1[f];
            r.n = t->n;
            r.w = t->w;
            r.h = t->h;
            r.cw = t->cw;
            r.ch = t->ch;
            r.map = t->tmap[f];
            r.tiles_x = (t->w + 15) / 16;
            // VPT from field f into the field a one-pass refresh from f writes
            const int out = refresh_target_field(1, f);
            VptBatchItem& v = vpt[f][i];
            v.p = base;
            v.p.in0 = t->cand0[f];
            v.p.in1 = t->cand1[f];
            v.p.out0 = t->cand0[out];
            v.p.out1 = t->cand1[out];
            v.p.pass_offset = 0;
            v.vgeom = t->vgeom;
            v.blocks_x = (t->cw + 31) / 32;
        }
    }
    tile_prefix[B] = b->total_tiles;
    vpt_prefix[B] = b->total_vpt;
    b->site_grid = static_cast<uint32_t>(std::min<uint64_t>(std::max<uint64_t>(sum_n, 1), 152ull * 8 * 256));

    auto a256 = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t bytes = a256(B * sizeof(SiteBatchItem)) + a256((B + 1) * sizeof(uint32_t));
    if (!b->tables) SAD_TRY(check_cuda(cudaMalloc(&b->tables, bytes), "sad_batch_init: table allocation"));
    char* base = static_cast<char*>(b->tables);
    std::vector<char> host(bytes, 0);
    size_t off = 0;
    auto put = [&](auto*& dst, const void* src, size_t n) {
        dst = reinterpret_cast<std::remove_reference_t<decltype(dst)>>(base + off);
        std::memcpy(host.data() + off, src, n);
        off += a256(n);
    };
    put(b->site_items, site.data(), B * sizeof(SiteBatchItem));
    put(b->site_prefix, tile_prefix.data(), (B + 1) * sizeof(uint32_t));  // rewritten on the device below
    for (int f = 0; f < 3; ++f) {
        b->grad_items[f] = grad[f];
        b->reg_items[f] = reg[f];
        b->vpt_items[f] = vpt[f];
    }
    b->tile_prefix = tile_prefix;
    b->vpt_prefix = vpt_prefix;
    SAD_TRY(check_cuda(cudaMemcpyAsync(b->tables, host.data(), bytes, cudaMemcpyHostToDevice, b->st),
                       "sad_batch_init: table upload"));
    launch_batch_site_prefix(b->site_items, B, b->site_prefix, b->st);
    return check_launch("sad_batch_init: tables");
}

// One lockstep iteration of every image (the trainer's iteration_body, batched).
void batch_iteration(sad_batch* b, bool upd, bool prune, int field, cudaStream_t s) {
    const uint32_t B = b->count;
    const sad_train_config_t& c = b->cfg;
    int next = field;
    if (upd) {
        NvtxRange r("batch: candidate refresh (VPT, tile registration)");
        next = refresh_target_field(1, field);
        cudaEventRecord(b->ev_fork, s);
        cudaStreamWaitEvent(b->side, b->ev_fork, 0);
        launch_pack_geom_batch(b->site_items, b->site_prefix, B, b->site_grid, b->side);
        launch_vpt_batch(b->vpt_items[field].data(), b->vpt_prefix.data(), B, b->side);
        launch_register_tiles_batch(b->reg_items[next].data(), b->tile_prefix.data(), B, b->side);
        cudaEventRecord(b->ev_join, b->side);
    }
    const bool timed = b->timing && b->tev_used + 2 <= b->tev.size();
    if (timed) cudaEventRecord(b->tev[b->tev_used], s);
    {
        NvtxRange r("batch: gradients");
        launch_gradients_batch(b->grad_items[field].data(), b->tile_prefix.data(), B, prune, false, s);
    }
    if (timed) {
        cudaEventRecord(b->tev[b->tev_used + 1], s);
        b->tev_used += 2;
    }
    if (upd) cudaStreamWaitEvent(s, b->ev_join, 0);
    {
        NvtxRange r("batch: tau diffusion and Adam");
        launch_tau_first_batch(b->site_items, b->site_prefix, B, next, c.iterations, b->site_grid, s);
        launch_tau_list_batch(b->site_items, b->site_prefix, B, true, c.iterations, b->site_grid, s);
        launch_tau_list_batch(b->site_items, b->site_prefix, B, false, c.iterations, b->site_grid, s);
        AdamHyper hp{c.lr_pos * c.lr_scale, c.lr_tau * c.lr_scale, c.lr_radius * c.lr_scale, c.lr_color * c.lr_scale,
                     c.lr_dir * c.lr_scale, c.lr_aniso * c.lr_scale, c.beta1, c.beta2, c.eps};
        launch_adam_batch(b->site_items, b->site_prefix, B, hp, c.iterations, b->site_grid, s);
    }
    if (prune) {
        NvtxRange r("batch: prune (score, sort, mark, compact)");
        launch_prune_pairs_batch(b->site_items, b->site_prefix, B, b->site_grid, s);
        for (sad_trainer* t : b->tr)
            launch_radix_sort_dev(t->pairs, t->n, &t->state->n_alive, 0xFFFFFFFFu, t->sort_temp, s);
        launch_prune_sorted_batch(b->site_items, B, b->max_prune_k, s);
        launch_compact_batch(b->site_items, B, b->max_compact, s);
        launch_batch_site_prefix(b->site_items, B, b->site_prefix, s);
    }
    launch_advance_state_batch(b->site_items, B, upd ? 1u : 0u, c.beta1, c.beta2, s);
}

// A refresh window (cand_update_freq iterations: the refresh, then plain ones) captured whole.
sad_status_t capture_batch_window(sad_batch* b, int field, cudaGraphExec_t* out, uint64_t* kernels) {
    cudaGraph_t graph = nullptr;
    SAD_TRY(check_cuda(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal), "batch graph capture"));
    const uint64_t before = sad_launch_count();
    for (int k = 0; k < b->cfg.cand_update_freq; ++k)
        batch_iteration(b, k == 0, false, k == 0 ? field : refresh_target_field(1, field), b->st);
    *kernels = sad_launch_count() - before;
    unnote_launches(*kernels);
    cudaError_t e = cudaStreamEndCapture(b->st, &graph);
    if (e != cudaSuccess) return check_cuda(e, "batch graph capture end");
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    return check_cuda(e, "batch graph instantiate");
}

// Whether iterations [it, it + cand_update_freq) are a refresh window without a prune step
// inside this run call (the images share one schedule).
bool batch_window_at(const sad_batch* b, const std::vector<IterPlan>& plan, int it, int end) {
    const int len = b->cfg.cand_update_freq;
    if (len < 2 || it + len > end) return false;
    for (int k = 0; k < len; ++k)
        if ((k == 0) != (plan[it + k].upd != 0) || plan[it + k].prune || plan[it + k].dens) return false;
    return true;
}

sad_status_t capture_batch(sad_batch* b, bool upd, bool prune, int field, cudaGraphExec_t* out, uint64_t* kernels) {
    cudaGraph_t graph = nullptr;
    SAD_TRY(check_cuda(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal), "batch graph capture"));
    const uint64_t before = sad_launch_count();
    batch_iteration(b, upd, prune, field, b->st);
    *kernels = sad_launch_count() - before;
    unnote_launches(*kernels);  // captured, not run; each replay counts them
    cudaError_t e = cudaStreamEndCapture(b->st, &graph);
    if (e != cudaSuccess) return check_cuda(e, "batch graph capture end");
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    return check_cuda(e, "batch graph instantiate");
}

}  // namespace

extern "C" sad_status_t sad_batch_create(const sad_train_config_t* cfg, int n_images, const int* widths,
                                         const int* heights, sad_batch_t** out) {
    clear_error();
    SAD_REQUIRE(cfg && widths && heights && out, "sad_batch_create: null argument");
    SAD_REQUIRE(n_images > 0 && static_cast<uint32_t>(n_images) <= kMaxBatchItems,
                "sad_batch_create: n_images must be in [1, 1024]");
    *out = nullptr;
    sad_batch* b = new sad_batch();
    b->cfg = *cfg;
    b->count = static_cast<uint32_t>(n_images);
    sad_status_t s = SAD_OK;
    for (int i = 0; i < n_images && s == SAD_OK; ++i) {
        sad_trainer* t = nullptr;
        s = sad_trainer_create(cfg, widths[i], heights[i], &t);
        if (s == SAD_OK) b->tr.push_back(t);
    }
    if (s == SAD_OK) s = check_cuda(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking), "batch stream");
    if (s == SAD_OK) s = check_cuda(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking), "batch stream");
    if (s == SAD_OK) s = check_cuda(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming), "batch event");
    if (s == SAD_OK) s = check_cuda(cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming), "batch event");
    if (s == SAD_OK) s = check_cuda(cudaEventCreateWithFlags(&b->ev_done, cudaEventDisableTiming), "batch event");
    if (s != SAD_OK) {
        std::string msg = sad_last_error();
        sad_batch_destroy(b);
        set_error("%s", msg.c_str());
        return s;
    }
    *out = b;
    return SAD_OK;
}

extern "C" sad_status_t sad_batch_destroy(sad_batch_t* b) {
    if (!b) return SAD_OK;
    if (b->st) cudaStreamSynchronize(b->st);
    if (b->side) cudaStreamSynchronize(b->side);
    drop_batch_graphs(b);
    for (cudaEvent_t e : b->tev) cudaEventDestroy(e);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_join) cudaEventDestroy(b->ev_join);
    if (b->ev_done) cudaEventDestroy(b->ev_done);
    if (b->st) cudaStreamDestroy(b->st);
    if (b->side) cudaStreamDestroy(b->side);
    if (b->tables) cudaFree(b->tables);
    for (sad_trainer* t : b->tr) sad_trainer_destroy(t);
    delete b;
    return SAD_OK;
}

extern "C" sad_stream_t sad_batch_stream(sad_batch_t* b) { return b ? reinterpret_cast<sad_stream_t>(b->st) : nullptr; }

extern "C" sad_status_t sad_batch_trainer(sad_batch_t* b, int image, sad_trainer_t** out) {
    clear_error();
    SAD_REQUIRE(b && out && image >= 0 && static_cast<uint32_t>(image) < b->count, "sad_batch_trainer: bad argument");
    *out = b->tr[image];
    return SAD_OK;
}

extern "C" sad_status_t sad_batch_init(sad_batch_t* b) {
    clear_error();
    SAD_REQUIRE(b, "sad_batch_init: null batch");
    NvtxRange r("batch: init");
    const sad_train_config_t& c = b->cfg;
    if (std::max(1, c.cand_update_passes) != 1)
        return fail(SAD_ERR_UNSUPPORTED, "sad_batch_init: one VPT pass per refresh only");
    if (c.ssim_weight > 0.0f) return fail(SAD_ERR_UNSUPPORTED, "sad_batch_init: SSIM loss is not batched");
    for (sad_trainer* t : b->tr) {
        SAD_TRY(sad_trainer_init(t, nullptr, 0));
        for (const IterPlan& p : t->plan)
            if (p.dens) return fail(SAD_ERR_UNSUPPORTED, "sad_batch_init: a densify step fires; fit the images one by one");
    }
    const std::vector<IterPlan>& p0 = b->tr[0]->plan;
    for (sad_trainer* t : b->tr)
        for (size_t i = 0; i < p0.size(); ++i)
            if (t->plan[i].upd != p0[i].upd || t->plan[i].prune != p0[i].prune)
                return fail(SAD_ERR_UNSUPPORTED, "sad_batch_init: the images' schedules differ");
    // the Hilbert order of each image's starting sites (its site count never changes)
    const bool use_h = c.cand_hilbert_probes > 0 && c.cand_hilbert_window > 0;
    for (sad_trainer* t : b->tr) {
        if (use_h) SAD_TRY(trainer_build_hilbert(t, t->st));
        SAD_TRY(check_cuda(cudaStreamSynchronize(t->st), "sad_batch_init: trainer sync"));
    }
    drop_batch_graphs(b);
    SAD_TRY(build_tables(b));
    SAD_TRY(check_cuda(cudaStreamSynchronize(b->st), "sad_batch_init: sync"));
    b->iter = 0;
    b->cur = 0;
    b->grad_ms = 0.0;
    b->grad_launches = 0;
    b->ready = true;
    return SAD_OK;
}

extern "C" sad_status_t sad_batch_enable_timing(sad_batch_t* b, int enable) {
    clear_error();
    SAD_REQUIRE(b, "sad_batch_enable_timing: null batch");
    b->timing = enable != 0;
    if (b->timing && b->tev.empty()) {
        b->tev.resize(2 * static_cast<size_t>(std::max(1, b->cfg.iterations)));
        for (auto& e : b->tev) SAD_TRY(check_cuda(cudaEventCreate(&e), "batch timing events"));
    }
    return SAD_OK;
}

extern "C" sad_status_t sad_batch_run(sad_batch_t* b, int end) {
    clear_error();
    SAD_REQUIRE(b && b->ready, "sad_batch_run: batch not initialised");
    SAD_REQUIRE(end >= b->iter && end <= b->cfg.iterations, "sad_batch_run: end out of range");
    const std::vector<IterPlan>& plan = b->tr[0]->plan;
    const bool eager = !b->cfg.use_graphs || b->timing;
    b->tev_used = 0;
    NvtxRange r(eager ? "batch iterations (eager)" : "batch iterations (graph replays)");
    for (int it = b->iter; it < end; ++it) {
        const IterPlan& p = plan[it];
        if (!eager && batch_window_at(b, plan, it, end)) {
            cudaGraphExec_t& g = b->wgraphs[b->cur];
            uint64_t& nk = b->wgraph_kernels[b->cur];
            if (!g) SAD_TRY(capture_batch_window(b, b->cur, &g, &nk));
            SAD_TRY(check_cuda(cudaGraphLaunch(g, b->st), "batch graph launch"));
            note_launches(nk);
            SAD_TRY(check_launch("sad_batch_run"));
            b->cur = refresh_target_field(1, b->cur);
            it += b->cfg.cand_update_freq - 1;
            b->iter = it + 1;
            continue;
        }
        if (eager) {
            batch_iteration(b, p.upd, p.prune, b->cur, b->st);
        } else {
            cudaGraphExec_t& g = b->graphs[p.upd][p.prune][b->cur];
            uint64_t& nk = b->graph_kernels[p.upd][p.prune][b->cur];
            if (!g) SAD_TRY(capture_batch(b, p.upd, p.prune, b->cur, &g, &nk));
            SAD_TRY(check_cuda(cudaGraphLaunch(g, b->st), "batch graph launch"));
            note_launches(nk);
        }
        SAD_TRY(check_launch("sad_batch_run"));
        if (p.upd) b->cur = refresh_target_field(1, b->cur);
        for (sad_trainer* t : b->tr)
            if (t->plan[it].prune) t->active = std::max(0, t->active - static_cast<int>(t->plan[it].prune_k));
        b->iter = it + 1;
    }
    // the per-image trainers follow (their streams wait for the batch's work), so their
    // render / PSNR / site entry points see the fit
    SAD_TRY(check_cuda(cudaEventRecord(b->ev_done, b->st), "batch event"));
    for (sad_trainer* t : b->tr) {
        t->cur = b->cur;
        t->iter = b->iter;
        SAD_TRY(check_cuda(cudaStreamWaitEvent(t->st, b->ev_done, 0), "batch event wait"));
    }
    if (b->timing && b->tev_used > 0) {
        SAD_TRY(check_cuda(cudaStreamSynchronize(b->st), "batch timing sync"));
        for (size_t i = 0; i + 1 < b->tev_used; i += 2) {
            float ms = 0.0f;
            SAD_TRY(check_cuda(cudaEventElapsedTime(&ms, b->tev[i], b->tev[i + 1]), "batch timing"));
            b->grad_ms += ms;
            b->grad_launches += 1;
        }
    }
    return SAD_OK;
}

extern "C" sad_status_t sad_batch_synchronize(sad_batch_t* b) {
    clear_error();
    SAD_REQUIRE(b, "sad_batch_synchronize: null batch");
    return check_cuda(cudaStreamSynchronize(b->st), "sad_batch_synchronize");
}

extern "C" sad_status_t sad_batch_gradient_ms(sad_batch_t* b, double* ms_per_launch) {
    clear_error();
    SAD_REQUIRE(b && ms_per_launch, "sad_batch_gradient_ms: null argument");
    *ms_per_launch = b->grad_launches ? b->grad_ms / b->grad_launches : 0.0;
    return SAD_OK;
}
