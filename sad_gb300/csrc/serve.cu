// serve.cu -- render from a site list: candidate field construction + render.
//
// backends/cuda/src/sad_cuda.cu:1678-1858 (renderVoronoiFromSites) with its defaults:
// one JFA round, 16 VPT passes split over the rounds, Hilbert probes when enabled.
// Kept as the reference does it:
//   * the JFA flood ping-pongs between the two halves (slots 0-3 / 4-7) of the same
//     candidate field, so slots 4-7 hold an intermediate top-4 when the first VPT pass
//     starts (runJFA, sad_cuda.cu:1616-1655);
//   * without JFA the field starts random (seed 12345) plus the site seeds;
//   * VPT passes ping-pong between the two fields and the render reads the last one.
#include "common.cuh"
#include "host_common.h"
#include "kernels.h"

namespace sad {

static inline size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

struct RenderScratch {
    SiteGeom* geom;
    SiteColor* color;
    SiteGeom* vgeom;
    uint32_t* c0[2];
    uint32_t* c1[2];
    uint32_t* horder;
    uint32_t* hpos;
    uint32_t* hpairs;
    void* sort_temp;
    size_t total;
};

static RenderScratch carve(void* base, uint32_t n, int cw, int ch) {
    RenderScratch r{};
    char* p = static_cast<char*>(base);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* q = p ? p + off : nullptr;
        off += a256(bytes);
        return q;
    };
    size_t nc = static_cast<size_t>(cw) * ch * 16;
    uint32_t padded = (n + 1023u) / 1024u * 1024u;
    r.geom = reinterpret_cast<SiteGeom*>(take(static_cast<size_t>(n) * 32));
    r.color = reinterpret_cast<SiteColor*>(take(static_cast<size_t>(n) * 16));
    r.vgeom = reinterpret_cast<SiteGeom*>(take(static_cast<size_t>(n) * 32));
    for (int b = 0; b < 2; ++b) {
        r.c0[b] = reinterpret_cast<uint32_t*>(take(nc));
        r.c1[b] = reinterpret_cast<uint32_t*>(take(nc));
    }
    r.horder = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(n) * 4));
    r.hpos = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(n) * 4));
    r.hpairs = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(padded) * 8));
    r.sort_temp = take(radix_sort_temp_bytes(padded));
    r.total = off + 256;
    return r;
}

}  // namespace sad

using namespace sad;

extern "C" size_t sad_render_scratch_bytes(uint32_t site_count, int width, int height,
                                           int cand_downscale) {
    int ds = std::max(1, cand_downscale);
    int cw = std::max(1, (width + ds - 1) / ds), ch = std::max(1, (height + ds - 1) / ds);
    return carve(nullptr, site_count, cw, ch).total;
}

// ev (nullable): three events recorded before the candidate build, before the render and
// after it.
static sad_status_t render_from_sites_impl(const sad_render_config_t* cfg, const float* sites_f, uint32_t n,
                                           int width, int height, float* out_rgb, void* scratch,
                                           size_t scratch_bytes, sad_stream_t stream, cudaEvent_t* ev) {
    SAD_REQUIRE(cfg, "sad_render_from_sites: null config");
    SAD_REQUIRE(image_size_ok(width, height), "sad_render_from_sites: invalid size");
    SAD_REQUIRE(n > 0 && sites_f && out_rgb && scratch, "sad_render_from_sites: null buffer or no sites");
    SAD_REQUIRE(cfg->candidate_passes >= 0, "sad_render_from_sites: negative candidate passes");
    int ds = std::max(1, cfg->cand_downscale);
    int cw = std::max(1, (width + ds - 1) / ds), ch = std::max(1, (height + ds - 1) / ds);
    RenderScratch need = carve(nullptr, n, cw, ch);
    SAD_REQUIRE(scratch_bytes >= need.total,
                "sad_render_from_sites: scratch smaller than sad_render_scratch_bytes()");
    uintptr_t base = (reinterpret_cast<uintptr_t>(scratch) + 255) & ~uintptr_t(255);
    RenderScratch r = carve(reinterpret_cast<void*>(base), n, cw, ch);
    cudaStream_t st = as_stream(stream);
    const Site* sites = reinterpret_cast<const Site*>(sites_f);
    float md = static_cast<float>(std::max(width, height));
    float inv_s2 = 1.0f / (md * md);

    launch_prepare_sites(sites, r.geom, r.color, n, st);
    int a = 0;  // index of the current field ("A")
    if (!cfg->use_jfa) {
        launch_init_candidates(r.c0[a], r.c1[a], n, 12345u, 0, cw, ch, st);
        launch_jfa_seed(r.c0[a], sites, n, cw, ch, ds, st);
    }
    int passes = cfg->candidate_passes;
    int rounds = cfg->use_jfa ? std::max(1, cfg->jfa_rounds) : 1;
    int base_passes = passes / rounds, rem = passes % rounds;
    launch_pack_geom(sites, r.vgeom, n, st);
    bool use_h = cfg->cand_hilbert_probes > 0 && cfg->cand_hilbert_window > 0;
    if (use_h) {
        int bits = sad_hilbert_bits_for_size(width, height);
        uint32_t padded = (n + 1023u) / 1024u * 1024u;
        launch_hilbert_pairs(sites, r.hpairs, n, padded, width, height, bits, st);
        uint32_t maxk = bits >= 16 ? 0xFFFFFFFFu : (1u << (2 * bits));
        launch_radix_sort(r.hpairs, padded, maxk, r.sort_temp, st);
        launch_hilbert_order(r.hpairs, r.horder, r.hpos, n, st);
    }
    // the timed candidate build starts here, where the reference starts it: after the
    // per-site preparation, the packed copy and the Hilbert order (sad_cuda.cu:1760-1786)
    if (ev) SAD_TRY(check_cuda(cudaEventRecord(ev[0], st), "sad_render_from_sites: event"));
    uint32_t jump_pass = 0;
    for (int round = 0; round < rounds; ++round) {
        if (cfg->use_jfa) {
            launch_clear_candidates(r.c0[a], r.c1[a], cw, ch, st);
            launch_jfa_seed(r.c0[a], sites, n, cw, ch, ds, st);
            int maxd = std::max(cw, ch), step = 1;
            while (step < maxd) step <<= 1;
            uint32_t* in = r.c0[a];
            uint32_t* out = r.c1[a];
            for (int s = step / 2; s >= 1; s /= 2) {
                launch_jfa_flood_geom(in, out, r.geom, n, static_cast<uint32_t>(s), inv_s2, cw, ch, ds,
                                      width, height, st);
                std::swap(in, out);
            }
            if (in != r.c0[a])
                SAD_TRY(check_cuda(cudaMemcpyAsync(r.c0[a], in, static_cast<size_t>(cw) * ch * 16,
                                                   cudaMemcpyDeviceToDevice, st),
                                   "sad_render_from_sites: flood copy"));
        }
        int this_passes = base_passes + (round < rem ? 1 : 0);
        VptParams p{};
        p.site_count = n;
        p.inv_scale_sq = inv_s2;
        p.radius_scale = cfg->cand_radius_scale;
        p.radius_probes = cfg->cand_radius_probes;
        p.inject_count = cfg->cand_inject_count;
        p.hilbert_order = use_h ? r.horder : nullptr;
        p.hilbert_pos = use_h ? r.hpos : nullptr;
        p.hilbert_probes = use_h ? cfg->cand_hilbert_probes : 0u;
        p.hilbert_window = use_h ? cfg->cand_hilbert_window : 0u;
        p.cand_downscale = ds;
        p.target_width = width;
        p.target_height = height;
        p.width = cw;
        p.height = ch;
        p.state = nullptr;
        for (int i = 0; i < this_passes; ++i) {
            p.step = sad_pack_jump_step(jump_pass, cw, ch);
            p.step_high = jump_pass >> 16;
            p.in0 = r.c0[a];
            p.in1 = r.c1[a];
            p.out0 = r.c0[1 - a];
            p.out1 = r.c1[1 - a];
            launch_vpt_geom(p, r.vgeom, st);
            ++jump_pass;
            a = 1 - a;
        }
    }
    if (ev) SAD_TRY(check_cuda(cudaEventRecord(ev[1], st), "sad_render_from_sites: event"));
    launch_render_prepared(r.c0[a], r.c1[a], out_rgb, r.geom, r.color, inv_s2, n, width, height, cw,
                           ch, st);
    if (ev) SAD_TRY(check_cuda(cudaEventRecord(ev[2], st), "sad_render_from_sites: event"));
    return check_launch("sad_render_from_sites");
}

extern "C" sad_status_t sad_render_from_sites(const sad_render_config_t* cfg, const float* sites_f,
                                              uint32_t n, int width, int height, float* out_rgb,
                                              void* scratch, size_t scratch_bytes,
                                              sad_stream_t stream) {
    NvtxRange r_nvtx("render from sites");
    clear_error();
    return render_from_sites_impl(cfg, sites_f, n, width, height, out_rgb, scratch, scratch_bytes, stream,
                                  nullptr);
}

extern "C" sad_status_t sad_render_from_sites_timed(const sad_render_config_t* cfg, const float* sites_f,
                                                    uint32_t n, int width, int height, float* out_rgb,
                                                    void* scratch, size_t scratch_bytes, sad_stream_t stream,
                                                    float* cand_ms, float* render_ms) {
    clear_error();
    SAD_REQUIRE(cand_ms && render_ms, "sad_render_from_sites_timed: null timing output");
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    sad_status_t s = SAD_OK;
    for (auto& e : ev)
        if (s == SAD_OK) s = check_cuda(cudaEventCreate(&e), "sad_render_from_sites_timed: event");
    if (s == SAD_OK)
        s = render_from_sites_impl(cfg, sites_f, n, width, height, out_rgb, scratch, scratch_bytes, stream, ev);
    if (s == SAD_OK) s = check_cuda(cudaEventSynchronize(ev[2]), "sad_render_from_sites_timed: sync");
    if (s == SAD_OK) s = check_cuda(cudaEventElapsedTime(cand_ms, ev[0], ev[1]), "sad_render_from_sites_timed");
    if (s == SAD_OK) s = check_cuda(cudaEventElapsedTime(render_ms, ev[1], ev[2]), "sad_render_from_sites_timed");
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    return s;
}
