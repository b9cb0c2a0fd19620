/*
 * sad_oracle_fit.c -- CPU fit loop over the oracle kernels.
 *
 * TEST INFRASTRUCTURE ONLY: the timed CPU baseline of bench.py and the
 * end-to-end quality check of the tests.  Follows the iteration schedule of
 * backends/cuda/src/sad_cuda.cu:2158-2479 (trainVoronoi's loop): candidate
 * refresh every CAND_UPDATE_FREQ iterations (the gradient step of that
 * iteration still sees the old field, tau diffusion the new one), fused
 * gradients, 4 tau-diffusion passes with lambda = 0.05 (0.1 + 0.9 it/iters),
 * Adam with t = it + 1, gradient clear, and prune by removal-delta score.
 */
#include "sad_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

struct orc_fit {
    orc_fit_config c;
    int w, h, cw, ch;
    uint32_t cap, n;
    int active;
    float inv_s2;
    float* target;
    float* mask;
    float mask_sum;
    orc_site* sites;
    float* adam;
    float* grads;
    float *tau_raw, *tau_tmp, *removal;
    float* stats;
    uint32_t* pairs;
    uint32_t* idx;
    uint32_t *c0[2], *c1[2];
    int cur;
    uint16_t* packed;
    uint32_t *horder, *hpos;
    int hready;
    uint32_t hcount;
    uint32_t jump_pass;
    int eff_prune_start, eff_prune_end;
    float* render;
};

static void* xcalloc(size_t n, size_t s) { return calloc(n ? n : 1, s); }

orc_fit* orc_fit_create(const orc_fit_config* cfg, const float* target, int w, int h,
                        const orc_site* init_sites, int n_init) {
    orc_fit* f = (orc_fit*)xcalloc(1, sizeof(orc_fit));
    f->c = *cfg;
    if (f->c.threads > 0) orc_set_threads(f->c.threads);
    f->w = w; f->h = h; f->cw = w; f->ch = h;
    int n0 = init_sites ? n_init : cfg->n_sites;
    /* planSiteCapacity, backends/cuda/src/sad_cuda.cu:1079-1101 (densify is always
     * "enabled" in the reference CLI, so the capacity is max_sites). */
    int maxcap = cfg->max_sites > 0 ? cfg->max_sites : 2 * w * h;
    f->cap = (uint32_t)(n0 > maxcap ? n0 : maxcap);
    if (!cfg->densify) f->cap = (uint32_t)n0;
    f->n = (uint32_t)n0;
    f->active = n0;
    float md = (float)(w > h ? w : h);
    f->inv_s2 = 1.0f / (md * md);
    size_t np = (size_t)w * h;
    f->target = (float*)malloc(np * 3 * sizeof(float));
    memcpy(f->target, target, np * 3 * sizeof(float));
    f->mask = NULL;
    f->mask_sum = (float)np;
    f->sites = (orc_site*)xcalloc(f->cap, sizeof(orc_site));
    f->adam = (float*)xcalloc((size_t)f->cap * 20, sizeof(float));
    f->grads = (float*)xcalloc((size_t)f->cap * 10, sizeof(float));
    f->tau_raw = (float*)xcalloc(f->cap, sizeof(float));
    f->tau_tmp = (float*)xcalloc(f->cap, sizeof(float));
    f->removal = (float*)xcalloc(f->cap, sizeof(float));
    f->stats = (float*)xcalloc((size_t)f->cap * 8, sizeof(float));
    f->pairs = (uint32_t*)xcalloc((size_t)(f->cap + 1024) * 2, sizeof(uint32_t));
    f->idx = (uint32_t*)xcalloc(65536, sizeof(uint32_t));
    for (int b = 0; b < 2; b++) {
        f->c0[b] = (uint32_t*)xcalloc(np * 4, sizeof(uint32_t));
        f->c1[b] = (uint32_t*)xcalloc(np * 4, sizeof(uint32_t));
    }
    f->packed = (uint16_t*)xcalloc((size_t)f->cap * 8, sizeof(uint16_t));
    f->horder = (uint32_t*)xcalloc(f->cap, sizeof(uint32_t));
    f->hpos = (uint32_t*)xcalloc(f->cap, sizeof(uint32_t));
    f->render = (float*)xcalloc(np * 3, sizeof(float));
    for (uint32_t i = n0; i < f->cap; i++) { f->sites[i].px = -1.0f; f->sites[i].py = -1.0f; }
    if (init_sites) {
        memcpy(f->sites, init_sites, (size_t)n0 * sizeof(orc_site));
    } else {
        orc_init_gradient_weighted(f->sites, (uint32_t)n0, f->target, NULL, 0.01f, 256,
                                   cfg->init_log_tau, cfg->init_radius, w, h);
    }
    f->active = (int)orc_count_active(f->sites, f->n);
    if (!init_sites) f->active = n0; /* the reference counts host sites (all) here */
    orc_init_candidates(f->c0[0], f->c1[0], f->n, 0u, 0, f->cw, f->ch);
    orc_jfa_seed(f->c0[0], f->sites, f->n, f->cw, f->ch, 1);
    f->cur = 0;
    f->eff_prune_start = cfg->prune_start;
    if (cfg->densify && !cfg->prune_during_densify && cfg->prune_start < cfg->densify_end)
        f->eff_prune_start = cfg->densify_end;
    f->eff_prune_end = cfg->prune_end > 0 ? cfg->prune_end : cfg->iterations - 1;
    return f;
}

/* Float accumulation of the fused gradient terms: each OpenMP task owns a 16x16
 * tile, merges the tile's contributions per site in a small table, then adds
 * the table to the shared arrays with atomics. */
#define TILE 16
#define TSLOTS 512
static void fit_gradients(orc_fit* f, const uint32_t* c0, const uint32_t* c1, int want_removal) {
    int w = f->w, h = f->h;
    int tx = (w + TILE - 1) / TILE, ty = (h + TILE - 1) / TILE;
    uint32_t n = f->n;
    float* G = f->grads;
    float* R = f->removal;
#pragma omp parallel
    {
        uint32_t* keys = (uint32_t*)malloc(TSLOTS * sizeof(uint32_t));
        float* acc = (float*)malloc((size_t)TSLOTS * 11 * sizeof(float));
#pragma omp for schedule(dynamic, 8)
        for (int t = 0; t < tx * ty; t++) {
            for (int s = 0; s < TSLOTS; s++) keys[s] = ORC_EMPTY;
            memset(acc, 0, (size_t)TSLOTS * 11 * sizeof(float));
            int bx = (t % tx) * TILE, by = (t / tx) * TILE;
            for (int y = by; y < by + TILE && y < h; y++)
                for (int x = bx; x < bx + TILE && x < w; x++) {
                    uint32_t ids[ORC_K], rid[ORC_K];
                    float g[ORC_K][10], rd[ORC_K];
                    int nrem;
                    int cnt = orc_pixel_terms(c0, c1, f->target, f->sites, n, x, y, w, h, f->inv_s2,
                                              want_removal, ids, g, rid, rd, &nrem);
                    for (int i = 0; i < cnt + nrem; i++) {
                        uint32_t id = i < cnt ? ids[i] : rid[i - cnt];
                        uint32_t s = (id * 2654435761u) & (TSLOTS - 1);
                        int placed = 0;
                        for (int pr = 0; pr < TSLOTS; pr++) {
                            uint32_t q = (s + (uint32_t)pr) & (TSLOTS - 1);
                            if (keys[q] == ORC_EMPTY) keys[q] = id;
                            if (keys[q] == id) {
                                float* a = acc + (size_t)q * 11;
                                if (i < cnt) for (int c = 0; c < 10; c++) a[c] += g[i][c];
                                else a[10] += rd[i - cnt];
                                placed = 1;
                                break;
                            }
                        }
                        (void)placed;
                    }
                }
            for (int s = 0; s < TSLOTS; s++) {
                uint32_t id = keys[s];
                if (id == ORC_EMPTY) continue;
                float* a = acc + (size_t)s * 11;
                for (int c = 0; c < 10; c++) {
#pragma omp atomic
                    G[(size_t)c * f->cap + id] += a[c];
                }
                if (want_removal && a[10] != 0.0f) {
#pragma omp atomic
                    R[id] += a[10];
                }
            }
        }
        free(keys);
        free(acc);
    }
}

static void fit_hilbert(orc_fit* f) {
    uint32_t n = f->n;
    int bits = orc_hilbert_bits_for_size(f->w, f->h);
    uint32_t padded = (n + 1023u) / 1024u * 1024u;
    uint32_t* pairs = (uint32_t*)malloc((size_t)padded * 8);
    orc_hilbert_pairs(f->sites, pairs, n, padded, f->w, f->h, bits);
    uint32_t maxk = bits >= 16 ? 0xffffffffu : (1u << (2 * bits));
    orc_radix_sort_pairs(pairs, padded, maxk);
    orc_write_hilbert_order(pairs, f->horder, f->hpos, n);
    free(pairs);
}

int orc_fit_run(orc_fit* f, int begin, int end) {
    const orc_fit_config* c = &f->c;
    size_t np = (size_t)f->w * f->h;
    for (int it = begin; it < end; it++) {
        int upd = c->cand_freq > 0 && it % c->cand_freq == 0;
        int desired_splits = (int)(f->active * c->densify_pct);
        if (desired_splits < 0) desired_splits = 0;
        int dens = c->densify && it >= c->densify_start && it <= c->densify_end &&
                   it % (c->densify_freq > 1 ? c->densify_freq : 1) == 0 && f->n < f->cap &&
                   desired_splits > 0;
        int pending = -1;
        if (upd) {
            int uses_h = c->hilbert_probes > 0 && c->hilbert_window > 0;
            if (uses_h && (!f->hready || f->hcount != f->n)) {
                fit_hilbert(f);
                f->hready = 1;
                f->hcount = f->n;
            }
            orc_pack_candidate_sites(f->sites, f->packed, f->n);
            int src = f->cur;
            int passes = c->cand_passes > 1 ? c->cand_passes : 1;
            for (int p = 0; p < passes; p++) {
                uint32_t step = orc_pack_jump_step(f->jump_pass, f->cw, f->ch);
                uint32_t hi = f->jump_pass >> 16;
                orc_vpt_pass(f->c0[src], f->c1[src], f->c0[1 - src], f->c1[1 - src], f->packed, f->n,
                             step, f->inv_s2, hi, c->cand_radius_scale, c->cand_radius_probes,
                             c->cand_inject, uses_h ? f->horder : NULL, uses_h ? f->hpos : NULL,
                             uses_h ? c->hilbert_probes : 0, uses_h ? c->hilbert_window : 0, 1,
                             f->w, f->h, f->cw, f->ch);
                f->jump_pass++;
                src = 1 - src;
            }
            if (dens) f->cur = src; else pending = src;
        }
        if (dens) {
            double* st = (double*)calloc((size_t)f->n * 8, sizeof(double));
            orc_site_stats(f->c0[f->cur], f->c1[f->cur], f->target, NULL, f->sites, f->n, f->w, f->h,
                           f->cw, f->ch, f->inv_s2, st);
            for (size_t k = 0; k < (size_t)f->n * 8; k++) {
                size_t a = k / f->n, i = k % f->n;
                f->stats[a * f->cap + i] = (float)st[k];
            }
            free(st);
            float* S = f->stats;
            orc_densify_score_pairs(f->sites, S, S + f->cap, f->pairs, f->n, 1.0f, c->densify_alpha, f->cap);
            orc_radix_sort_pairs(f->pairs, f->cap, 0xffffffffu);
            int avail = (int)(f->cap - f->n);
            int k = desired_splits < avail ? desired_splits : avail;
            if (k > 65536) k = 65536;
            if (k > 0) {
                orc_write_split_indices(f->pairs, f->idx, (uint32_t)k);
                orc_split_sites(f->sites, f->adam, f->idx, (uint32_t)k, S, S + 2 * f->cap, S + 3 * f->cap,
                                S + 4 * f->cap, S + 5 * f->cap, S + 6 * f->cap, S + 7 * f->cap, f->n,
                                f->target, f->w, f->h);
                f->n += (uint32_t)k;
                f->active += k;
            }
        }
        int prune = c->prune_pct > 0.0f && it >= f->eff_prune_start && it < f->eff_prune_end &&
                    it % (c->prune_freq > 1 ? c->prune_freq : 1) == 0;
        if (prune) memset(f->removal, 0, f->n * sizeof(float));
        fit_gradients(f, f->c0[f->cur], f->c1[f->cur], prune);
        /* tau diffusion: raw copy, pending candidates applied, 4 Jacobi passes */
        float* glt = f->grads + 2 * (size_t)f->cap;
        memcpy(f->tau_raw, glt, f->n * sizeof(float));
        float blend = (float)it / (float)(c->iterations > 1 ? c->iterations : 1);
        float lambda = 0.05f * (0.1f + 0.9f * blend);
        if (pending >= 0) f->cur = pending;
        float* in = glt;
        float* out = f->tau_tmp;
        for (int p = 0; p < 4; p++) {
            orc_tau_diffuse(f->c0[f->cur], f->c1[f->cur], f->sites, f->tau_raw, in, out, f->n, lambda,
                            f->cw, f->ch, 1);
            float* t = in; in = out; out = t;
        }
        /* Adam over the first n sites (grads are SoA with stride cap) */
        {
            float* g = (float*)malloc((size_t)f->n * 10 * sizeof(float));
            for (int k = 0; k < 10; k++) memcpy(g + (size_t)k * f->n, f->grads + (size_t)k * f->cap, f->n * sizeof(float));
            orc_adam_update(f->sites, f->adam, g, f->n, c->lr_pos, c->lr_tau, c->lr_radius, c->lr_color,
                            c->lr_dir, c->lr_aniso, c->beta1, c->beta2, c->eps, (uint32_t)(it + 1), f->w, f->h);
            free(g);
        }
        for (int k = 0; k < 10; k++) memset(f->grads + (size_t)k * f->cap, 0, f->n * sizeof(float));
        if (prune) {
            orc_prune_score_pairs(f->sites, f->removal, f->pairs, f->n, 1.0f / fmaxf(1.0f, f->mask_sum), f->cap);
            orc_radix_sort_pairs(f->pairs, f->cap, 0xffffffffu);
            int k = (int)(f->active * c->prune_pct);
            if (k < 0) k = 0;
            if (k > 65536) k = 65536;
            if (k > 0) {
                orc_write_split_indices(f->pairs, f->idx, (uint32_t)k);
                orc_prune_sites(f->sites, f->idx, (uint32_t)k);
                f->active = f->active - k > 0 ? f->active - k : 0;
            }
        }
    }
    (void)np;
    return 0;
}

double orc_fit_psnr(orc_fit* f) {
    orc_render(f->c0[f->cur], f->c1[f->cur], f->sites, f->n, f->w, f->h, f->cw, f->ch, f->inv_s2, f->render);
    return orc_psnr(f->render, f->target, NULL, f->w, f->h);
}

int orc_fit_sites(orc_fit* f, orc_site* out, int capacity, int active_only) {
    int k = 0;
    for (uint32_t i = 0; i < f->n && k < capacity; i++) {
        if (active_only && f->sites[i].px < 0.0f) continue;
        out[k++] = f->sites[i];
    }
    return k;
}

void orc_fit_destroy(orc_fit* f) {
    if (!f) return;
    free(f->target); free(f->sites); free(f->adam); free(f->grads); free(f->tau_raw);
    free(f->tau_tmp); free(f->removal); free(f->stats); free(f->pairs); free(f->idx);
    for (int b = 0; b < 2; b++) { free(f->c0[b]); free(f->c1[b]); }
    free(f->packed); free(f->horder); free(f->hpos); free(f->render);
    free(f);
}
