/*
 * sad_oracle.h -- CPU restatement of SAD's fit-and-render path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path in
 * sad_gb300/csrc: only tests/, __graft_entry__.smoke() and the cpu_baseline /
 * --impl reference legs of bench.py may load it.  The product never links or
 * calls it.
 *
 * Every function restates one reference kernel or host routine of LuckyIYI/SAD
 * (paths relative to the reference project root) and cites it.  Arithmetic is
 * plain C float with -ffp-contract=off so the result is the same on x86-64 and
 * aarch64; the CUDA build contracts a*b+c into FMA and uses CUDA's expf/rsqrtf,
 * so CUDA-vs-oracle comparisons use the tolerances written in the tests, and
 * candidate-id comparisons are tie-tolerant.
 *
 * Layouts (identical to the reference's):
 *   site   : 10 x f32 = pos_x, pos_y, log_tau, radius, r, g, b, dir_x, dir_y,
 *            log_aniso  (backends/cuda/src/sad_common.cuh:21-31)
 *   adam   : 20 x f32 per site = m_pos.xy, v_pos, m_tau, v_tau, m_rad, v_rad,
 *            m_col.rgb, v_col.rgb, m_dir.xy, v_dir, m_aniso, v_aniso, pad, pad
 *   cand   : two [W*H][4] u32 arrays, 0xFFFFFFFF = empty
 *   packed : 8 x f16 per site (backends/cuda/src/candidate_pack.cu:3-28)
 *   pairs  : [M][2] u32 = (key, value)
 */
#ifndef SAD_ORACLE_H
#define SAD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_K 8
#define ORC_EMPTY 0xFFFFFFFFu

typedef struct {
    float px, py, log_tau, radius, r, g, b, dx, dy, log_aniso;
} orc_site;

typedef struct {
    double px, py, log_tau, radius, r, g, b, dx, dy, log_aniso;
} orc_site_d;

/* ---- scalar helpers ---------------------------------------------------- */
uint16_t orc_f32_to_f16(float f);
float orc_f16_to_f32(uint16_t h);
uint32_t orc_xorshift32(uint32_t x);
uint32_t orc_jump_step_for_index(uint32_t step_index, int width, int height);
uint32_t orc_pack_jump_step(uint32_t step_index, int width, int height);
uint32_t orc_hilbert_index(uint32_t x, uint32_t y, int bits);
int orc_hilbert_bits_for_size(int width, int height);
float orc_dmix2(const orc_site* s, float ux, float uy, float inv_scale_sq);

/* ---- render / adjoint ---------------------------------------------------- */
void orc_render(const uint32_t* cand0, const uint32_t* cand1, const orc_site* sites,
                uint32_t site_count, int width, int height, int cand_width, int cand_height,
                float inv_scale_sq, float* out_rgb);
void orc_render_d(const uint32_t* cand0, const uint32_t* cand1, const orc_site_d* sites,
                  uint32_t site_count, int width, int height, double inv_scale_sq, double* out_rgb);
/* grad_sites [N,10] is accumulated (caller zeroes it); abs_sites (nullable)
 * receives the sum of |term| per component, the scale used by tolerance checks. */
void orc_render_backward(const uint32_t* cand0, const uint32_t* cand1, const orc_site* sites,
                         uint32_t site_count, int width, int height, int cand_width, int cand_height,
                         float inv_scale_sq, const float* grad_out, double* grad_sites, double* abs_sites);
void orc_render_backward_d(const uint32_t* cand0, const uint32_t* cand1, const orc_site_d* sites,
                           uint32_t site_count, int width, int height, double inv_scale_sq,
                           const double* grad_out, double* grad_sites);

/* ---- candidates ---------------------------------------------------------- */
void orc_init_candidates(uint32_t* cand0, uint32_t* cand1, uint32_t site_count, uint32_t seed,
                         int per_pixel, int width, int height);
void orc_clear_candidates(uint32_t* cand0, uint32_t* cand1, int width, int height);
void orc_pack_candidate_sites(const orc_site* sites, uint16_t* packed, uint32_t site_count);
void orc_jfa_seed(uint32_t* cand0, const orc_site* sites, uint32_t site_count, int width,
                  int height, int cand_downscale);
void orc_jfa_flood(const uint32_t* in0, uint32_t* out0, const orc_site* sites, uint32_t site_count,
                   uint32_t step, float inv_scale_sq, int width, int height, int cand_downscale,
                   int target_width, int target_height);
void orc_vpt_pass(const uint32_t* in0, const uint32_t* in1, uint32_t* out0, uint32_t* out1,
                  const uint16_t* packed, uint32_t site_count, uint32_t step, float inv_scale_sq,
                  uint32_t step_high, float radius_scale, uint32_t radius_probes, uint32_t inject_count,
                  const uint32_t* hilbert_order, const uint32_t* hilbert_pos, uint32_t hilbert_probes,
                  uint32_t hilbert_window, int cand_downscale, int target_width, int target_height,
                  int width, int height);
/* distance used to rank candidates in the VPT pass (f16-packed site) */
float orc_packed_distance(const uint16_t* packed_site, float ux, float uy, float inv_scale_sq);

/* ---- training ------------------------------------------------------------ */
/* grads: 10 arrays of N floats, SoA order pos_x,pos_y,log_tau,radius,r,g,b,dir_x,dir_y,log_aniso
 * accumulated in double; removal (nullable) accumulated in double. */
void orc_compute_gradients(const uint32_t* cand0, const uint32_t* cand1, const float* target,
                           const float* rendered, const float* mask, const orc_site* sites,
                           uint32_t site_count, int width, int height, int cand_width,
                           int cand_height, float inv_scale_sq, float ssim_weight,
                           double* grads, double* abs_grads, double* removal);
void orc_tau_diffuse(const uint32_t* cand0, const uint32_t* cand1, const orc_site* sites,
                     const float* grad_raw, const float* grad_in, float* grad_out,
                     uint32_t site_count, float lambda, int width, int height, int cand_downscale);
void orc_adam_update(orc_site* sites, float* adam, const float* grads /*10 x N SoA*/, uint32_t n,
                     float lr_pos, float lr_tau, float lr_radius, float lr_color, float lr_dir,
                     float lr_aniso, float beta1, float beta2, float eps, uint32_t t, int width,
                     int height);
void orc_densify_score_pairs(const orc_site* sites, const float* mass, const float* energy,
                             uint32_t* pairs, uint32_t site_count, float min_mass, float alpha,
                             uint32_t pair_count);
void orc_prune_score_pairs(const orc_site* sites, const float* removal, uint32_t* pairs,
                           uint32_t site_count, float delta_norm, uint32_t pair_count);
/* stable LSD semantics of backends/cuda/src/radix_sort.cu: sort by (key & mask),
 * mask = 0xFFFF when max_key_exclusive <= 65536 else 0xFFFFFFFF. */
void orc_radix_sort_pairs(uint32_t* pairs, uint32_t count, uint32_t max_key_exclusive);
void orc_write_split_indices(const uint32_t* pairs, uint32_t* indices, uint32_t k);
void orc_prune_sites(orc_site* sites, const uint32_t* indices, uint32_t count);
void orc_split_sites(orc_site* sites, float* adam, const uint32_t* split_idx, uint32_t num,
                     const float* mass, const float* err_w, const float* err_wx, const float* err_wy,
                     const float* err_wxx, const float* err_wxy, const float* err_wyy,
                     uint32_t current_count, const float* target, int width, int height);
void orc_init_gradient_weighted(orc_site* sites, uint32_t n, const float* target, const float* mask,
                                float grad_threshold, uint32_t max_attempts, float init_log_tau,
                                float init_radius, int width, int height);
void orc_site_stats(const uint32_t* cand0, const uint32_t* cand1, const float* target,
                    const float* mask, const orc_site* sites, uint32_t site_count, int width,
                    int height, int cand_width, int cand_height, float inv_scale_sq, double* stats8);
void orc_hilbert_pairs(const orc_site* sites, uint32_t* pairs, uint32_t site_count,
                       uint32_t padded_count, int width, int height, int bits);
void orc_write_hilbert_order(const uint32_t* pairs, uint32_t* order, uint32_t* pos, uint32_t n);
double orc_psnr(const float* rendered, const float* target, const float* mask, int width, int height);
double orc_ssim_sum(const float* rendered, const float* target, const float* mask, int width, int height);
uint32_t orc_count_active(const orc_site* sites, uint32_t n);

/* ---- host schedule ------------------------------------------------------- */
int orc_simulate_final_sites(int init_sites, int max_sites, int iters, int densify_enabled,
                             int densify_start, int densify_end, int densify_freq,
                             float densify_pct, int prune_during_densify, int prune_start,
                             int prune_end, int prune_freq, float prune_pct, int max_split);
/* out4 = {densify_pct, prune_pct, final_sites, achieved_bpp} */
void orc_solve_target_bpp(float target_bpp, int width, int height, int init_sites, int max_sites,
                          int iters, int densify_enabled, int densify_start, int densify_end,
                          int densify_freq, float base_densify, int prune_during_densify,
                          int prune_start, int prune_end, int prune_freq, float base_prune,
                          int max_split, float* out4);

/* Per-pixel terms of the fused gradient kernel (full-resolution candidate
 * field, no SSIM): candidate entries in ids/g, unique-site removal deltas in
 * rid/rdelta.  Returns the number of candidate entries. */
int orc_pixel_terms(const uint32_t* cand0, const uint32_t* cand1, const float* target,
                    const orc_site* sites, uint32_t site_count, int x, int y, int width, int height,
                    float inv_scale_sq, int want_removal, uint32_t* ids, float (*g)[10],
                    uint32_t* rid, float* rdelta, int* nrem);

/* ---- CPU fit (timed CPU baseline) ---------------------------------------- */
typedef struct {
    int iterations, n_sites, max_sites;
    float prune_pct; int prune_start, prune_freq, prune_end;
    int densify; float densify_pct, densify_alpha; int densify_start, densify_freq, densify_end;
    int prune_during_densify;
    int cand_freq, cand_passes;
    float cand_radius_scale; uint32_t cand_radius_probes, cand_inject;
    uint32_t hilbert_window, hilbert_probes;
    float lr_pos, lr_tau, lr_radius, lr_color, lr_dir, lr_aniso;
    float beta1, beta2, eps, init_log_tau, init_radius;
    int threads;
} orc_fit_config;

typedef struct orc_fit orc_fit;
orc_fit* orc_fit_create(const orc_fit_config* cfg, const float* target, int width, int height,
                        const orc_site* init_sites /* nullable: gradient-weighted init */,
                        int n_init);
/* runs iterations [begin, end) of the schedule; returns 0 */
int orc_fit_run(orc_fit* f, int begin, int end);
double orc_fit_psnr(orc_fit* f);
int orc_fit_sites(orc_fit* f, orc_site* out, int capacity, int active_only);
void orc_fit_destroy(orc_fit* f);
void orc_set_threads(int n);

/* 16-byte quantised inference sites: packed [n][4] u32, quant the 10 range floats
 * (log_tau min/scale, radius min/scale, r, g, b min/scale). */
void orc_pack_inference_sites(const orc_site* sites, uint32_t n, int width, int height,
                              uint32_t* packed, float* quant);
void orc_unpack_inference_sites(const uint32_t* packed, const float* quant, uint32_t n, int width,
                                int height, orc_site* sites);

#ifdef __cplusplus
}
#endif
#endif
