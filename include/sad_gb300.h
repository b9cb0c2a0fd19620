/*
 * sad_gb300.h -- C ABI of the GB300-native SAD fit-and-render path.
 *
 * One shared library, libsad_gb300.so, built for sm_103a.  Conventions:
 *   - Every pointer argument named *_dev / cand / sites / grad / pairs ... is a device
 *     pointer owned by the caller, unless the comment says "host".
 *   - Every call is asynchronous on the given stream (NULL = legacy default stream) and
 *     returns a status; sad_last_error() gives the message of the last failure on the
 *     calling thread.  Launch-configuration errors are reported by the call itself;
 *     faults inside a kernel surface at the next synchronising call, as with any CUDA
 *     work.
 *   - Layouts are the reference's (LuckyIYI/SAD): a site is 10 f32 (pos_x, pos_y,
 *     log_tau, radius, r, g, b, dir_x, dir_y, log_aniso); a candidate field is two
 *     [W*H][4] u32 arrays, 0xFFFFFFFF = empty; score pairs are [M][2] u32 (key, value);
 *     the f16 packed site is 8 halves (pos, log_tau, radius, dir, log_aniso, 0).
 *   - The Adam state is 20 f32 per site: m_pos.xy, v_pos, m_log_tau, v_log_tau,
 *     m_radius, v_radius, m_color.rgb, v_color.rgb, m_dir.xy, v_dir, m_log_aniso,
 *     v_log_aniso, 2 x pad.  (The reference reinterprets a [N,20] tensor as its
 *     88-byte AdamState struct, which reads past the tensor; this layout is the packed
 *     20-float order the tensor shape implies.)
 *
 * The "replaces" line of each entry point cites the reference interface it stands in
 * for (file:line within the reference project).
 */
#ifndef SAD_GB300_H
#define SAD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SAD_GB300_ABI_VERSION 1
#define SAD_NUM_CANDIDATES 8
#define SAD_SITE_FLOATS 10
#define SAD_ADAM_FLOATS 20
#define SAD_MAX_SPLIT_INDICES 65536

typedef struct CUstream_st* sad_stream_t; /* == cudaStream_t */

typedef enum {
    SAD_OK = 0,
    SAD_ERR_INVALID_ARGUMENT = 1,
    SAD_ERR_CUDA = 2,
    SAD_ERR_OUT_OF_MEMORY = 3,
    SAD_ERR_UNSUPPORTED = 4,
    SAD_ERR_INTERNAL = 5,
    SAD_ERR_CANCELLED = 6   /* an executor request withdrawn before it started */
} sad_status_t;

/* ------------------------------------------------------------------------ */
/* library                                                                   */
/* ------------------------------------------------------------------------ */
const char* sad_last_error(void);
const char* sad_version(void);
int sad_abi_version(void);
/* Number of kernel launches issued by this library since load (graph replays count
 * every kernel node they run). */
uint64_t sad_launch_count(void);

/* ------------------------------------------------------------------------ */
/* per-pixel kernels                                                          */
/* ------------------------------------------------------------------------ */

/* Softmax-over-8-candidates render, out_rgb [H,W,3] f32.
 * replaces: launchRenderVoronoi, backends/cuda/src/render.cu:159-179 */
sad_status_t sad_render(const uint32_t* cand0, const uint32_t* cand1, float* out_rgb,
                        const float* sites, float inv_scale_sq, uint32_t site_count, int width,
                        int height, int cand_width, int cand_height, sad_stream_t stream);

/* Adjoint of sad_render: dL/dsites [N,10] ACCUMULATED into grad_sites (zero it first).
 * Softmax weights are recomputed, nothing is stored by the forward.
 * replaces: render_sad_backward_kernel, backends/pytorch/torch_ext/cuda/sad_bindings.cu:100-207
 * (launched at sad_bindings.cu:733-747) */
sad_status_t sad_render_backward(const uint32_t* cand0, const uint32_t* cand1,
                                 const float* grad_rgb, float* grad_sites, const float* sites,
                                 float inv_scale_sq, uint32_t site_count, int width, int height,
                                 int cand_width, int cand_height, sad_stream_t stream);

/* Random (xorshift) or per-pixel-neighbourhood candidate init.
 * replaces: launchInitCandidates, backends/cuda/src/render.cu:181-197 */
sad_status_t sad_init_candidates(uint32_t* cand0, uint32_t* cand1, uint32_t site_count,
                                 uint32_t seed, int per_pixel, int width, int height,
                                 sad_stream_t stream);

/* Fill both fields with 0xFFFFFFFF.
 * replaces: launchClearCandidates, backends/cuda/src/render.cu:199-211 */
sad_status_t sad_clear_candidates(uint32_t* cand0, uint32_t* cand1, int width, int height,
                                  sad_stream_t stream);

/* ------------------------------------------------------------------------ */
/* candidate search                                                           */
/* ------------------------------------------------------------------------ */

/* Site -> 8 x f16 (round to nearest even).  packed is [N,8] f16.
 * replaces: launchPackCandidateSites, backends/cuda/src/candidate_pack.cu:31-38 */
sad_status_t sad_pack_candidate_sites(const float* sites, uint16_t* packed, uint32_t site_count,
                                      sad_stream_t stream);

/* Write each active site's id into slot 0 of its home texel of cand0.  Where several
 * sites share a texel the lowest id wins (the reference's store is an unordered race).
 * replaces: launchJFASeed, backends/cuda/src/jfa.cu:391-406 */
sad_status_t sad_jfa_seed(uint32_t* cand0, const float* sites, uint32_t site_count, int width,
                          int height, int cand_downscale, sad_stream_t stream);

/* One jump-flood pass keeping the 4 closest (cand0 only).
 * replaces: launchJFAFlood, backends/cuda/src/jfa.cu:408-429 */
sad_status_t sad_jfa_flood(const uint32_t* in_cand0, uint32_t* out_cand0, const float* sites,
                           uint32_t site_count, uint32_t step_size, float inv_scale_sq, int width,
                           int height, int cand_downscale, int target_width, int target_height,
                           sad_stream_t stream);

/* One VPT top-8 propagation pass over f16 packed sites.  step = (jump << 16) | index.
 * hilbert_order / hilbert_pos may be NULL when hilbert_probes or hilbert_window is 0.
 * replaces: launchUpdateCandidates, backends/cuda/src/jfa.cu:431-464 */
sad_status_t sad_update_candidates(const uint32_t* in_cand0, const uint32_t* in_cand1,
                                   uint32_t* out_cand0, uint32_t* out_cand1,
                                   const uint16_t* packed_sites, uint32_t site_count,
                                   uint32_t step, float inv_scale_sq, uint32_t step_high,
                                   float radius_scale, uint32_t radius_probes,
                                   uint32_t inject_count, const uint32_t* hilbert_order,
                                   const uint32_t* hilbert_pos, uint32_t hilbert_probes,
                                   uint32_t hilbert_window, int cand_downscale, int target_width,
                                   int target_height, int width, int height, sad_stream_t stream);

/* Jump step of the VPT schedule: pow2(maxdim) >> (min(i, stages-1) + 1), and its packed
 * form (jump << 16) | (i & 0xffff).
 * replaces: jumpStepForIndex / packJumpStep, backends/cuda/src/sad_cuda.cu:1157-1183 */
uint32_t sad_jump_step_for_index(uint32_t step_index, int width, int height);
uint32_t sad_pack_jump_step(uint32_t step_index, int width, int height);

/* ------------------------------------------------------------------------ */
/* training kernels                                                           */
/* ------------------------------------------------------------------------ */

/* Fused forward + dL/dpred = 2 (pred - target) (+ SSIM term when ssim_weight > 0, which
 * reads `rendered`) + per-site gradients ACCUMULATED into the 10 SoA arrays; when
 * compute_removal != 0 also accumulates the removal delta.  mask may be NULL (all 1).
 * replaces: launchComputeGradientsTiled, backends/cuda/src/gradients.cu:491-531 */
sad_status_t sad_compute_gradients_tiled(
    const uint32_t* cand0, const uint32_t* cand1, const float* target, const float* rendered,
    const float* mask, float* grad_pos_x, float* grad_pos_y, float* grad_log_tau,
    float* grad_radius, float* grad_color_r, float* grad_color_g, float* grad_color_b,
    float* grad_dir_x, float* grad_dir_y, float* grad_log_aniso, const float* sites,
    float inv_scale_sq, uint32_t site_count, float* removal_delta, uint32_t compute_removal,
    float ssim_weight, int width, int height, int cand_width, int cand_height,
    sad_stream_t stream);

/* The trainer's form of the same evaluation, the kernel a fit runs every iteration: the
 * candidate field's 16x16-tile registration, then per-site sums in exact 64-bit fixed
 * point (value * 2^24, bitwise reproducible).  fix12_out is a zero-initialised device
 * [site_count][12] int64 buffer receiving the sums: slots 0-9 the gradients in the order
 * of sad_compute_gradients_tiled's arrays; with compute_removal, slot 10 the removal delta
 * times *removal_scale_out (a power of two, which may exceed 1, chosen for the image size
 * so that the sums fit in int64) and slot 11 the
 * number of pixels whose delta is the 1e6 sentinel (excluded from slot 10).
 * scratch: sad_compute_gradients_fixed_scratch_bytes(site_count, width, height) bytes.
 * replaces: launchComputeGradientsTiled, backends/cuda/src/gradients.cu:491-531, as
 * trainVoronoi calls it each iteration (backends/cuda/src/sad_cuda.cu:2319-2331) */
size_t sad_compute_gradients_fixed_scratch_bytes(uint32_t site_count, int width, int height);
sad_status_t sad_compute_gradients_fixed(
    const uint32_t* cand0, const uint32_t* cand1, const float* target, const float* rendered,
    const float* mask, const float* sites, float inv_scale_sq, uint32_t site_count,
    uint32_t compute_removal, float ssim_weight, int width, int height, int cand_width,
    int cand_height, long long* fix12_out, float* removal_scale_out, void* scratch,
    size_t scratch_bytes, sad_stream_t stream);

/* One Jacobi pass of the log_tau gradient diffusion.
 * replaces: launchTauDiffuse, backends/cuda/src/tau_diffusion.cu:88-101 */
sad_status_t sad_tau_diffuse(const uint32_t* cand0, const uint32_t* cand1, const float* sites,
                             const float* grad_raw, const float* grad_in, float* grad_out,
                             uint32_t site_count, float lambda, int width, int height,
                             int cand_downscale, sad_stream_t stream);

/* Per-site Adam step (t = 1-based step), gradients normalised by 1/(W*H); inactive
 * sites are skipped.
 * replaces: launchAdamUpdate, backends/cuda/src/adam.cu:224-251 */
sad_status_t sad_adam_update(float* sites, float* adam, const float* grad_pos_x,
                             const float* grad_pos_y, const float* grad_log_tau,
                             const float* grad_radius, const float* grad_color_r,
                             const float* grad_color_g, const float* grad_color_b,
                             const float* grad_dir_x, const float* grad_dir_y,
                             const float* grad_log_aniso, float lr_pos, float lr_tau,
                             float lr_radius, float lr_color, float lr_dir, float lr_aniso,
                             float beta1, float beta2, float eps, uint32_t t,
                             uint32_t site_count, int width, int height, sad_stream_t stream);

/* replaces: launchClearGradients / launchClearBuffer, backends/cuda/src/adam.cu:253-281 */
sad_status_t sad_clear_gradients(float* grad_pos_x, float* grad_pos_y, float* grad_log_tau,
                                 float* grad_radius, float* grad_color_r, float* grad_color_g,
                                 float* grad_color_b, float* grad_dir_x, float* grad_dir_y,
                                 float* grad_log_aniso, uint32_t count, sad_stream_t stream);
sad_status_t sad_clear_buffer(float* buffer, uint32_t count, sad_stream_t stream);

/* ------------------------------------------------------------------------ */
/* densify / prune / sort                                                     */
/* ------------------------------------------------------------------------ */

/* key = 0xFFFFFFFF - bits(max(energy,0) / max(mass,1e-8)^alpha) for active sites with
 * mass > min_mass and finite energy, else (0xFFFFFFFF, 0xFFFFFFFF); pairs [pair_count][2].
 * replaces: launchComputeDensifyScorePairs, backends/cuda/src/densify_prune.cu:359-376 */
sad_status_t sad_compute_densify_score_pairs(const float* sites, const float* mass,
                                             const float* energy, uint32_t* pairs,
                                             uint32_t site_count, float min_mass,
                                             float score_alpha, uint32_t pair_count,
                                             sad_stream_t stream);

/* key = bits(max(removal_delta * delta_norm, 0)) for active sites with a finite value.
 * replaces: launchComputePruneScorePairs, backends/cuda/src/densify_prune.cu:378-393 */
sad_status_t sad_compute_prune_score_pairs(const float* sites, const float* removal_delta,
                                           uint32_t* pairs, uint32_t site_count,
                                           float delta_norm, uint32_t pair_count,
                                           sad_stream_t stream);

/* Stable LSD radix sort of (key, value) pairs by key, ascending: 2 eight-bit passes
 * (low 16 key bits) when max_key_exclusive <= 65536, else 4.  `temp` is device scratch
 * of at least sad_radix_sort_temp_bytes(count) bytes.
 * replaces: launchRadixSortUInt2, backends/cuda/src/radix_sort.cu:279-336 */
size_t sad_radix_sort_temp_bytes(uint32_t count);
sad_status_t sad_radix_sort_pairs(uint32_t* pairs, uint32_t count, uint32_t max_key_exclusive,
                                  void* temp, size_t temp_bytes, sad_stream_t stream);

/* The same sort without caller scratch and without allocating: its scratch is a fixed
 * device array of the library, sized for SAD_NOALLOC_SORT_MAX_PAIRS pairs; larger counts
 * are rejected (SAD_ERR_INVALID_ARGUMENT).  It serves hosts that must not allocate device
 * memory on their call path: one with a fixed, pre-reserved memory budget, or a
 * latency-bound loop in which an allocation call (which can synchronise the device) is
 * not acceptable.  Each call looks the array's address up on the current device (a host
 * lookup); the first call on a device may load the module and should come before any
 * stream capture.  Nothing in the scratch needs to
 * start at zero.  Overlapping calls on one device (other streams or host threads) share
 * the scratch and race: the caller must serialise them.
 * No counterpart in the reference (its sort always takes caller-allocated scratch). */
#define SAD_NOALLOC_SORT_MAX_PAIRS 262144
sad_status_t sad_radix_sort_pairs_noalloc(uint32_t* pairs, uint32_t count,
                                          uint32_t max_key_exclusive, sad_stream_t stream);

/* indices[i] = pairs[i].value for i < k.
 * replaces: launchWriteSplitIndicesFromSorted, backends/cuda/src/densify_prune.cu:395-407 */
sad_status_t sad_write_split_indices(const uint32_t* pairs, uint32_t* indices, uint32_t k,
                                     sad_stream_t stream);

/* Mark listed sites inactive (position = (-1,-1)); 0xFFFFFFFF entries are skipped.
 * replaces: launchPruneSitesByIndex, backends/cuda/src/densify_prune.cu:409-421 */
sad_status_t sad_prune_sites(float* sites, const uint32_t* indices, uint32_t count,
                             sad_stream_t stream);

/* Stream compaction of the active sites: alive_out[0..k) = the ascending indices i <
 * site_count whose pos_x >= 0, and *count_dev = k (a device word, written on the stream).
 * scratch: sad_compact_active_scratch_bytes(site_count) bytes.  The trainer runs the same
 * kernels after every prune, so its per-site kernels walk only the active sites.
 * replaces: filterActiveSites, backends/cuda/src/sad_cuda.cu:1657-1666 (the reference
 * compacts only on the host, at export) */
size_t sad_compact_active_scratch_bytes(uint32_t site_count);
sad_status_t sad_compact_active(const float* sites, uint32_t site_count, uint32_t* alive_out,
                                uint32_t* count_dev, void* scratch, size_t scratch_bytes,
                                sad_stream_t stream);

/* Split parents along the error-covariance principal axis (or the image gradient); the
 * second child goes to current_site_count + i; both Adam states are reset.
 * replaces: launchSplitSites, backends/cuda/src/densify_prune.cu:335-357 */
sad_status_t sad_split_sites(float* sites, float* adam, const uint32_t* split_indices,
                             uint32_t num_to_split, const float* mass, const float* err_w,
                             const float* err_wx, const float* err_wy, const float* err_wxx,
                             const float* err_wxy, const float* err_wyy,
                             uint32_t current_site_count, const float* target, int width,
                             int height, sad_stream_t stream);

/* Per-site mass, energy and error moments (8 arrays of site_count, ACCUMULATED).
 * replaces: launchComputeSiteStatsSimple, backends/cuda/src/utils.cu:314-350 (which
 * also zeroes the arrays; here the caller does) */
sad_status_t sad_compute_site_stats(const uint32_t* cand0, const uint32_t* cand1,
                                    const float* target, const float* mask, const float* sites,
                                    float inv_scale_sq, uint32_t site_count, float* mass,
                                    float* energy, float* err_w, float* err_wx, float* err_wy,
                                    float* err_wxx, float* err_wxy, float* err_wyy, int width,
                                    int height, int cand_width, int cand_height,
                                    sad_stream_t stream);

/* Gradient-weighted site init: R2 low-discrepancy proposals accepted where the Sobel
 * magnitude of the target exceeds grad_threshold, up to max_attempts per site, seeds
 * handed out in site order.  Synchronises `stream` (it sizes its proposal batches on the
 * host); temp is device scratch of sad_init_temp_bytes(site_count) bytes.
 * replaces: launchInitGradientWeighted, backends/cuda/src/densify_prune.cu:312-333 */
size_t sad_init_temp_bytes(uint32_t site_count);
sad_status_t sad_init_gradient_weighted(float* sites, uint32_t site_count, const float* target,
                                        const float* mask, float grad_threshold,
                                        uint32_t max_attempts, float init_log_tau,
                                        float init_radius, int width, int height, void* temp,
                                        size_t temp_bytes, sad_stream_t stream);

/* Hilbert key pairs (key, site) for the first site_count of padded_count entries, the
 * rest (0xFFFFFFFF, 0); and the order / inverse-order arrays of sorted pairs.
 * replaces: computeHilbertPairsKernel / writeHilbertOrderKernel,
 * backends/cuda/src/sad_cuda.cu:1547-1584 */
sad_status_t sad_hilbert_pairs(const float* sites, uint32_t* pairs, uint32_t site_count,
                               uint32_t padded_count, int width, int height, int bits,
                               sad_stream_t stream);
sad_status_t sad_write_hilbert_order(const uint32_t* sorted_pairs, uint32_t* order,
                                     uint32_t* pos, uint32_t site_count, sad_stream_t stream);
int sad_hilbert_bits_for_size(int width, int height);

/* Sum of squared error over masked pixels (atomically added to *mse_accum, zero it
 * first), the SSIM sum, and the active-site count (added to *count).
 * replaces: launchComputePSNR / launchComputeSSIM / launchCountActiveSites,
 * backends/cuda/src/utils.cu:258-312 */
sad_status_t sad_compute_mse(const float* rendered, const float* target, const float* mask,
                             float* mse_accum, int width, int height, sad_stream_t stream);
sad_status_t sad_compute_ssim(const float* rendered, const float* target, const float* mask,
                              float* ssim_accum, int width, int height, sad_stream_t stream);
sad_status_t sad_count_active_sites(const float* sites, uint32_t* count, uint32_t site_count,
                                    sad_stream_t stream);

/* ------------------------------------------------------------------------ */
/* host schedule                                                              */
/* ------------------------------------------------------------------------ */

/* bpp -> site-count rule: target = round(bpp * W * H / 128); the densify / prune
 * percentiles are scaled by the factor whose simulated final count is closest.
 * replaces: solveTargetBpp / simulateFinalSites, backends/cuda/src/sad_cuda.cu:904-1066 */
typedef struct {
    float densify_percentile;
    float prune_percentile;
    int final_sites;
    float achieved_bpp;
} sad_bpp_solution_t;
sad_status_t sad_solve_target_bpp(float target_bpp, int width, int height, int init_sites,
                                  int max_sites, int iters, int densify_enabled,
                                  int densify_start, int densify_end, int densify_freq,
                                  float base_densify, int prune_during_densify, int prune_start,
                                  int prune_end, int prune_freq, float base_prune,
                                  int max_split_indices, sad_bpp_solution_t* out);
int sad_simulate_final_sites(int init_sites, int max_sites, int iters, int densify_enabled,
                             int densify_start, int densify_end, int densify_freq,
                             float densify_percentile, int prune_during_densify,
                             int prune_start, int prune_end, int prune_freq,
                             float prune_percentile, int max_split_indices);

/* ------------------------------------------------------------------------ */
/* trainer: the whole fit on the device                                       */
/* ------------------------------------------------------------------------ */

/* The training_config.json knobs (names in comments) plus the CLI-only options.
 * replaces: Defaults / TrainingOptions, backends/cuda/src/sad_cuda.cu:422-640 */
typedef struct {
    int n_sites;                   /* DEFAULT_SITES */
    int max_sites;                 /* DEFAULT_MAX_SITES */
    int iterations;                /* DEFAULT_ITERS */
    float target_bpp;              /* DEFAULT_TARGET_BPP (<= 0: off) */
    float prune_percentile;        /* PRUNE_PERCENTILE */
    int prune_during_densify;      /* PRUNE_DURING_DENSIFY */
    int prune_start, prune_freq, prune_end;       /* PRUNE_START/FREQ/END */
    int densify;                   /* densify enabled (the reference CLI always sets it) */
    int densify_start, densify_freq, densify_end; /* DENSIFY_START/FREQ/END */
    float densify_percentile;      /* DENSIFY_PERCENTILE */
    float densify_score_alpha;     /* DENSIFY_SCORE_ALPHA */
    int cand_update_freq;          /* CAND_UPDATE_FREQ */
    int cand_update_passes;        /* CAND_UPDATE_PASSES */
    int cand_downscale;            /* CAND_DOWNSCALE */
    float cand_radius_scale;       /* CAND_RADIUS_SCALE */
    uint32_t cand_radius_probes;   /* CAND_RADIUS_PROBES */
    uint32_t cand_inject_count;    /* CAND_INJECT_COUNT */
    uint32_t cand_hilbert_window;  /* CAND_HILBERT_WINDOW */
    uint32_t cand_hilbert_probes;  /* CAND_HILBERT_PROBES */
    float lr_pos, lr_tau, lr_radius, lr_color, lr_dir, lr_aniso; /* LR_*_BASE */
    float lr_scale;                /* --lr */
    float init_log_tau, init_radius;  /* INIT_LOG_TAU, INIT_RADIUS */
    float init_gradient_alpha;     /* --init-gradient-alpha */
    float beta1, beta2, eps;       /* BETA1, BETA2, EPS */
    float ssim_weight;             /* --ssim-weight */
    int log_freq;                  /* --log-freq (0: no intermediate logs) */
    int use_graphs;                /* replay each iteration kind from a CUDA graph */
    int init_per_pixel;            /* --init-per-pixel: sites given one per pixel, candidates
                                      initialised per pixel (launchInitCandidates' flag) */
    int autotune;                  /* 1: pick the gradient kernel's tile-table shape rule by
                                      timing refresh windows during the fit; every rule gives
                                      the same sums, so the fit is unchanged.  0 (default):
                                      the fixed rule, which measured as fast or faster at
                                      256^2-1024^2.  No reference knob. */
} sad_train_config_t;

/* Fill with the reference's training_config.json values. */
void sad_train_config_default(sad_train_config_t* cfg);

typedef struct sad_trainer sad_trainer_t;

/* Allocates every buffer of a fit of a width x height image (one device allocation).
 * The bpp rule is applied here when target_bpp > 0. */
sad_status_t sad_trainer_create(const sad_train_config_t* cfg, int width, int height,
                                sad_trainer_t** out);
/* Device bytes of all buffers of such a fit (0 for an invalid configuration). */
size_t sad_trainer_memory_bytes(const sad_train_config_t* cfg, int width, int height);
/* As sad_trainer_create, with every buffer in caller-owned device memory of at least
 * sad_trainer_memory_bytes() bytes: no allocation.  The memory must stay valid, and be
 * ready (any stream-ordered allocation complete), until sad_trainer_destroy returns. */
sad_status_t sad_trainer_create_in(const sad_train_config_t* cfg, int width, int height,
                                   void* device_memory, size_t bytes, sad_trainer_t** out);
sad_status_t sad_trainer_destroy(sad_trainer_t* t);
sad_stream_t sad_trainer_stream(sad_trainer_t* t);

/* Target image [H,W,3] f32 and optional mask [H,W] (NULL = all ones), from device or
 * host memory (host variants copy on the trainer's stream). */
sad_status_t sad_trainer_set_target_device(sad_trainer_t* t, const float* target,
                                           const float* mask);
sad_status_t sad_trainer_set_target_host(sad_trainer_t* t, const float* target_host,
                                         const float* mask_host);

/* Initialise the sites: gradient-weighted (sites_host == NULL) or from host sites
 * [n,10]; resets Adam state, candidates (random + JFA seed) and the schedule. */
sad_status_t sad_trainer_init(sad_trainer_t* t, const float* sites_host, int n);

/* Run iterations [iter, end) of the schedule; end <= iterations. */
sad_status_t sad_trainer_run(sad_trainer_t* t, int end);

/* Render the current sites with the current candidate field; rgb_out (nullable) is a
 * device [H,W,3] f32 buffer that receives the image; psnr_out (nullable) receives the
 * PSNR against the target, 20 log10(1 / sqrt(mse)) over masked pixels (synchronises). */
sad_status_t sad_trainer_render(sad_trainer_t* t, float* rgb_out, float* psnr_out);

/* Copy the sites to host memory: all buffer slots (active_only = 0) or the active ones
 * in order.  Returns the number written in *written. Synchronises. */
sad_status_t sad_trainer_get_sites(sad_trainer_t* t, float* sites_host, int capacity,
                                   int active_only, int* written);

typedef struct {
    int width, height;
    int iteration;          /* next iteration to run */
    int site_buffer;        /* slots in use (actualNSites) */
    int active_estimate;    /* host-side estimate (activeSitesEstimate) */
    int capacity;
    float prune_percentile, densify_percentile; /* after the bpp rule */
    double gpu_ms_gradients; /* summed device time of the fused gradient kernel */
    int gradient_launches;
    uint64_t kernel_launches;
    int wide_far_refs;      /* tile-table shape rule in use: a tile is wide when more than
                               this many of its (pixel, candidate) references name far
                               entries (the autotuner's pick, or the fixed default) */
    int tune_rounds;        /* autotuner rounds completed in this fit */
} sad_trainer_info_t;
sad_status_t sad_trainer_info(sad_trainer_t* t, sad_trainer_info_t* info);
/* Time the fused gradient kernel with CUDA events on the trainer's stream. */
sad_status_t sad_trainer_enable_timing(sad_trainer_t* t, int enable);

/* One whole fit from host memory: copy target (and mask), init, run all iterations,
 * copy back the active sites (up to capacity) and the final PSNR. */
sad_status_t sad_trainer_fit_host(sad_trainer_t* t, const float* target_host,
                                  const float* mask_host, float* sites_host, int capacity,
                                  int* written, float* psnr_out);

/* ------------------------------------------------------------------------ */
/* batched fits: many images in lockstep, one launch per stage               */
/* ------------------------------------------------------------------------ */

/* A batch of n_images fits with one configuration (sizes may differ): each image owns a
 * trainer (reachable with sad_batch_trainer for its target, PSNR, render and sites), and
 * every iteration runs each stage as one launch over all images -- the per-pixel kernels
 * over a per-image tile work list, the per-site kernels over the images' compacted active
 * lists walked as one -- replayed as one CUDA graph per iteration kind.  Per image the
 * result is bitwise that of its own sad_trainer fit.  The schedule must be common: one VPT
 * pass per refresh, no SSIM loss, and no densify step firing (the default configuration);
 * sad_batch_init rejects others with SAD_ERR_UNSUPPORTED.  At most 1024 images.
 * No counterpart in the reference: it fits one image per process (run.sh batch mode,
 * run.sh:262-373). */
typedef struct sad_batch sad_batch_t;
sad_status_t sad_batch_create(const sad_train_config_t* cfg, int n_images, const int* widths,
                              const int* heights, sad_batch_t** out);
sad_status_t sad_batch_destroy(sad_batch_t* b);
/* The trainer of image i (owned by the batch): set its target before sad_batch_init. */
sad_status_t sad_batch_trainer(sad_batch_t* b, int image, sad_trainer_t** out);
/* Gradient-weighted init of every image and the batch's launch tables. */
sad_status_t sad_batch_init(sad_batch_t* b);
/* Iterations up to `end` (exclusive) of every image, on the batch's stream. */
sad_status_t sad_batch_run(sad_batch_t* b, int end);
sad_status_t sad_batch_synchronize(sad_batch_t* b);
sad_stream_t sad_batch_stream(sad_batch_t* b);
/* Event-time every batched gradient launch (eager launches while enabled) and report
 * the mean launch duration of the last sad_batch_run. */
sad_status_t sad_batch_enable_timing(sad_batch_t* b, int enable);
sad_status_t sad_batch_gradient_ms(sad_batch_t* b, double* ms_per_launch);

/* ------------------------------------------------------------------------ */
/* render from sites (serving path)                                          */
/* ------------------------------------------------------------------------ */

/* Build the candidate field (JFA rounds + VPT passes) for n sites and render it.
 * sites and out_rgb are device pointers; scratch is sad_render_scratch_bytes().
 * replaces: renderVoronoiFromSites, backends/cuda/src/sad_cuda.cu:1678-1858 */
typedef struct {
    int candidate_passes;   /* --render-cand-passes (16) */
    int use_jfa;            /* !--render-no-jfa */
    int jfa_rounds;         /* --render-jfa-rounds (1) */
    int cand_downscale;     /* --render-cand-downscale */
    float cand_radius_scale;
    uint32_t cand_radius_probes;
    uint32_t cand_inject_count;
    uint32_t cand_hilbert_window;
    uint32_t cand_hilbert_probes;
} sad_render_config_t;
void sad_render_config_default(sad_render_config_t* cfg);
size_t sad_render_scratch_bytes(uint32_t site_count, int width, int height, int cand_downscale);
sad_status_t sad_render_from_sites(const sad_render_config_t* cfg, const float* sites,
                                   uint32_t site_count, int width, int height, float* out_rgb,
                                   void* scratch, size_t scratch_bytes, sad_stream_t stream);
/* As sad_render_from_sites, then waits for it and reports the device time of the
 * candidate build (JFA rounds and VPT passes, after the per-site preparation and the
 * Hilbert order, as the reference times it) and of the render (CUDA events on the
 * stream): the two numbers of the reference's "Candidate build: X ms | Render: Y ms"
 * line (sad_cuda.cu:1760-1836). */
sad_status_t sad_render_from_sites_timed(const sad_render_config_t* cfg, const float* sites,
                                         uint32_t site_count, int width, int height, float* out_rgb,
                                         void* scratch, size_t scratch_bytes, sad_stream_t stream,
                                         float* cand_ms, float* render_ms);

/* ------------------------------------------------------------------------ */
/* 16-byte quantised inference sites (the Metal backend's serving format)     */
/* ------------------------------------------------------------------------ */

/* One packed site is four u32 words:
 *   w0  x as unorm15 of [0, W-1] | y as unorm15 of [0, H-1] << 15 | inactive << 30
 *   w1  r unorm11 | g unorm11 << 11 | b unorm10 << 22, over the ranges below
 *   w2  log_tau unorm16 | radius unorm16 << 16, over the ranges below
 *   w3  direction angle atan2(dy, dx) as unorm16 of [-pi, pi] | log_aniso as f16 << 16
 * Ranges (min, scale = max(max - min, 1e-6)) are over the active sites' finite values.
 * format: backends/metal/sources/utils/packed_inference.swift:3-18, 164-196 */
typedef struct {
    float log_tau_min, log_tau_scale;
    float radius_min, radius_scale;
    float r_min, r_scale;
    float g_min, g_scale;
    float b_min, b_scale;
} sad_packed_quant_t;

/* Pack site_count sites ([n,10] f32, device) into packed ([n][4] u32, device); quant
 * (device) receives the ranges.  Inactive sites (x < 0 or y < 0) keep their slot with the
 * inactive bit set.  Sides above 32768 are rejected (15-bit positions).
 * replaces: makePackedInferenceSites, backends/metal/sources/utils/packed_inference.swift:86-199 */
sad_status_t sad_pack_inference_sites(const float* sites, uint32_t site_count, int width, int height,
                                      uint32_t* packed, sad_packed_quant_t* quant, sad_stream_t stream);

/* Decode packed sites (device) to [n,10] f32 (device); inactive sites come out at
 * position (-1, -1).
 * replaces: decodePackedSite, backends/metal/shaders/sad_common.metal:89-120 */
sad_status_t sad_unpack_inference_sites(const uint32_t* packed, const sad_packed_quant_t* quant,
                                        uint32_t site_count, int width, int height, float* sites,
                                        sad_stream_t stream);

/* Render packed sites over a given candidate field (same softmax-over-8 as sad_render).
 * replaces: renderVoronoiPacked, backends/metal/shaders/encoders/packed_render_encoder.metal:3-31 */
sad_status_t sad_render_packed(const uint32_t* cand0, const uint32_t* cand1, float* out_rgb,
                               const uint32_t* packed, const sad_packed_quant_t* quant,
                               float inv_scale_sq, uint32_t site_count, int width, int height,
                               int cand_width, int cand_height, sad_stream_t stream);

/* Build the candidate field from packed sites and render them (render mode with packed
 * sites); scratch is sad_render_packed_scratch_bytes().
 * replaces: renderPackedInference, backends/metal/sources/rendering/packed_renderer.swift:15-135 */
size_t sad_render_packed_scratch_bytes(uint32_t site_count, int width, int height, int cand_downscale);
sad_status_t sad_render_packed_from_sites(const sad_render_config_t* cfg, const uint32_t* packed,
                                          const sad_packed_quant_t* quant, uint32_t site_count,
                                          int width, int height, float* out_rgb, void* scratch,
                                          size_t scratch_bytes, sad_stream_t stream);

/* Pack the trainer's sites and render them with its current candidate field; rgb_out and
 * psnr_out as in sad_trainer_render.  quant_out (nullable, host) receives the ranges.
 * replaces: the --packed-psnr re-render, backends/metal/sources/training/training.swift:676-705 */
sad_status_t sad_trainer_render_packed(sad_trainer_t* t, float* rgb_out, float* psnr_out,
                                       sad_packed_quant_t* quant_out);

/* ------------------------------------------------------------------------ */
/* executor: many fits and renders in flight on one GPU                       */
/* ------------------------------------------------------------------------ */

/* Host worker threads, each with its own streams, take requests first in, first out
 * (a render may pass a fit that waits for a fit slot).
 * Every request runs in one slab from the device's stream-ordered memory pool; a request
 * waits while the slabs of running requests plus its own exceed hbm_budget_bytes
 * (0: no limit; a request larger than the budget runs alone).
 * No counterpart in the reference: it fits one image per process, and its run.sh batch
 * mode (run.sh:262-373) runs the CLI once per file. */
typedef struct {
    int workers;              /* default 8 */
    size_t hbm_budget_bytes;  /* default 0 */
    int max_running_fits;     /* default 0 (no cap): at most this many fits run at once;
                                 renders queued behind a waiting fit pass it */
} sad_executor_config_t;

typedef struct {
    sad_status_t status;
    int sites_written;  /* fit: active sites copied to sites_host */
    float psnr;         /* fit: final PSNR */
    double queue_ms;    /* submission to start */
    double run_ms;      /* start to results in host memory */
    char message[192];  /* error text when status != SAD_OK */
    int iteration;      /* fit session: iterations run so far */
} sad_request_result_t;

typedef struct sad_executor sad_executor_t;
void sad_executor_config_default(sad_executor_config_t* cfg);
sad_status_t sad_executor_create(const sad_executor_config_t* cfg, sad_executor_t** out);
/* Queue a whole fit (sad_trainer_fit_host semantics).  Host buffers must stay valid until
 * the request completes; result is written by then. */
sad_status_t sad_executor_submit_fit(sad_executor_t* ex, const sad_train_config_t* cfg,
                                     const float* target_host, const float* mask_host, int width,
                                     int height, float* sites_host, int capacity,
                                     sad_request_result_t* result, uint64_t* ticket);
/* Queue a render from host sites ([n,10] f32) into rgb_host ([H,W,3] f32). */
sad_status_t sad_executor_submit_render(sad_executor_t* ex, const sad_render_config_t* cfg,
                                        const float* sites_host, uint32_t site_count, int width,
                                        int height, float* rgb_host, sad_request_result_t* result,
                                        uint64_t* ticket);
/* Resident fit sessions: a fit whose trainer -- sites, Adam moments, candidate fields and
 * device counters -- stays on the device between requests.  open_fit queues the session's
 * start (its slab from the stream-ordered pool, the target uploaded, init; result->psnr is
 * the initial PSNR) and returns its id; the slab counts against the HBM budget until the
 * session is closed.  submit_continue queues `iterations` more iterations of the same fit
 * (stopping at the configuration's total), then copies its active sites (up to capacity)
 * and PSNR back and reports the iterations run so far in result->iteration.  A session's
 * requests run one at a time, in submission order, between other requests; a fit
 * continued in several requests gives the sites of one uninterrupted fit, bit for bit.
 * close_fit queues the session's end (its slab freed); later requests of it are refused.
 * Host buffers must stay valid until their request completes.
 * The reference's nearest behaviour restarts a fit from a sites file
 * (--init-from-sites, backends/cuda/src/sad_cuda.cu:790-792, 1908-1922), without its Adam
 * moments. */
sad_status_t sad_executor_open_fit(sad_executor_t* ex, const sad_train_config_t* cfg,
                                   const float* target_host, const float* mask_host, int width,
                                   int height, sad_request_result_t* result, uint64_t* session,
                                   uint64_t* ticket);
sad_status_t sad_executor_submit_continue(sad_executor_t* ex, uint64_t session, int iterations,
                                          float* sites_host, int capacity,
                                          sad_request_result_t* result, uint64_t* ticket);
sad_status_t sad_executor_close_fit(sad_executor_t* ex, uint64_t session,
                                    sad_request_result_t* result, uint64_t* ticket);
sad_status_t sad_executor_wait(sad_executor_t* ex, uint64_t ticket);
sad_status_t sad_executor_wait_all(sad_executor_t* ex);
/* Withdraw a queued request.  *cancelled = 1 when it had not started: it is removed, its
 * result has status SAD_ERR_CANCELLED and its host buffers are released at once;
 * *cancelled = 0 when it has started or finished (it then completes as submitted). */
sad_status_t sad_executor_cancel(sad_executor_t* ex, uint64_t ticket, int* cancelled);
/* Failure testing without a GPU fault: the next `count` slab allocations are refused on the
 * host, as if the memory pool were exhausted (SAD_ERR_OUT_OF_MEMORY on those requests; no
 * CUDA call is made for them).  The executor keeps serving the requests after them. */
sad_status_t sad_executor_inject_slab_failures(sad_executor_t* ex, int count);
/* Runs what is queued, then joins the workers. */
sad_status_t sad_executor_destroy(sad_executor_t* ex);

#ifdef __cplusplus
}
#endif
#endif /* SAD_GB300_H */
