// kernels.h -- internal launch functions shared by the C-ABI wrappers and the trainer.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <algorithm>

#include "common.cuh"

namespace sad {

// Batched launches (one grid over the blocks of every image of a batch) take their images
// by value: kernel parameters sit in the constant bank, so every block reads its image's
// parameters through the constant cache (block-uniform and read-only, so neither copied
// into shared memory nor aliased by the kernel's shared-memory stores and atomics).  One
// launch covers up to kBatchLaunchItems images; block_prefix[i] is image i's first block
// within the launch and block_prefix[n_items] the launch's block count.
constexpr uint32_t kBatchLaunchItems = 96;
template <class Item>
struct BatchArgs {
    uint32_t n_items;
    uint32_t block_prefix[kBatchLaunchItems + 1];
    Item items[kBatchLaunchItems];
    // the image of block b: the last item whose first block is <= b
    __device__ __forceinline__ uint32_t item_of(uint32_t b) const {
        uint32_t lo = 0, hi = n_items;  // block_prefix[lo] <= b < block_prefix[hi]
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (block_prefix[mid] <= b) lo = mid;
            else hi = mid;
        }
        return lo;
    }
};

// Calls launch(args, blocks) for each run of up to kBatchLaunchItems images of the host
// arrays items[n] and prefix[n + 1] (prefix[i]: image i's first block; prefix[0] = 0),
// skipping runs without blocks.  The arguments are built on the caller's stack (at most
// 22 KB, for the gradient kernel's items).
template <class Item, class Launch>
inline void for_each_batch_launch(const Item* items, const uint32_t* prefix, uint32_t n, Launch&& launch) {
    static_assert(sizeof(BatchArgs<Item>) <= 32000, "kernel parameters are limited to 32,764 bytes");
    BatchArgs<Item> a;
    for (uint32_t first = 0; first < n; first += kBatchLaunchItems) {
        const uint32_t k = std::min(n - first, kBatchLaunchItems);
        const uint32_t base = prefix[first], blocks = prefix[first + k] - base;
        if (blocks == 0) continue;
        a.n_items = k;
        for (uint32_t i = 0; i <= k; ++i) a.block_prefix[i] = prefix[first + i] - base;
        for (uint32_t i = 0; i < k; ++i) a.items[i] = items[first + i];
        launch(a, blocks);
    }
}

struct VptParams {
    const uint32_t* in0;
    const uint32_t* in1;
    uint32_t* out0;
    uint32_t* out1;
    uint32_t site_count;
    uint32_t step;       // packed (jump << 16) | index, used when state == nullptr
    uint32_t step_high;  // index >> 16
    float inv_scale_sq;
    float radius_scale;
    uint32_t radius_probes;
    uint32_t inject_count;
    const uint32_t* hilbert_order;
    const uint32_t* hilbert_pos;
    uint32_t hilbert_probes;
    uint32_t hilbert_window;
    int cand_downscale;
    int target_width, target_height;
    int width, height;  // candidate field
    // trainer mode: step taken from state->vpt_pass + pass_offset
    const DevState* state;
    uint32_t pass_offset;
    uint32_t pow2, stages;
};

// Batched VPT pass: one grid over the 32x8 blocks of every image (host arrays: items[n],
// block_prefix[n + 1], image i's first block; BatchArgs).
struct VptBatchItem {
    VptParams p;
    const SiteGeom* vgeom;
    int blocks_x;
};
void launch_vpt_batch(const VptBatchItem* items, const uint32_t* block_prefix, uint32_t n_items, cudaStream_t st);

// render.cu
void launch_prepare_sites(const Site* sites, SiteGeom* geom, SiteColor* color, uint32_t n,
                          cudaStream_t st);
void launch_render_raw(const uint32_t* c0, const uint32_t* c1, float* out, const Site* sites,
                       float inv_s2, uint32_t n, int w, int h, int cw, int ch, cudaStream_t st);
void launch_render_prepared(const uint32_t* c0, const uint32_t* c1, float* out,
                            const SiteGeom* geom, const SiteColor* color, float inv_s2,
                            uint32_t n, int w, int h, int cw, int ch, cudaStream_t st);
void launch_render_packed(const uint32_t* c0, const uint32_t* c1, float* out, const uint32_t* packed,
                          const float* quant, float inv_s2, uint32_t n, int w, int h, int cw, int ch,
                          cudaStream_t st);
void launch_pack_inference(const Site* sites, uint32_t n, int w, int h, float* quant, uint32_t* packed,
                           cudaStream_t st);
void launch_unpack_inference(const uint32_t* packed, const float* quant, uint32_t n, int w, int h, Site* sites,
                             cudaStream_t st);
void launch_init_candidates(uint32_t* c0, uint32_t* c1, uint32_t n, uint32_t seed, int per_pixel,
                            int w, int h, cudaStream_t st);
void launch_clear_candidates(uint32_t* c0, uint32_t* c1, int w, int h, cudaStream_t st);
void launch_render_backward_raw(const uint32_t* c0, const uint32_t* c1, const float* grad_rgb,
                                float* grad_sites, const Site* sites, float inv_s2, uint32_t n,
                                int w, int h, int cw, int ch, cudaStream_t st);

// candidates.cu
void launch_pack_sites(const Site* sites, uint16_t* packed, uint32_t n, cudaStream_t st);
void launch_pack_geom(const Site* sites, SiteGeom* out, uint32_t n, cudaStream_t st);
// the same for the sites of the compacted active list (state->n_alive of at most max_alive)
void launch_pack_geom_alive(const Site* sites, SiteGeom* out, const uint32_t* alive,
                            const DevState* state, uint32_t max_alive, cudaStream_t st);
void launch_vpt_packed(const VptParams& prm, const uint16_t* packed, cudaStream_t st);
void launch_vpt_geom(const VptParams& prm, const SiteGeom* geom, cudaStream_t st);
void launch_jfa_seed(uint32_t* cand0, const Site* sites, uint32_t n, int w, int h, int ds,
                     cudaStream_t st);
void launch_jfa_flood_raw(const uint32_t* in0, uint32_t* out0, const Site* sites, uint32_t n,
                          uint32_t step, float inv_s2, int w, int h, int ds, int tw, int th,
                          cudaStream_t st);
void launch_jfa_flood_geom(const uint32_t* in0, uint32_t* out0, const SiteGeom* geom, uint32_t n,
                           uint32_t step, float inv_s2, int w, int h, int ds, int tw, int th,
                           cudaStream_t st);
uint32_t host_jump_step_for_index(uint32_t idx, int w, int h);
void jump_schedule_constants(int w, int h, uint32_t* pow2, uint32_t* stages);

// gradients.cu
struct GradParams {
    const uint32_t* cand0;
    const uint32_t* cand1;
    const float* target;    // [H,W,3]
    const float* rendered;  // [H,W,3], read only when ssim_weight > 0
    const float* mask;      // [H,W] or nullptr
    float inv_scale_sq;
    uint32_t site_count;
    float ssim_weight;
    int width, height, cand_width, cand_height;
    // outputs: either 10 float SoA arrays (+ removal), accumulated, or the trainer's [N][12]
    // records of 64-bit fixed point (2^-32 units; slots 0-9 gradients, 10 removal delta)
    float* soa[10];
    float* removal;
    long long* fix12;
    float removal_fix_mul;  // fixed-point path: removal delta pre-scale (a power of two, may exceed 1)
    int compute_removal;
    // trainer: the candidate field's tile registration, computed once per field refresh
    // (nullptr: register keys inside the gradient kernel)
    const uint4* slot_map;     // [H*W] 8 x u16 tile-table index per candidate, 0xFFFF none
    const uint32_t* tile_keys;  // [tiles][kTileKeys] keys by table index
    const int* tile_count;      // [tiles] keys in use | kTileWideFlag for a wide word table
};
struct TileMap {
    uint4* slot_map;
    uint32_t* tile_keys;
    int* tile_count;
    const int* wide_far_refs;  // device word with the tile-table shape rule (nullptr: kWideFarRefs)
};
// Batched launches: one grid over the tiles of every image of a batch; tile_prefix[i] is
// image i's first block (tile_prefix[n_items] = total_tiles); host arrays, passed to the
// kernels as BatchArgs.
struct GradBatchItem {
    GradParams p;
    const SiteGeom* geom;
    const SiteColor* color;
    int tiles_x;
};
struct RegisterBatchItem {
    const uint32_t* c0;
    const uint32_t* c1;
    uint32_t n;
    int w, h, cw, ch;
    TileMap map;
    int tiles_x;
};
void launch_gradients_batch(const GradBatchItem* items, const uint32_t* tile_prefix, uint32_t n_items,
                            bool removal, bool ssim, cudaStream_t st);
void launch_register_tiles_batch(const RegisterBatchItem* items, const uint32_t* tile_prefix, uint32_t n_items,
                                 cudaStream_t st);
size_t tile_map_words(int w, int h);  // u32 words of one TileMap (slot map + keys + counts)
TileMap tile_map_at(uint32_t* base, int w, int h);
void launch_register_tiles(const uint32_t* c0, const uint32_t* c1, uint32_t n, int w, int h,
                           int cw, int ch, const TileMap& map, cudaStream_t st);
void launch_gradients_raw(const GradParams& p, const Site* sites, cudaStream_t st);
// Opts the >48 KB shared-memory variants in; call once per device before any capture.
cudaError_t prepare_gradient_kernels();
void launch_gradients_prepared(const GradParams& p, const SiteGeom* geom, const SiteColor* color,
                               cudaStream_t st);

// optim.cu
void launch_tau_diffuse_raw(const uint32_t* c0, const uint32_t* c1, const Site* sites,
                            const float* raw, const float* gin, float* gout, uint32_t n,
                            float lambda, int w, int h, int ds, cudaStream_t st);
// trainer form, first Jacobi pass over the compacted active list (alive, state->n_alive
// entries, at most max_alive): raw log-tau gradient from slot 2 of the fixed-point
// records; records each listed site's neighbour list nbr[n][8] and raw[n]
void launch_tau_first_pass(const uint32_t* c0, const uint32_t* c1, const SiteGeom* geom,
                           const long long* fix12, uint32_t* nbr, float* raw, const uint32_t* alive,
                           float* gout, uint32_t n, uint32_t max_alive, const DevState* state,
                           int iterations, int w, int h, int ds, cudaStream_t st);
// trainer form, middle passes from the recorded lists
void launch_tau_list_pass(const uint32_t* nbr, const float* raw, const uint32_t* alive,
                          const float* gin, float* gout, uint32_t max_alive, const DevState* state,
                          int iterations, cudaStream_t st);
struct AdamHyper {
    float lr_pos, lr_tau, lr_radius, lr_color, lr_dir, lr_aniso;
    float beta1, beta2, eps;
};
void launch_adam_soa(Site* sites, float* adam, const float* const g[10], const AdamHyper& hp,
                     uint32_t t, uint32_t n, int w, int h, cudaStream_t st);
// trainer form over the compacted active list: last tau pass (from tau_gin and the lists)
// fused with Adam on the fixed-point records (slots 0-9 consumed and zeroed), refreshing
// SiteGeom/SiteColor; t = state->iter + 1
void launch_adam_train(Site* sites, float* adam, long long* fix12, const uint32_t* nbr,
                       const float* raw, const uint32_t* alive, const float* tau_gin,
                       SiteGeom* geom, SiteColor* color, const AdamHyper& hp,
                       const DevState* state, int iterations, uint32_t max_alive, int w, int h,
                       cudaStream_t st);
// Batched per-site launches over the compacted active lists of every image of a batch,
// walked as one flat list: site_prefix[i] = sum of the n_alive of images < i (in device
// memory, written by launch_batch_site_prefix after each compaction); grid-stride, so the
// grid size is only a size hint.  items in device memory.
struct SiteBatchItem {
    Site* sites;
    SiteGeom* geom;
    SiteColor* color;
    SiteGeom* vgeom;
    float* adam;
    long long* grads;
    float* tau_a;
    float* tau_b;
    uint32_t* tau_nbr;
    float* tau_raw;
    uint32_t* alive;
    uint32_t* alive_blocks;
    DevState* state;
    const uint32_t* cand0[3];
    const uint32_t* cand1[3];
    uint32_t* pairs;
    const uint32_t* prune_k;
    uint32_t n;  // buffer site count
    int w, h, cw, ch, ds;
    float removal_inv_mul;  // 1 / the removal pre-scale of the gradient records
    float delta_norm;
};
void launch_batch_site_prefix(const SiteBatchItem* items, uint32_t n_items, uint32_t* site_prefix, cudaStream_t st);
void launch_tau_first_batch(const SiteBatchItem* items, const uint32_t* site_prefix, uint32_t n_items, int field,
                            int iterations, uint32_t grid_threads, cudaStream_t st);
// a_to_b: tau_a -> tau_b, else tau_b -> tau_a
void launch_tau_list_batch(const SiteBatchItem* items, const uint32_t* site_prefix, uint32_t n_items, bool a_to_b,
                           int iterations, uint32_t grid_threads, cudaStream_t st);
void launch_adam_batch(const SiteBatchItem* items, const uint32_t* site_prefix, uint32_t n_items,
                       const AdamHyper& hp, int iterations, uint32_t grid_threads, cudaStream_t st);
void launch_advance_state_batch(const SiteBatchItem* items, uint32_t n_items, uint32_t vpt_passes, float beta1,
                                float beta2, cudaStream_t st);
void launch_pack_geom_batch(const SiteBatchItem* items, const uint32_t* site_prefix, uint32_t n_items,
                            uint32_t grid_threads, cudaStream_t st);
void launch_prune_pairs_batch(const SiteBatchItem* items, const uint32_t* site_prefix, uint32_t n_items,
                              uint32_t grid_threads, cudaStream_t st);
void launch_prune_sorted_batch(const SiteBatchItem* items, uint32_t n_items, uint32_t max_k, cudaStream_t st);
// compaction of every image's [0, n) (max_blocks = the largest compact_blocks(n) of the batch)
void launch_compact_batch(const SiteBatchItem* items, uint32_t n_items, uint32_t max_blocks, cudaStream_t st);
void launch_clear_f32(float* buf, size_t count, cudaStream_t st);
// iteration counter, VPT pass counter and the next iteration's Adam bias corrections
void launch_reset_state(DevState* state, float beta1, float beta2, cudaStream_t st);
// Set the tile-table shape rule read by the next tile registrations.
void launch_set_wide_far_refs(DevState* state, int value, cudaStream_t st);
void launch_advance_state(DevState* state, uint32_t vpt_passes, float beta1, float beta2,
                          cudaStream_t st);

// sort.cu
size_t radix_sort_temp_bytes(uint32_t count);
void launch_radix_sort(uint32_t* pairs, uint32_t count, uint32_t max_key_exclusive, void* temp,
                       cudaStream_t st);
// The same sort of *dev_count pairs (at most max_count; temp sized for max_count), the
// count read on the device so a captured graph serves any count.
void launch_radix_sort_dev(uint32_t* pairs, uint32_t max_count, const uint32_t* dev_count,
                           uint32_t max_key_exclusive, void* temp, cudaStream_t st);
// exclusive scan of `count` words in place by one CTA; *total (nullable) = sum
void launch_scan_single(uint32_t* data, uint32_t count, uint32_t* total, cudaStream_t st);

// topology.cu
void launch_densify_pairs(const Site* sites, const float* mass, const float* energy,
                          uint32_t* pairs, uint32_t n, float min_mass, float alpha,
                          uint32_t pair_count, cudaStream_t st);
void launch_prune_pairs(const Site* sites, const float* removal, int removal_stride,
                        uint32_t* pairs, uint32_t n, float delta_norm, uint32_t pair_count,
                        cudaStream_t st);
// trainer form: removal delta from slots 10 (fixed point, pre-scaled by fix_mul) and 11
// (count of 1e6 sentinels) of the gradient records, both cleared
void launch_prune_pairs_fixed(const Site* sites, long long* fix12, float fix_mul, uint32_t* pairs,
                              uint32_t n, float delta_norm, uint32_t pair_count, cudaStream_t st);
void launch_write_indices(const uint32_t* pairs, uint32_t* idx, uint32_t k, cudaStream_t st);
void launch_prune_by_index(Site* sites, const uint32_t* idx, uint32_t k, cudaStream_t st);
// trainer form over the compacted active list (state->n_alive pairs, at most max_alive)
void launch_prune_pairs_alive(long long* fix12, float fix_mul, uint32_t* pairs, const uint32_t* alive,
                              const DevState* state, uint32_t max_alive, float delta_norm, cudaStream_t st);
// trainer form: prune the first prune_k[state->iter] entries of sorted pairs, also in the
// prepared and the VPT geometry
void launch_prune_sorted_train(Site* sites, SiteGeom* geom, SiteGeom* vgeom, const uint32_t* pairs,
                               const uint32_t* prune_k, const DevState* state, uint32_t max_k,
                               cudaStream_t st);
// stream compaction of the active set: alive = ascending active slots of [0, n) (prepared
// geometry px >= 0), *n_alive = their number; block_counts holds compact_blocks(n) words
uint32_t compact_blocks(uint32_t n);
void launch_compact_active(const SiteGeom* geom, uint32_t n, uint32_t* block_counts, uint32_t* alive,
                           uint32_t* n_alive, cudaStream_t st);
void launch_split(Site* sites, float* adam, const uint32_t* split_idx, uint32_t num,
                  const float* const stats[7], uint32_t cur, const float* target, int w, int h,
                  cudaStream_t st);
void launch_site_stats(const uint32_t* c0, const uint32_t* c1, const float* target,
                       const float* mask, const Site* sites, float inv_s2, uint32_t n,
                       float* const out[8], int w, int h, int cw, int ch, cudaStream_t st);
// trainer form: 64-bit fixed-point accumulation into fix ([8][stride], zero on entry, left
// zeroed), converted into out[k][0..n) -- bitwise reproducible
void launch_site_stats_fixed(const uint32_t* c0, const uint32_t* c1, const float* target,
                             const float* mask, const Site* sites, float inv_s2, uint32_t n,
                             long long* fix, size_t stride, float* const out[8], int w, int h,
                             int cw, int ch, cudaStream_t st);
// pre-scale of the removal delta in the trainer's fixed-point gradient records
float removal_fix_mul(int w, int h);
void launch_hilbert_pairs(const Site* sites, uint32_t* pairs, uint32_t n, uint32_t padded, int w,
                          int h, int bits, cudaStream_t st);
void launch_hilbert_order(const uint32_t* pairs, uint32_t* order, uint32_t* pos, uint32_t n,
                          cudaStream_t st);
void launch_mse(const float* ren, const float* tgt, const float* mask, float* acc, int w, int h,
                cudaStream_t st);
// reproducible form: fixed-point (2^-24) sum into *acc
void launch_mse_fixed(const float* ren, const float* tgt, const float* mask, long long* acc, int w,
                      int h, cudaStream_t st);
void launch_ssim(const float* ren, const float* tgt, const float* mask, float* acc, int w, int h,
                 cudaStream_t st);
void launch_count_active(const Site* sites, uint32_t* count, uint32_t n, cudaStream_t st);
size_t init_temp_bytes(uint32_t n);
cudaError_t run_init_gradient_weighted(Site* sites, uint32_t n, const float* target,
                                       const float* mask, float thr, uint32_t max_attempts,
                                       float init_log_tau, float init_radius, int w, int h,
                                       void* temp, cudaStream_t st);

}  // namespace sad
