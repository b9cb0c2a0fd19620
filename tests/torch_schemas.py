"""The 24 operator schemas of the reference extension's TORCH_LIBRARY(sad) block
(backends/pytorch/torch_ext/torch_binding.cpp:6-30), verbatim: the registered operators of
this library must carry exactly these signatures, so code written against the reference
extension runs unchanged."""

SCHEMAS = {
    "render_sad": "render_sad(Tensor cand0, Tensor cand1, Tensor sites, float inv_scale_sq, int width, int height) -> Tensor",
    "render_sad_padded": "render_sad_padded(Tensor cand0, Tensor cand1, Tensor sites, float inv_scale_sq, int width, int height, int cand_width, int cand_height) -> Tensor",
    "init_candidates": "init_candidates(int width, int height, int site_count, int seed) -> (Tensor, Tensor)",
    "vpt_pass": "vpt_pass(Tensor cand0, Tensor cand1, Tensor sites, float inv_scale_sq, int width, int height, int jump, int radius_probes, float radius_scale, int inject_count, int seed) -> (Tensor, Tensor)",
    "render_sad_backward": "render_sad_backward(Tensor cand0, Tensor cand1, Tensor sites, Tensor grad_output, float inv_scale_sq, int width, int height) -> Tensor",
    "clear_buffer": "clear_buffer(Tensor buffer, int count) -> Tensor",
    "pack_candidate_sites": "pack_candidate_sites(Tensor sites, Tensor packed, int site_count) -> Tensor",
    "update_candidates_compact": "update_candidates_compact(Tensor cand0_in, Tensor cand1_in, Tensor cand0_out, Tensor cand1_out, Tensor packed_sites, Tensor hilbert_order, Tensor hilbert_pos, float inv_scale_sq, int site_count, int step, int step_high, float radius_scale, int radius_probes, int inject_count, int hilbert_probes, int hilbert_window, int cand_downscale, int target_width, int target_height, int cand_width, int cand_height) -> Tensor",
    "jfa_clear": "jfa_clear(Tensor cand0, Tensor cand1, int cand_width, int cand_height) -> Tensor",
    "jfa_seed": "jfa_seed(Tensor cand0, Tensor sites, int site_count, int cand_downscale, int cand_width, int cand_height) -> Tensor",
    "jfa_flood": "jfa_flood(Tensor cand0_in, Tensor cand0_out, Tensor sites, float inv_scale_sq, int site_count, int step_size, int cand_downscale, int cand_width, int cand_height) -> Tensor",
    "compute_gradients_tiled": "compute_gradients_tiled(Tensor cand0, Tensor cand1, Tensor target, Tensor rendered, Tensor mask, Tensor sites, Tensor grad_pos_x, Tensor grad_pos_y, Tensor grad_log_tau, Tensor grad_radius, Tensor grad_color_r, Tensor grad_color_g, Tensor grad_color_b, Tensor grad_dir_x, Tensor grad_dir_y, Tensor grad_log_aniso, Tensor removal_delta, float inv_scale_sq, int site_count, int compute_removal, float ssim_weight, int cand_width, int cand_height) -> Tensor",
    "tau_diffuse": "tau_diffuse(Tensor cand0, Tensor cand1, Tensor sites, Tensor grad_raw, Tensor grad_in, Tensor grad_out, int site_count, float lambda, int cand_downscale, int cand_width, int cand_height) -> Tensor",
    "adam_update": "adam_update(Tensor sites, Tensor adam, Tensor grad_pos_x, Tensor grad_pos_y, Tensor grad_log_tau, Tensor grad_radius, Tensor grad_color_r, Tensor grad_color_g, Tensor grad_color_b, Tensor grad_dir_x, Tensor grad_dir_y, Tensor grad_log_aniso, float lr_pos, float lr_tau, float lr_radius, float lr_color, float lr_dir, float lr_aniso, float beta1, float beta2, float eps, int t, int width, int height) -> Tensor",
    "compute_site_stats_tiled": "compute_site_stats_tiled(Tensor cand0, Tensor cand1, Tensor target, Tensor mask, Tensor sites, Tensor mass, Tensor energy, Tensor err_w, Tensor err_wx, Tensor err_wy, Tensor err_wxx, Tensor err_wxy, Tensor err_wyy, float inv_scale_sq, int site_count, int cand_width, int cand_height) -> Tensor",
    "compute_densify_score_pairs": "compute_densify_score_pairs(Tensor sites, Tensor mass, Tensor energy, Tensor pairs, int site_count, float min_mass, float score_alpha, int pair_count) -> Tensor",
    "compute_prune_score_pairs": "compute_prune_score_pairs(Tensor sites, Tensor removal_delta, Tensor pairs, int site_count, float delta_norm, int pair_count) -> Tensor",
    "radix_sort_pairs": "radix_sort_pairs(Tensor pairs, int max_key_exclusive) -> Tensor",
    "write_split_indices": "write_split_indices(Tensor pairs, Tensor indices, int num_to_split) -> Tensor",
    "split_sites": "split_sites(Tensor sites, Tensor adam, Tensor split_indices, Tensor mass, Tensor err_w, Tensor err_wx, Tensor err_wy, Tensor err_wxx, Tensor err_wxy, Tensor err_wyy, int current_site_count, int num_to_split, Tensor target) -> Tensor",
    "prune_sites": "prune_sites(Tensor sites, Tensor indices, int count) -> Tensor",
    "build_hilbert_pairs": "build_hilbert_pairs(Tensor sites, Tensor pairs, int site_count, int padded_count, int width, int height, int bits) -> Tensor",
    "write_hilbert_order": "write_hilbert_order(Tensor pairs, Tensor order, Tensor pos, int site_count) -> Tensor",
    "init_gradient_weighted": "init_gradient_weighted(Tensor sites, Tensor target, Tensor mask, int site_count, float init_log_tau, float init_radius, float gradient_alpha) -> Tensor",
}
