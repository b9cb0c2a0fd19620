// sad_torch_ops.cpp -- the reference's `torch.ops.sad` operators, registered from C++ on top
// of libsad_gb300's C ABI.
//
// Schemas: backends/pytorch/torch_ext/torch_binding.cpp:6-30, verbatim, so code written
// against the reference extension runs unchanged.  Argument checks and error texts follow
// backends/pytorch/torch_ext/cuda/sad_bindings.cu (each function cites its lines); every
// operator runs on the caller's current CUDA stream (the reference launches on the device
// default stream), so operators can be captured in CUDA graphs and ordered with other
// work.  No device code here: each operator is argument checks plus one or two C-ABI calls.
#include <ATen/ATen.h>
#include <c10/cuda/CUDAGuard.h>
#include <c10/cuda/CUDAStream.h>
#include <torch/library.h>

#include <algorithm>
#include <tuple>
#include <vector>

#include "sad_gb300.h"

namespace {

using at::Tensor;

void ok(sad_status_t s) { TORCH_CHECK(s == SAD_OK, sad_last_error()); }

sad_stream_t stream_of(const Tensor& t) {
    return reinterpret_cast<sad_stream_t>(c10::cuda::getCurrentCUDAStream(t.device().index()).stream());
}

void need_cuda(const Tensor& t, const char* name) {
    TORCH_CHECK(t.defined() && t.is_cuda(), name, " must be a CUDA tensor");
}

void need_type(const Tensor& t, at::ScalarType dt, const char* name) {
    const char* label = dt == at::kFloat ? "float32" : dt == at::kInt ? "int32" : "float16";
    TORCH_CHECK(t.scalar_type() == dt, name, " must be ", label);
}

void need(const Tensor& t, at::ScalarType dt, const char* name) {
    need_cuda(t, name);
    need_type(t, dt, name);
}

void need_cand(const Tensor& c, const char* name) {
    need(c, at::kInt, name);
    TORCH_CHECK(c.dim() == 2 && c.size(1) == 4, name, " must be [M,4]");
}

void need_sites(const Tensor& s, const char* name = "sites") {
    need(s, at::kFloat, name);
    TORCH_CHECK(s.dim() == 2 && s.size(1) == 10, name, " must be [N,10]");
}

template <class T = float>
T* ptr(const Tensor& t) {
    return reinterpret_cast<T*>(t.data_ptr());
}

uint32_t u32(int64_t v) { return static_cast<uint32_t>(v); }

// ---------------------------------------------------------------------------
// render / adjoint / candidates
// ---------------------------------------------------------------------------

// sad_bindings.cu:541-589 (renderVoronoiPadded)
Tensor render_sad_padded(const Tensor& cand0_, const Tensor& cand1_, const Tensor& sites_, double inv_scale_sq,
                         int64_t width, int64_t height, int64_t cand_width, int64_t cand_height) {
    need_cand(cand0_, "cand0");
    need_cand(cand1_, "cand1");
    need_sites(sites_);
    TORCH_CHECK(width > 0 && height > 0, "width/height must be positive");
    TORCH_CHECK(cand_width > 0 && cand_height > 0, "invalid cand size");
    TORCH_CHECK(cand0_.size(0) == cand_width * cand_height, "cand0 size must match cand_width*cand_height");
    TORCH_CHECK(cand1_.size(0) == cand_width * cand_height, "cand1 size must match cand_width*cand_height");
    c10::cuda::CUDAGuard guard(cand0_.device());
    Tensor cand0 = cand0_.contiguous(), cand1 = cand1_.contiguous(), sites = sites_.contiguous();
    Tensor out = at::empty({height, width, 3}, cand0.options().dtype(at::kFloat));
    ok(sad_render(ptr<uint32_t>(cand0), ptr<uint32_t>(cand1), ptr(out), ptr(sites), static_cast<float>(inv_scale_sq),
                  u32(sites.size(0)), static_cast<int>(width), static_cast<int>(height),
                  static_cast<int>(cand_width), static_cast<int>(cand_height), stream_of(cand0)));
    return out;
}

// sad_bindings.cu:496-538 (renderVoronoi)
Tensor render_sad(const Tensor& cand0, const Tensor& cand1, const Tensor& sites, double inv_scale_sq, int64_t width,
                  int64_t height) {
    need_cand(cand0, "cand0");
    need_cand(cand1, "cand1");
    TORCH_CHECK(width > 0 && height > 0, "width/height must be positive");
    TORCH_CHECK(cand0.size(0) == width * height, "cand0 size must match width*height");
    TORCH_CHECK(cand1.size(0) == width * height, "cand1 size must match width*height");
    return render_sad_padded(cand0, cand1, sites, inv_scale_sq, width, height, width, height);
}

// sad_bindings.cu:591-621; per-pixel neighbourhood mode when site_count == W*H
std::tuple<Tensor, Tensor> init_candidates(int64_t width, int64_t height, int64_t site_count, int64_t seed) {
    TORCH_CHECK(width > 0 && height > 0, "invalid cand size");
    TORCH_CHECK(site_count >= 0, "site_count must be non-negative");
    auto opts = at::TensorOptions().dtype(at::kInt).device(at::kCUDA, c10::cuda::current_device());
    Tensor cand0 = at::empty({width * height, 4}, opts);
    Tensor cand1 = at::empty_like(cand0);
    ok(sad_init_candidates(ptr<uint32_t>(cand0), ptr<uint32_t>(cand1), u32(site_count), u32(seed),
                           site_count == width * height ? 1 : 0, static_cast<int>(width), static_cast<int>(height),
                           stream_of(cand0)));
    return {cand0, cand1};
}

// sad_bindings.cu:623-696 (vptPass): packs the sites to f16 and runs one pass with
// step = jump << 16 and no Hilbert probes; `seed` is unused, as in the reference.
std::tuple<Tensor, Tensor> vpt_pass(const Tensor& cand0_, const Tensor& cand1_, const Tensor& sites_,
                                    double inv_scale_sq, int64_t width, int64_t height, int64_t jump,
                                    int64_t radius_probes, double radius_scale, int64_t inject_count, int64_t seed) {
    (void)seed;
    need_cand(cand0_, "cand0");
    need_cand(cand1_, "cand1");
    need_sites(sites_);
    TORCH_CHECK(cand0_.size(0) == width * height, "cand0 size must match width*height");
    TORCH_CHECK(cand1_.size(0) == width * height, "cand1 size must match width*height");
    c10::cuda::CUDAGuard guard(cand0_.device());
    Tensor cand0 = cand0_.contiguous(), cand1 = cand1_.contiguous(), sites = sites_.contiguous();
    Tensor out0 = at::empty_like(cand0), out1 = at::empty_like(cand1);
    Tensor packed = at::empty({sites.size(0), 8}, sites.options().dtype(at::kHalf));
    sad_stream_t s = stream_of(cand0);
    ok(sad_pack_candidate_sites(ptr(sites), ptr<uint16_t>(packed), u32(sites.size(0)), s));
    ok(sad_update_candidates(ptr<uint32_t>(cand0), ptr<uint32_t>(cand1), ptr<uint32_t>(out0), ptr<uint32_t>(out1),
                             ptr<uint16_t>(packed), u32(sites.size(0)), u32(jump << 16),
                             static_cast<float>(inv_scale_sq), 0u, static_cast<float>(radius_scale),
                             u32(radius_probes), u32(inject_count), nullptr, nullptr, 0u, 0u, 1,
                             static_cast<int>(width), static_cast<int>(height), static_cast<int>(width),
                             static_cast<int>(height), s));
    return {out0, out1};
}

// sad_bindings.cu:698-749 (renderVoronoiBackward): returns dL/dsites [N,10]
Tensor render_sad_backward(const Tensor& cand0_, const Tensor& cand1_, const Tensor& sites_,
                           const Tensor& grad_output_, double inv_scale_sq, int64_t width, int64_t height) {
    need_cand(cand0_, "cand0");
    need_cand(cand1_, "cand1");
    need_sites(sites_);
    need(grad_output_, at::kFloat, "grad_output");
    TORCH_CHECK(grad_output_.dim() == 3 && grad_output_.size(2) == 3, "grad_output must be [H,W,3]");
    TORCH_CHECK(grad_output_.size(0) == height && grad_output_.size(1) == width,
                "grad_output size must match height/width");
    TORCH_CHECK(cand0_.size(0) == width * height, "cand0 size must match width*height");
    TORCH_CHECK(cand1_.size(0) == width * height, "cand1 size must match width*height");
    c10::cuda::CUDAGuard guard(cand0_.device());
    Tensor cand0 = cand0_.contiguous(), cand1 = cand1_.contiguous();
    Tensor sites = sites_.contiguous(), grad_output = grad_output_.contiguous();
    Tensor grad_sites = at::zeros({sites.size(0), 10}, sites.options());
    ok(sad_render_backward(ptr<uint32_t>(cand0), ptr<uint32_t>(cand1), ptr(grad_output), ptr(grad_sites), ptr(sites),
                           static_cast<float>(inv_scale_sq), u32(sites.size(0)), static_cast<int>(width),
                           static_cast<int>(height), static_cast<int>(width), static_cast<int>(height),
                           stream_of(cand0)));
    return grad_sites;
}

// sad_bindings.cu:751-764
Tensor clear_buffer(const Tensor& buffer_, int64_t count) {
    need(buffer_, at::kFloat, "buffer");
    c10::cuda::CUDAGuard guard(buffer_.device());
    Tensor buffer = buffer_.contiguous();
    int64_t n = buffer.numel();
    if (count <= 0 || count > n) count = n;
    ok(sad_clear_buffer(ptr(buffer), u32(count), stream_of(buffer)));
    return buffer;
}

// sad_bindings.cu:766-784
Tensor pack_candidate_sites(const Tensor& sites_, const Tensor& packed_, int64_t site_count) {
    need_sites(sites_);
    need(packed_, at::kHalf, "packed");
    TORCH_CHECK(packed_.dim() == 2 && packed_.size(1) == 8, "packed must be [N,8]");
    c10::cuda::CUDAGuard guard(sites_.device());
    Tensor sites = sites_.contiguous(), packed = packed_.contiguous();
    if (site_count <= 0) site_count = sites.size(0);
    TORCH_CHECK(site_count <= sites.size(0) && site_count <= packed.size(0), "site_count exceeds buffers");
    ok(sad_pack_candidate_sites(ptr(sites), ptr<uint16_t>(packed), u32(site_count), stream_of(sites)));
    return packed;
}

// sad_bindings.cu:786-863
Tensor update_candidates_compact(const Tensor& cand0_in_, const Tensor& cand1_in_, const Tensor& cand0_out_,
                                 const Tensor& cand1_out_, const Tensor& packed_sites_, const Tensor& hilbert_order,
                                 const Tensor& hilbert_pos, double inv_scale_sq, int64_t site_count, int64_t step,
                                 int64_t step_high, double radius_scale, int64_t radius_probes, int64_t inject_count,
                                 int64_t hilbert_probes, int64_t hilbert_window, int64_t cand_downscale,
                                 int64_t target_width, int64_t target_height, int64_t cand_width,
                                 int64_t cand_height) {
    const std::pair<const Tensor*, const char*> cands[] = {
        {&cand0_in_, "cand0_in"}, {&cand1_in_, "cand1_in"}, {&cand0_out_, "cand0_out"}, {&cand1_out_, "cand1_out"}};
    for (const auto& c : cands) {
        need_cand(*c.first, c.second);
        TORCH_CHECK(c.first->size(0) == cand_width * cand_height, c.second, " size mismatch");
    }
    need(packed_sites_, at::kHalf, "packed_sites");
    TORCH_CHECK(packed_sites_.dim() == 2 && packed_sites_.size(1) == 8, "packed_sites must be [N,8]");
    c10::cuda::CUDAGuard guard(cand0_in_.device());
    Tensor cand0_in = cand0_in_.contiguous(), cand1_in = cand1_in_.contiguous();
    Tensor cand0_out = cand0_out_.contiguous(), cand1_out = cand1_out_.contiguous();
    Tensor packed_sites = packed_sites_.contiguous();
    if (site_count <= 0) site_count = packed_sites.size(0);
    Tensor ho, hp;
    const uint32_t* hop = nullptr;
    const uint32_t* hpp = nullptr;
    if (hilbert_probes > 0 && hilbert_window > 0) {
        need(hilbert_order, at::kInt, "hilbert_order");
        need(hilbert_pos, at::kInt, "hilbert_pos");
        ho = hilbert_order.contiguous();
        hp = hilbert_pos.contiguous();
        hop = ptr<uint32_t>(ho);
        hpp = ptr<uint32_t>(hp);
    }
    ok(sad_update_candidates(ptr<uint32_t>(cand0_in), ptr<uint32_t>(cand1_in), ptr<uint32_t>(cand0_out),
                             ptr<uint32_t>(cand1_out), ptr<uint16_t>(packed_sites), u32(site_count), u32(step),
                             static_cast<float>(inv_scale_sq), u32(step_high), static_cast<float>(radius_scale),
                             u32(radius_probes), u32(inject_count), hop, hpp, u32(hilbert_probes),
                             u32(hilbert_window), static_cast<int>(cand_downscale), static_cast<int>(target_width),
                             static_cast<int>(target_height), static_cast<int>(cand_width),
                             static_cast<int>(cand_height), stream_of(cand0_in)));
    return cand0_out;
}

// sad_bindings.cu:865-881
Tensor jfa_clear(const Tensor& cand0_, const Tensor& cand1_, int64_t cand_width, int64_t cand_height) {
    need_cand(cand0_, "cand0");
    need_cand(cand1_, "cand1");
    c10::cuda::CUDAGuard guard(cand0_.device());
    Tensor cand0 = cand0_.contiguous(), cand1 = cand1_.contiguous();
    TORCH_CHECK(cand0.size(0) >= cand_width * cand_height && cand1.size(0) >= cand_width * cand_height,
                "cand size must cover cand_width*cand_height");
    ok(sad_clear_candidates(ptr<uint32_t>(cand0), ptr<uint32_t>(cand1), static_cast<int>(cand_width),
                            static_cast<int>(cand_height), stream_of(cand0)));
    return cand0;
}

// sad_bindings.cu:883-906 (lowest site id wins a shared texel)
Tensor jfa_seed(const Tensor& cand0_, const Tensor& sites_, int64_t site_count, int64_t cand_downscale,
                int64_t cand_width, int64_t cand_height) {
    need_cand(cand0_, "cand0");
    need_sites(sites_);
    TORCH_CHECK(cand0_.size(0) == cand_width * cand_height, "cand0 size must match cand_width*cand_height");
    c10::cuda::CUDAGuard guard(cand0_.device());
    Tensor cand0 = cand0_.contiguous(), sites = sites_.contiguous();
    if (site_count <= 0) site_count = sites.size(0);
    ok(sad_jfa_seed(ptr<uint32_t>(cand0), ptr(sites), u32(site_count), static_cast<int>(cand_width),
                    static_cast<int>(cand_height), static_cast<int>(cand_downscale), stream_of(cand0)));
    return cand0;
}

// sad_bindings.cu:908-942
Tensor jfa_flood(const Tensor& cand0_in_, const Tensor& cand0_out_, const Tensor& sites_, double inv_scale_sq,
                 int64_t site_count, int64_t step_size, int64_t cand_downscale, int64_t cand_width,
                 int64_t cand_height) {
    need_cand(cand0_in_, "cand0_in");
    need_cand(cand0_out_, "cand0_out");
    need_sites(sites_);
    TORCH_CHECK(cand0_in_.size(0) == cand_width * cand_height, "cand0_in size must match cand_width*cand_height");
    TORCH_CHECK(cand0_out_.size(0) == cand_width * cand_height, "cand0_out size must match cand_width*cand_height");
    c10::cuda::CUDAGuard guard(cand0_in_.device());
    Tensor cand0_in = cand0_in_.contiguous(), cand0_out = cand0_out_.contiguous(), sites = sites_.contiguous();
    if (site_count <= 0) site_count = sites.size(0);
    ok(sad_jfa_flood(ptr<uint32_t>(cand0_in), ptr<uint32_t>(cand0_out), ptr(sites), u32(site_count), u32(step_size),
                     static_cast<float>(inv_scale_sq), static_cast<int>(cand_width), static_cast<int>(cand_height),
                     static_cast<int>(cand_downscale), static_cast<int>(cand_width * cand_downscale),
                     static_cast<int>(cand_height * cand_downscale), stream_of(cand0_in)));
    return cand0_out;
}

// ---------------------------------------------------------------------------
// training operators
// ---------------------------------------------------------------------------

void need_target(const Tensor& target, const Tensor& mask) {
    TORCH_CHECK(target.dim() == 3 && target.size(2) == 3, "target must be [H,W,3]");
    TORCH_CHECK(mask.dim() == 2, "mask must be [H,W]");
    TORCH_CHECK(mask.size(0) == target.size(0) && mask.size(1) == target.size(1), "mask size must match target");
}

// sad_bindings.cu:944-1013 (grads and removal are accumulated)
Tensor compute_gradients_tiled(const Tensor& cand0_, const Tensor& cand1_, const Tensor& target_,
                               const Tensor& rendered_, const Tensor& mask_, const Tensor& sites_,
                               const Tensor& grad_pos_x, const Tensor& grad_pos_y, const Tensor& grad_log_tau,
                               const Tensor& grad_radius, const Tensor& grad_color_r, const Tensor& grad_color_g,
                               const Tensor& grad_color_b, const Tensor& grad_dir_x, const Tensor& grad_dir_y,
                               const Tensor& grad_log_aniso, const Tensor& removal_delta, double inv_scale_sq,
                               int64_t site_count, int64_t compute_removal, double ssim_weight, int64_t cand_width,
                               int64_t cand_height) {
    need(cand0_, at::kInt, "cand0");
    need(cand1_, at::kInt, "cand1");
    need(target_, at::kFloat, "target");
    need(rendered_, at::kFloat, "rendered");
    need(mask_, at::kFloat, "mask");
    need(sites_, at::kFloat, "sites");
    TORCH_CHECK(target_.dim() == 3 && target_.size(2) == 3, "target must be [H,W,3]");
    TORCH_CHECK(rendered_.dim() == 3 && rendered_.size(2) == 3, "rendered must be [H,W,3]");
    need_target(target_, mask_);
    TORCH_CHECK(sites_.dim() == 2 && sites_.size(1) == 10, "sites must be [N,10]");
    const Tensor* grads[] = {&grad_pos_x, &grad_pos_y, &grad_log_tau, &grad_radius, &grad_color_r,
                             &grad_color_g, &grad_color_b, &grad_dir_x, &grad_dir_y, &grad_log_aniso, &removal_delta};
    for (const Tensor* g : grads) {
        need(*g, at::kFloat, "gradient buffer");
        TORCH_CHECK(g->is_contiguous(), "gradient buffers must be contiguous");
    }
    c10::cuda::CUDAGuard guard(cand0_.device());
    Tensor cand0 = cand0_.contiguous(), cand1 = cand1_.contiguous(), target = target_.contiguous();
    Tensor rendered = rendered_.contiguous(), mask = mask_.contiguous(), sites = sites_.contiguous();
    if (site_count <= 0) site_count = sites.size(0);
    ok(sad_compute_gradients_tiled(
        ptr<uint32_t>(cand0), ptr<uint32_t>(cand1), ptr(target), ptr(rendered), ptr(mask), ptr(grad_pos_x),
        ptr(grad_pos_y), ptr(grad_log_tau), ptr(grad_radius), ptr(grad_color_r), ptr(grad_color_g),
        ptr(grad_color_b), ptr(grad_dir_x), ptr(grad_dir_y), ptr(grad_log_aniso), ptr(sites),
        static_cast<float>(inv_scale_sq), u32(site_count), ptr(removal_delta), u32(compute_removal),
        static_cast<float>(ssim_weight), static_cast<int>(target.size(1)), static_cast<int>(target.size(0)),
        static_cast<int>(cand_width), static_cast<int>(cand_height), stream_of(cand0)));
    return grad_pos_x;
}

// sad_bindings.cu:1015-1057
Tensor tau_diffuse(const Tensor& cand0_, const Tensor& cand1_, const Tensor& sites_, const Tensor& grad_raw_,
                   const Tensor& grad_in_, const Tensor& grad_out_, int64_t site_count, double lambda,
                   int64_t cand_downscale, int64_t cand_width, int64_t cand_height) {
    need(cand0_, at::kInt, "cand0");
    need(cand1_, at::kInt, "cand1");
    need_sites(sites_);
    need(grad_raw_, at::kFloat, "grad_raw");
    need(grad_in_, at::kFloat, "grad_in");
    need(grad_out_, at::kFloat, "grad_out");
    c10::cuda::CUDAGuard guard(cand0_.device());
    Tensor cand0 = cand0_.contiguous(), cand1 = cand1_.contiguous(), sites = sites_.contiguous();
    Tensor grad_raw = grad_raw_.contiguous(), grad_in = grad_in_.contiguous(), grad_out = grad_out_.contiguous();
    if (site_count <= 0) site_count = sites.size(0);
    ok(sad_tau_diffuse(ptr<uint32_t>(cand0), ptr<uint32_t>(cand1), ptr(sites), ptr(grad_raw), ptr(grad_in),
                       ptr(grad_out), u32(site_count), static_cast<float>(lambda), static_cast<int>(cand_width),
                       static_cast<int>(cand_height), static_cast<int>(cand_downscale), stream_of(cand0)));
    return grad_out;
}

// sad_bindings.cu:1059-1104 (every site of the tensor is stepped)
Tensor adam_update(const Tensor& sites_, const Tensor& adam_, const Tensor& grad_pos_x, const Tensor& grad_pos_y,
                   const Tensor& grad_log_tau, const Tensor& grad_radius, const Tensor& grad_color_r,
                   const Tensor& grad_color_g, const Tensor& grad_color_b, const Tensor& grad_dir_x,
                   const Tensor& grad_dir_y, const Tensor& grad_log_aniso, double lr_pos, double lr_tau,
                   double lr_radius, double lr_color, double lr_dir, double lr_aniso, double beta1, double beta2,
                   double eps, int64_t t, int64_t width, int64_t height) {
    need_sites(sites_);
    need(adam_, at::kFloat, "adam");
    TORCH_CHECK(adam_.dim() == 2 && adam_.size(1) == 20, "adam must be [N,20]");
    TORCH_CHECK(adam_.size(0) >= sites_.size(0), "adam must have a row per site");
    const Tensor* in[] = {&grad_pos_x, &grad_pos_y, &grad_log_tau, &grad_radius, &grad_color_r,
                          &grad_color_g, &grad_color_b, &grad_dir_x, &grad_dir_y, &grad_log_aniso};
    for (const Tensor* g : in) {
        need(*g, at::kFloat, "gradient buffer");
        TORCH_CHECK(g->numel() >= sites_.size(0), "gradient buffers must cover every site");
    }
    c10::cuda::CUDAGuard guard(sites_.device());
    Tensor sites = sites_.contiguous(), adam = adam_.contiguous();
    std::vector<Tensor> g;
    for (const Tensor* x : in) g.push_back(x->contiguous());
    ok(sad_adam_update(ptr(sites), ptr(adam), ptr(g[0]), ptr(g[1]), ptr(g[2]), ptr(g[3]), ptr(g[4]), ptr(g[5]),
                       ptr(g[6]), ptr(g[7]), ptr(g[8]), ptr(g[9]), static_cast<float>(lr_pos),
                       static_cast<float>(lr_tau), static_cast<float>(lr_radius), static_cast<float>(lr_color),
                       static_cast<float>(lr_dir), static_cast<float>(lr_aniso), static_cast<float>(beta1),
                       static_cast<float>(beta2), static_cast<float>(eps), u32(t), u32(sites.size(0)),
                       static_cast<int>(width), static_cast<int>(height), stream_of(sites)));
    return sites;
}

// sad_bindings.cu:1106-1161 (the 8 arrays are zeroed for site_count first, as
// launchComputeSiteStatsSimple does)
Tensor compute_site_stats_tiled(const Tensor& cand0_, const Tensor& cand1_, const Tensor& target_,
                                const Tensor& mask_, const Tensor& sites_, const Tensor& mass, const Tensor& energy,
                                const Tensor& err_w, const Tensor& err_wx, const Tensor& err_wy,
                                const Tensor& err_wxx, const Tensor& err_wxy, const Tensor& err_wyy,
                                double inv_scale_sq, int64_t site_count, int64_t cand_width, int64_t cand_height) {
    need(cand0_, at::kInt, "cand0");
    need(cand1_, at::kInt, "cand1");
    need(target_, at::kFloat, "target");
    need(mask_, at::kFloat, "mask");
    need(sites_, at::kFloat, "sites");
    need_target(target_, mask_);
    TORCH_CHECK(sites_.dim() == 2 && sites_.size(1) == 10, "sites must be [N,10]");
    const Tensor* outs[] = {&mass, &energy, &err_w, &err_wx, &err_wy, &err_wxx, &err_wxy, &err_wyy};
    for (const Tensor* o : outs) {
        need(*o, at::kFloat, "stat buffer");
        TORCH_CHECK(o->is_contiguous(), "stat buffers must be contiguous");
    }
    c10::cuda::CUDAGuard guard(cand0_.device());
    Tensor cand0 = cand0_.contiguous(), cand1 = cand1_.contiguous(), target = target_.contiguous();
    Tensor mask = mask_.contiguous(), sites = sites_.contiguous();
    if (site_count <= 0) site_count = sites.size(0);
    sad_stream_t s = stream_of(cand0);
    for (const Tensor* o : outs) ok(sad_clear_buffer(ptr(*o), u32(site_count), s));
    ok(sad_compute_site_stats(ptr<uint32_t>(cand0), ptr<uint32_t>(cand1), ptr(target), ptr(mask), ptr(sites),
                              static_cast<float>(inv_scale_sq), u32(site_count), ptr(mass), ptr(energy), ptr(err_w),
                              ptr(err_wx), ptr(err_wy), ptr(err_wxx), ptr(err_wxy), ptr(err_wyy),
                              static_cast<int>(target.size(1)), static_cast<int>(target.size(0)),
                              static_cast<int>(cand_width), static_cast<int>(cand_height), s));
    return mass;
}

void need_pairs(const Tensor& pairs, const char* shape_msg) {
    need(pairs, at::kInt, "pairs");
    TORCH_CHECK(pairs.dim() == 2 && pairs.size(1) == 2, shape_msg);
}

// sad_bindings.cu:1163-1198
Tensor compute_densify_score_pairs(const Tensor& sites_, const Tensor& mass_, const Tensor& energy_,
                                   const Tensor& pairs_, int64_t site_count, double min_mass, double score_alpha,
                                   int64_t pair_count) {
    need_sites(sites_);
    need(mass_, at::kFloat, "mass");
    need(energy_, at::kFloat, "energy");
    need_pairs(pairs_, "pairs must be [M,2]");
    c10::cuda::CUDAGuard guard(sites_.device());
    Tensor sites = sites_.contiguous(), mass = mass_.contiguous(), energy = energy_.contiguous();
    Tensor pairs = pairs_.contiguous();
    if (site_count <= 0) site_count = sites.size(0);
    if (pair_count <= 0) pair_count = pairs.size(0);
    ok(sad_compute_densify_score_pairs(ptr(sites), ptr(mass), ptr(energy), ptr<uint32_t>(pairs), u32(site_count),
                                       static_cast<float>(min_mass), static_cast<float>(score_alpha),
                                       u32(pair_count), stream_of(sites)));
    return pairs;
}

// sad_bindings.cu:1200-1229
Tensor compute_prune_score_pairs(const Tensor& sites_, const Tensor& removal_delta_, const Tensor& pairs_,
                                 int64_t site_count, double delta_norm, int64_t pair_count) {
    need_sites(sites_);
    need(removal_delta_, at::kFloat, "removal_delta");
    need_pairs(pairs_, "pairs must be [M,2]");
    c10::cuda::CUDAGuard guard(sites_.device());
    Tensor sites = sites_.contiguous(), removal = removal_delta_.contiguous(), pairs = pairs_.contiguous();
    if (site_count <= 0) site_count = sites.size(0);
    if (pair_count <= 0) pair_count = pairs.size(0);
    ok(sad_compute_prune_score_pairs(ptr(sites), ptr(removal), ptr<uint32_t>(pairs), u32(site_count),
                                     static_cast<float>(delta_norm), u32(pair_count), stream_of(sites)));
    return pairs;
}

// sad_bindings.cu:1231-1264
Tensor radix_sort_pairs(const Tensor& pairs_, int64_t max_key_exclusive) {
    need_pairs(pairs_, "pairs must be [N,2]");
    c10::cuda::CUDAGuard guard(pairs_.device());
    Tensor pairs = pairs_.contiguous();
    int64_t count = pairs.size(0);
    TORCH_CHECK(count > 0, "pairs must be non-empty");
    size_t nbytes = sad_radix_sort_temp_bytes(u32(count));
    Tensor temp = at::empty({static_cast<int64_t>((nbytes + 15) / 16 * 16)}, pairs.options().dtype(at::kByte));
    ok(sad_radix_sort_pairs(ptr<uint32_t>(pairs), u32(count), u32(max_key_exclusive), temp.data_ptr(),
                            static_cast<size_t>(temp.numel()), stream_of(pairs)));
    return pairs;
}

// sad_bindings.cu:1266-1282
Tensor write_split_indices(const Tensor& pairs_, const Tensor& indices_, int64_t num_to_split) {
    need(pairs_, at::kInt, "pairs");
    need(indices_, at::kInt, "indices");
    TORCH_CHECK(pairs_.dim() == 2 && pairs_.size(1) == 2, "pairs must be [N,2]");
    TORCH_CHECK(indices_.dim() == 1, "indices must be [K]");
    TORCH_CHECK(num_to_split <= indices_.size(0) && num_to_split <= pairs_.size(0), "num_to_split exceeds buffers");
    c10::cuda::CUDAGuard guard(pairs_.device());
    Tensor pairs = pairs_.contiguous(), indices = indices_.contiguous();
    ok(sad_write_split_indices(ptr<uint32_t>(pairs), ptr<uint32_t>(indices), u32(std::max<int64_t>(0, num_to_split)),
                               stream_of(pairs)));
    return indices;
}

// sad_bindings.cu:1284-1322
Tensor split_sites(const Tensor& sites_, const Tensor& adam_, const Tensor& split_indices_, const Tensor& mass,
                   const Tensor& err_w, const Tensor& err_wx, const Tensor& err_wy, const Tensor& err_wxx,
                   const Tensor& err_wxy, const Tensor& err_wyy, int64_t current_site_count, int64_t num_to_split,
                   const Tensor& target_) {
    need_sites(sites_);
    need(adam_, at::kFloat, "adam");
    TORCH_CHECK(adam_.dim() == 2 && adam_.size(1) == 20, "adam must be [N,20]");
    need(split_indices_, at::kInt, "split_indices");
    need(target_, at::kFloat, "target");
    TORCH_CHECK(target_.dim() == 3 && target_.size(2) == 3, "target must be [H,W,3]");
    TORCH_CHECK(current_site_count + num_to_split <= sites_.size(0), "split children exceed the site buffer");
    c10::cuda::CUDAGuard guard(sites_.device());
    Tensor sites = sites_.contiguous(), adam = adam_.contiguous();
    Tensor split_indices = split_indices_.contiguous(), target = target_.contiguous();
    std::vector<Tensor> st;
    for (const Tensor* x : {&mass, &err_w, &err_wx, &err_wy, &err_wxx, &err_wxy, &err_wyy}) st.push_back(x->contiguous());
    ok(sad_split_sites(ptr(sites), ptr(adam), ptr<uint32_t>(split_indices), u32(num_to_split), ptr(st[0]), ptr(st[1]),
                       ptr(st[2]), ptr(st[3]), ptr(st[4]), ptr(st[5]), ptr(st[6]), u32(current_site_count),
                       ptr(target), static_cast<int>(target.size(1)), static_cast<int>(target.size(0)),
                       stream_of(sites)));
    return sites;
}

// sad_bindings.cu:1324-1339
Tensor prune_sites(const Tensor& sites_, const Tensor& indices_, int64_t count) {
    need_sites(sites_);
    need(indices_, at::kInt, "indices");
    TORCH_CHECK(count <= indices_.numel(), "count exceeds indices");
    c10::cuda::CUDAGuard guard(sites_.device());
    Tensor sites = sites_.contiguous(), indices = indices_.contiguous();
    ok(sad_prune_sites(ptr(sites), ptr<uint32_t>(indices), u32(std::max<int64_t>(0, count)), stream_of(sites)));
    return sites;
}

// sad_bindings.cu:1341-1372
Tensor build_hilbert_pairs(const Tensor& sites_, const Tensor& pairs_, int64_t site_count, int64_t padded_count,
                           int64_t width, int64_t height, int64_t bits) {
    need_sites(sites_);
    need_pairs(pairs_, "pairs must be [M,2]");
    c10::cuda::CUDAGuard guard(sites_.device());
    Tensor sites = sites_.contiguous(), pairs = pairs_.contiguous();
    if (site_count <= 0) site_count = sites.size(0);
    if (padded_count <= 0)
        padded_count = pairs.size(0);
    else
        TORCH_CHECK(pairs.size(0) == padded_count, "pairs size must match padded_count");
    ok(sad_hilbert_pairs(ptr(sites), ptr<uint32_t>(pairs), u32(site_count), u32(padded_count), static_cast<int>(width),
                         static_cast<int>(height), static_cast<int>(bits), stream_of(sites)));
    return pairs;
}

// sad_bindings.cu:1374-1397
Tensor write_hilbert_order(const Tensor& pairs_, const Tensor& order_, const Tensor& pos_, int64_t site_count) {
    need(pairs_, at::kInt, "pairs");
    need(order_, at::kInt, "order");
    need(pos_, at::kInt, "pos");
    TORCH_CHECK(pairs_.dim() == 2 && pairs_.size(1) == 2, "pairs must be [N,2]");
    c10::cuda::CUDAGuard guard(pairs_.device());
    Tensor pairs = pairs_.contiguous(), order = order_.contiguous(), pos = pos_.contiguous();
    if (site_count <= 0) site_count = order.size(0);
    ok(sad_write_hilbert_order(ptr<uint32_t>(pairs), ptr<uint32_t>(order), ptr<uint32_t>(pos), u32(site_count),
                               stream_of(pairs)));
    return order;
}

// sad_bindings.cu:1399-1437 (threshold 0.01 * alpha, 256 attempts per site; seeds handed
// out in site order)
Tensor init_gradient_weighted(const Tensor& sites_, const Tensor& target_, const Tensor& mask_, int64_t site_count,
                              double init_log_tau, double init_radius, double gradient_alpha) {
    need_sites(sites_);
    need(target_, at::kFloat, "target");
    need(mask_, at::kFloat, "mask");
    need_target(target_, mask_);
    c10::cuda::CUDAGuard guard(sites_.device());
    Tensor sites = sites_.contiguous(), target = target_.contiguous(), mask = mask_.contiguous();
    if (site_count <= 0) site_count = sites.size(0);
    size_t nbytes = sad_init_temp_bytes(u32(site_count));
    Tensor temp = at::empty({static_cast<int64_t>(nbytes)}, sites.options().dtype(at::kByte));
    ok(sad_init_gradient_weighted(ptr(sites), u32(site_count), ptr(target), ptr(mask),
                                  0.01f * static_cast<float>(gradient_alpha), 256u, static_cast<float>(init_log_tau),
                                  static_cast<float>(init_radius), static_cast<int>(target.size(1)),
                                  static_cast<int>(target.size(0)), temp.data_ptr(), static_cast<size_t>(temp.numel()),
                                  stream_of(sites)));
    return sites;
}

}  // namespace

TORCH_LIBRARY(sad, m) {
    m.def("render_sad(Tensor cand0, Tensor cand1, Tensor sites, float inv_scale_sq, int width, int height) -> Tensor");
    m.def("render_sad_padded(Tensor cand0, Tensor cand1, Tensor sites, float inv_scale_sq, int width, int height, int cand_width, int cand_height) -> Tensor");
    m.def("init_candidates(int width, int height, int site_count, int seed) -> (Tensor, Tensor)");
    m.def("vpt_pass(Tensor cand0, Tensor cand1, Tensor sites, float inv_scale_sq, int width, int height, int jump, int radius_probes, float radius_scale, int inject_count, int seed) -> (Tensor, Tensor)");
    m.def("render_sad_backward(Tensor cand0, Tensor cand1, Tensor sites, Tensor grad_output, float inv_scale_sq, int width, int height) -> Tensor");
    m.def("clear_buffer(Tensor buffer, int count) -> Tensor");
    m.def("pack_candidate_sites(Tensor sites, Tensor packed, int site_count) -> Tensor");
    m.def("update_candidates_compact(Tensor cand0_in, Tensor cand1_in, Tensor cand0_out, Tensor cand1_out, Tensor packed_sites, Tensor hilbert_order, Tensor hilbert_pos, float inv_scale_sq, int site_count, int step, int step_high, float radius_scale, int radius_probes, int inject_count, int hilbert_probes, int hilbert_window, int cand_downscale, int target_width, int target_height, int cand_width, int cand_height) -> Tensor");
    m.def("jfa_clear(Tensor cand0, Tensor cand1, int cand_width, int cand_height) -> Tensor");
    m.def("jfa_seed(Tensor cand0, Tensor sites, int site_count, int cand_downscale, int cand_width, int cand_height) -> Tensor");
    m.def("jfa_flood(Tensor cand0_in, Tensor cand0_out, Tensor sites, float inv_scale_sq, int site_count, int step_size, int cand_downscale, int cand_width, int cand_height) -> Tensor");
    m.def("compute_gradients_tiled(Tensor cand0, Tensor cand1, Tensor target, Tensor rendered, Tensor mask, Tensor sites, Tensor grad_pos_x, Tensor grad_pos_y, Tensor grad_log_tau, Tensor grad_radius, Tensor grad_color_r, Tensor grad_color_g, Tensor grad_color_b, Tensor grad_dir_x, Tensor grad_dir_y, Tensor grad_log_aniso, Tensor removal_delta, float inv_scale_sq, int site_count, int compute_removal, float ssim_weight, int cand_width, int cand_height) -> Tensor");
    m.def("tau_diffuse(Tensor cand0, Tensor cand1, Tensor sites, Tensor grad_raw, Tensor grad_in, Tensor grad_out, int site_count, float lambda, int cand_downscale, int cand_width, int cand_height) -> Tensor");
    m.def("adam_update(Tensor sites, Tensor adam, Tensor grad_pos_x, Tensor grad_pos_y, Tensor grad_log_tau, Tensor grad_radius, Tensor grad_color_r, Tensor grad_color_g, Tensor grad_color_b, Tensor grad_dir_x, Tensor grad_dir_y, Tensor grad_log_aniso, float lr_pos, float lr_tau, float lr_radius, float lr_color, float lr_dir, float lr_aniso, float beta1, float beta2, float eps, int t, int width, int height) -> Tensor");
    m.def("compute_site_stats_tiled(Tensor cand0, Tensor cand1, Tensor target, Tensor mask, Tensor sites, Tensor mass, Tensor energy, Tensor err_w, Tensor err_wx, Tensor err_wy, Tensor err_wxx, Tensor err_wxy, Tensor err_wyy, float inv_scale_sq, int site_count, int cand_width, int cand_height) -> Tensor");
    m.def("compute_densify_score_pairs(Tensor sites, Tensor mass, Tensor energy, Tensor pairs, int site_count, float min_mass, float score_alpha, int pair_count) -> Tensor");
    m.def("compute_prune_score_pairs(Tensor sites, Tensor removal_delta, Tensor pairs, int site_count, float delta_norm, int pair_count) -> Tensor");
    m.def("radix_sort_pairs(Tensor pairs, int max_key_exclusive) -> Tensor");
    m.def("write_split_indices(Tensor pairs, Tensor indices, int num_to_split) -> Tensor");
    m.def("split_sites(Tensor sites, Tensor adam, Tensor split_indices, Tensor mass, Tensor err_w, Tensor err_wx, Tensor err_wy, Tensor err_wxx, Tensor err_wxy, Tensor err_wyy, int current_site_count, int num_to_split, Tensor target) -> Tensor");
    m.def("prune_sites(Tensor sites, Tensor indices, int count) -> Tensor");
    m.def("build_hilbert_pairs(Tensor sites, Tensor pairs, int site_count, int padded_count, int width, int height, int bits) -> Tensor");
    m.def("write_hilbert_order(Tensor pairs, Tensor order, Tensor pos, int site_count) -> Tensor");
    m.def("init_gradient_weighted(Tensor sites, Tensor target, Tensor mask, int site_count, float init_log_tau, float init_radius, float gradient_alpha) -> Tensor");
    // no tensor arguments: a catch-all kernel, as the reference registers it
    m.impl("init_candidates", &init_candidates);
}

TORCH_LIBRARY_IMPL(sad, CUDA, m) {
    m.impl("render_sad", &render_sad);
    m.impl("render_sad_padded", &render_sad_padded);
    m.impl("vpt_pass", &vpt_pass);
    m.impl("render_sad_backward", &render_sad_backward);
    m.impl("clear_buffer", &clear_buffer);
    m.impl("pack_candidate_sites", &pack_candidate_sites);
    m.impl("update_candidates_compact", &update_candidates_compact);
    m.impl("jfa_clear", &jfa_clear);
    m.impl("jfa_seed", &jfa_seed);
    m.impl("jfa_flood", &jfa_flood);
    m.impl("compute_gradients_tiled", &compute_gradients_tiled);
    m.impl("tau_diffuse", &tau_diffuse);
    m.impl("adam_update", &adam_update);
    m.impl("compute_site_stats_tiled", &compute_site_stats_tiled);
    m.impl("compute_densify_score_pairs", &compute_densify_score_pairs);
    m.impl("compute_prune_score_pairs", &compute_prune_score_pairs);
    m.impl("radix_sort_pairs", &radix_sort_pairs);
    m.impl("write_split_indices", &write_split_indices);
    m.impl("split_sites", &split_sites);
    m.impl("prune_sites", &prune_sites);
    m.impl("build_hilbert_pairs", &build_hilbert_pairs);
    m.impl("write_hilbert_order", &write_hilbert_order);
    m.impl("init_gradient_weighted", &init_gradient_weighted);
}
