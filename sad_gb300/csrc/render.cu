// render.cu -- per-site preparation, softmax-over-candidates render, candidate init, and
// the autograd adjoint of the render.
//
// Launch shape of the per-pixel kernels: 32x8 threads, one pixel per thread, so a warp
// reads one 512-byte row segment of each candidate field (two 16-byte loads per lane).
#include "accum.cuh"
#include "common.cuh"
#include "sources.cuh"
#include "host_common.h"
#include "kernels.h"

namespace sad {

// ---------------------------------------------------------------------------
// prepare: Site -> SiteGeom + SiteColor
// ---------------------------------------------------------------------------
__global__ void prepare_sites_kernel(const Site* __restrict__ sites, SiteGeom* __restrict__ geom,
                                     SiteColor* __restrict__ color, uint32_t n) {
    pdl_wait();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2* q = reinterpret_cast<const float2*>(sites + i);
    float2 a = q[0], b = q[1], c = q[2], d = q[3], e = q[4];
    store_geom(geom, i, make_geom(a.x, a.y, b.x, b.y, d.y, e.x, e.y));
    reinterpret_cast<float4*>(color)[i] = make_float4(c.x, c.y, d.x, 0.0f);
}

void launch_prepare_sites(const Site* sites, SiteGeom* geom, SiteColor* color, uint32_t n,
                          cudaStream_t st) {
    if (n == 0) return;
    launch_pdl(prepare_sites_kernel, dim3(blocks_for(n, 256)), dim3(256), 0, st, sites, geom, color, n);
    note_launches(1);
}

// ---------------------------------------------------------------------------
// forward render (backends/cuda/src/render.cu:5-92)
// ---------------------------------------------------------------------------
template <class Src>
__global__ void __launch_bounds__(256) render_kernel(const uint4* __restrict__ cand0,
                                                     const uint4* __restrict__ cand1,
                                                     float* __restrict__ out, Src src,
                                                     float inv_s2, uint32_t n, int w, int h,
                                                     int cw, int ch) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    pdl_wait();
    if (x >= w || y >= h) return;
    src.prepare();
    int p = y * w + x;
    float ux = static_cast<float>(x), uy = static_cast<float>(y);
    float inv_scale = sqrtf(inv_s2);
    int ci = cand_index_for_pixel(x, y, w, h, cw, ch);
    uint4 a = __ldg(cand0 + ci), b = __ldg(cand1 + ci);
    uint32_t ids[kCand] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};

    float logits[kCand];
    float3 cols[kCand];
    float mx = -INFINITY;
    uint32_t blend = 0;  // sites the colour blend reads: position.x >= 0 (render.cu:83)
#pragma unroll
    for (int i = 0; i < kCand; ++i) {
        logits[i] = -INFINITY;
        cols[i] = make_float3(0.f, 0.f, 0.f);
        uint32_t id = ids[i];
        if (id >= n) continue;
        SiteGeom g;
        src.load(id, g, cols[i]);
        if (g.px < 0.0f) continue;
        if (g.px >= 0.0f) blend |= 1u << i;
        float tau = g.tau;
        float d = dmix2(g, ux, uy, inv_s2, inv_scale);
        logits[i] = -tau * d;
        mx = fmaxf(mx, logits[i]);
    }
    float r = 0.f, gg = 0.f, bb = 0.f;
    if (!(isinf(mx) && mx < 0.0f)) {
        float wts[kCand];
        float sum = 0.0f;
#pragma unroll
        for (int i = 0; i < kCand; ++i) {
            wts[i] = expf(logits[i] - mx);
            sum += wts[i];
        }
        float inv_sum = 1.0f / fmaxf(sum, 1e-8f);
#pragma unroll
        for (int i = 0; i < kCand; ++i) {
            float wi = wts[i] * inv_sum;
            if (!isnan(wi) && !isinf(wi) && (blend >> i & 1u)) {
                r += wi * cols[i].x;
                gg += wi * cols[i].y;
                bb += wi * cols[i].z;
            }
        }
    }
    out[3 * p + 0] = r;
    out[3 * p + 1] = gg;
    out[3 * p + 2] = bb;
}

static dim3 pixel_grid(int w, int h) { return dim3((w + 31) / 32, (h + 7) / 8); }

void launch_render_raw(const uint32_t* c0, const uint32_t* c1, float* out, const Site* sites,
                       float inv_s2, uint32_t n, int w, int h, int cw, int ch, cudaStream_t st) {
    render_kernel<RawSites><<<pixel_grid(w, h), dim3(32, 8), 0, st>>>(
        reinterpret_cast<const uint4*>(c0), reinterpret_cast<const uint4*>(c1), out,
        RawSites{sites}, inv_s2, n, w, h, cw, ch);
    note_launches(1);
}

void launch_render_prepared(const uint32_t* c0, const uint32_t* c1, float* out,
                            const SiteGeom* geom, const SiteColor* color, float inv_s2,
                            uint32_t n, int w, int h, int cw, int ch, cudaStream_t st) {
    launch_pdl(render_kernel<PreparedSites>, pixel_grid(w, h), dim3(32, 8), 0, st,
               reinterpret_cast<const uint4*>(c0), reinterpret_cast<const uint4*>(c1), out,
               PreparedSites{geom, color}, inv_s2, n, w, h, cw, ch);
    note_launches(1);
}

// renderVoronoiPacked (backends/metal/shaders/encoders/packed_render_encoder.metal:3-31):
// the same render over 16-byte quantised sites.
void launch_render_packed(const uint32_t* c0, const uint32_t* c1, float* out, const uint32_t* packed,
                          const float* quant, float inv_s2, uint32_t n, int w, int h, int cw, int ch,
                          cudaStream_t st) {
    PackedSites src{};
    src.p = reinterpret_cast<const uint4*>(packed);
    src.quant = quant;
    src.dim_x = static_cast<float>(w - 1);
    src.dim_y = static_cast<float>(h - 1);
    render_kernel<PackedSites><<<pixel_grid(w, h), dim3(32, 8), 0, st>>>(
        reinterpret_cast<const uint4*>(c0), reinterpret_cast<const uint4*>(c1), out, src, inv_s2, n, w, h,
        cw, ch);
    note_launches(1);
}

// ---------------------------------------------------------------------------
// candidate init / clear (backends/cuda/src/render.cu:95-154)
// ---------------------------------------------------------------------------
__global__ void init_candidates_kernel(uint4* __restrict__ c0, uint4* __restrict__ c1, uint32_t n,
                                       uint32_t seed, int per_pixel, int w, int h) {
    pdl_wait();
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    int p = y * w + x;
    uint32_t idx[kCand];
    if (per_pixel && n == static_cast<uint32_t>(w * h)) {
        const int nb[7][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}, {-1, -1}, {1, -1}, {-1, 1}};
        idx[0] = static_cast<uint32_t>(p);
#pragma unroll
        for (int i = 0; i < 7; ++i) {
            int nx = clampi(x + nb[i][0], 0, w - 1), ny = clampi(y + nb[i][1], 0, h - 1);
            idx[i + 1] = static_cast<uint32_t>(ny * w + nx);
        }
    } else if (n == 0) {
#pragma unroll
        for (int i = 0; i < kCand; ++i) idx[i] = kEmpty;
    } else {
        uint32_t s = seed ^ (static_cast<uint32_t>(x) * 1973u) ^ (static_cast<uint32_t>(y) * 9277u);
#pragma unroll
        for (int i = 0; i < kCand; ++i) {
            s = xorshift32(s + static_cast<uint32_t>(i));
            idx[i] = s % n;
        }
    }
    c0[p] = make_uint4(idx[0], idx[1], idx[2], idx[3]);
    c1[p] = make_uint4(idx[4], idx[5], idx[6], idx[7]);
}

__global__ void fill_u32x4_kernel(uint4* __restrict__ a, uint4* __restrict__ b, size_t count,
                                  uint32_t v) {
    pdl_wait();
    size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
    size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    uint4 f = make_uint4(v, v, v, v);
    for (; i < count; i += stride) {
        a[i] = f;
        if (b) b[i] = f;
    }
}

void launch_init_candidates(uint32_t* c0, uint32_t* c1, uint32_t n, uint32_t seed, int per_pixel,
                            int w, int h, cudaStream_t st) {
    launch_pdl(init_candidates_kernel, pixel_grid(w, h), dim3(32, 8), 0, st, reinterpret_cast<uint4*>(c0),
               reinterpret_cast<uint4*>(c1), n, seed, per_pixel, w, h);
    note_launches(1);
}

void launch_clear_candidates(uint32_t* c0, uint32_t* c1, int w, int h, cudaStream_t st) {
    size_t count = static_cast<size_t>(w) * h;
    unsigned blocks = static_cast<unsigned>(std::min<size_t>((count + 255) / 256, 152 * 16));
    launch_pdl(fill_u32x4_kernel, dim3(blocks), dim3(256), 0, st, reinterpret_cast<uint4*>(c0),
               reinterpret_cast<uint4*>(c1), count, kEmpty);
    note_launches(1);
}

// ---------------------------------------------------------------------------
// autograd adjoint (backends/pytorch/torch_ext/cuda/sad_bindings.cu:41-207)
// ---------------------------------------------------------------------------
// Key-table size per 256-pixel tile: 256 slots while sites are sparse enough (at most one
// per four pixels: a tile then sees well under 200 distinct candidates), 512 above that.
// Four blocks per SM (64 registers a thread) keep 32 warps resident for the latency of the
// shared-memory atomics.
template <class Src, int kBwdSlots>
__global__ void __launch_bounds__(256, 4) render_backward_kernel(
    const uint4* __restrict__ cand0, const uint4* __restrict__ cand1,
    const float* __restrict__ grad_rgb, float* __restrict__ grad_sites, Src src, float inv_s2,
    uint32_t n, int w, int h, int cw, int ch) {
    using Table = TileTable<10, kBwdSlots, AccFloat>;
    auto& table = shared_table<Table>();
    int tid = threadIdx.y * blockDim.x + threadIdx.x;
    table.init(tid, 256);
    __syncthreads();

    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    bool inb = x < w && y < h;
    float ux = static_cast<float>(x), uy = static_cast<float>(y);
    float inv_scale = sqrtf(inv_s2);
    uint32_t ids[kCand];
    float wts[kCand];
    float3 pred = make_float3(0.f, 0.f, 0.f);
    float3 dLdp = make_float3(0.f, 0.f, 0.f);
    uint32_t valid = 0;  // softmax members: id < n and !(position.x < 0)
    uint32_t blend = 0;  // colour contributors: position.x >= 0
#pragma unroll
    for (int i = 0; i < kCand; ++i) {
        ids[i] = kEmpty;
        wts[i] = 0.0f;
    }
    if (inb) {
        int p = y * w + x;
        int ci = cand_index_for_pixel(x, y, w, h, cw, ch);
        uint4 a = __ldg(cand0 + ci), b = __ldg(cand1 + ci);
        ids[0] = a.x; ids[1] = a.y; ids[2] = a.z; ids[3] = a.w;
        ids[4] = b.x; ids[5] = b.y; ids[6] = b.z; ids[7] = b.w;
        float logits[kCand];
        float3 cols[kCand];
        float mx = -INFINITY;
#pragma unroll
        for (int i = 0; i < kCand; ++i) {
            logits[i] = -INFINITY;
            cols[i] = make_float3(0.f, 0.f, 0.f);
            if (ids[i] >= n) continue;
            SiteGeom g;
            src.load(ids[i], g, cols[i]);
            if (g.px < 0.0f) continue;
            valid |= 1u << i;
            if (g.px >= 0.0f) blend |= 1u << i;
            logits[i] = -g.tau * dmix2(g, ux, uy, inv_s2, inv_scale);
            mx = fmaxf(mx, logits[i]);
        }
        // compute_candidate_weights_raw bails out when nothing is valid or max is +-inf
        if (valid == 0u || isinf(mx)) {
            valid = 0u;
        } else {
            float sum = 0.0f;
#pragma unroll
            for (int i = 0; i < kCand; ++i) {
                wts[i] = expf(logits[i] - mx);
                sum += wts[i];
            }
            float inv_sum = 1.0f / fmaxf(sum, 1e-8f);
#pragma unroll
            for (int i = 0; i < kCand; ++i) {
                wts[i] *= inv_sum;
                if (blend >> i & 1u) {
                    pred.x += wts[i] * cols[i].x;
                    pred.y += wts[i] * cols[i].y;
                    pred.z += wts[i] * cols[i].z;
                }
            }
            dLdp = make_float3(__ldg(grad_rgb + 3 * p), __ldg(grad_rgb + 3 * p + 1),
                               __ldg(grad_rgb + 3 * p + 2));
        }
    }
    int slots[kCand];
#pragma unroll
    for (int i = 0; i < kCand; ++i)
        slots[i] = register_key(table, (valid >> i & 1u) ? ids[i] : kEmpty);
    const uint32_t r = lane_rotation();
    rotate8(ids, r);
    rotate8(wts, r);
    rotate8(slots, r);
    const uint32_t vr = rotate_mask8(valid, r);
#pragma unroll
    for (int j = 0; j < kCand; ++j) {
        if (!(vr >> j & 1u)) continue;
        SiteGeom g;
        float3 col;
        src.load(ids[j], g, col);
        float v[10];
        candidate_grads(g, col, ux, uy, inv_s2, inv_scale, wts[j], dLdp, pred, false, v);
        if (slots[j] >= 0) {
            table.add(slots[j], v);
        } else {
            float* gs = grad_sites + static_cast<size_t>(ids[j]) * 10;
#pragma unroll
            for (int k = 0; k < 10; ++k) atomicAdd(gs + k, v[k]);
        }
    }
    __syncthreads();
    const int used = table.size();
    for (int d = tid; d < used; d += 256) {
        float* gs = grad_sites + static_cast<size_t>(table.key_at(d)) * 10;
#pragma unroll
        for (int k = 0; k < 10; ++k) atomicAdd(gs + k, table.value(k, d));
    }
}

void launch_render_backward_raw(const uint32_t* c0, const uint32_t* c1, const float* grad_rgb,
                                float* grad_sites, const Site* sites, float inv_s2, uint32_t n,
                                int w, int h, int cw, int ch, cudaStream_t st) {
    auto c0v = reinterpret_cast<const uint4*>(c0);
    auto c1v = reinterpret_cast<const uint4*>(c1);
    if (static_cast<double>(n) * 4.0 <= static_cast<double>(w) * h)
        render_backward_kernel<RawSites, 256><<<pixel_grid(w, h), dim3(32, 8),
                                                sizeof(TileTable<10, 256, AccFloat>), st>>>(
            c0v, c1v, grad_rgb, grad_sites, RawSites{sites}, inv_s2, n, w, h, cw, ch);
    else
        render_backward_kernel<RawSites, 512><<<pixel_grid(w, h), dim3(32, 8),
                                                sizeof(TileTable<10, 512, AccFloat>), st>>>(
            c0v, c1v, grad_rgb, grad_sites, RawSites{sites}, inv_s2, n, w, h, cw, ch);
    note_launches(1);
}

}  // namespace sad

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace sad;

extern "C" sad_status_t sad_render(const uint32_t* cand0, const uint32_t* cand1, float* out_rgb,
                                   const float* sites, float inv_scale_sq, uint32_t site_count,
                                   int width, int height, int cand_width, int cand_height,
                                   sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_render: invalid image size");
    SAD_REQUIRE(image_size_ok(cand_width, cand_height), "sad_render: invalid cand size");
    SAD_REQUIRE(cand0 && cand1 && out_rgb, "sad_render: null buffer");
    SAD_REQUIRE(sites || site_count == 0, "sad_render: null sites");
    launch_render_raw(cand0, cand1, out_rgb, reinterpret_cast<const Site*>(sites), inv_scale_sq,
                      site_count, width, height, cand_width, cand_height, as_stream(stream));
    return check_launch("sad_render");
}

extern "C" sad_status_t sad_render_backward(const uint32_t* cand0, const uint32_t* cand1,
                                            const float* grad_rgb, float* grad_sites,
                                            const float* sites, float inv_scale_sq,
                                            uint32_t site_count, int width, int height,
                                            int cand_width, int cand_height, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_render_backward: invalid image size");
    SAD_REQUIRE(image_size_ok(cand_width, cand_height), "sad_render_backward: invalid cand size");
    SAD_REQUIRE(cand0 && cand1 && grad_rgb && grad_sites, "sad_render_backward: null buffer");
    SAD_REQUIRE(sites || site_count == 0, "sad_render_backward: null sites");
    launch_render_backward_raw(cand0, cand1, grad_rgb, grad_sites,
                               reinterpret_cast<const Site*>(sites), inv_scale_sq, site_count,
                               width, height, cand_width, cand_height, as_stream(stream));
    return check_launch("sad_render_backward");
}

extern "C" sad_status_t sad_init_candidates(uint32_t* cand0, uint32_t* cand1, uint32_t site_count,
                                            uint32_t seed, int per_pixel, int width, int height,
                                            sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_init_candidates: invalid cand size");
    SAD_REQUIRE(cand0 && cand1, "sad_init_candidates: null buffer");
    launch_init_candidates(cand0, cand1, site_count, seed, per_pixel, width, height,
                           as_stream(stream));
    return check_launch("sad_init_candidates");
}

extern "C" sad_status_t sad_clear_candidates(uint32_t* cand0, uint32_t* cand1, int width,
                                             int height, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_clear_candidates: invalid cand size");
    SAD_REQUIRE(cand0 && cand1, "sad_clear_candidates: null buffer");
    launch_clear_candidates(cand0, cand1, width, height, as_stream(stream));
    return check_launch("sad_clear_candidates");
}
