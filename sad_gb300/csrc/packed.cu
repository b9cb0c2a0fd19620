// packed.cu -- the 16-byte quantised inference format: pack (with the quantisation ranges
// reduced on the device), unpack, and render from packed sites.
//
// backends/metal/sources/utils/packed_inference.swift:86-199 packs on the host after a fit;
// here the ranges and the words are computed where the sites already are (HBM), so a fit's
// serving copy is 16 bytes per site without a host round trip.  Every product, sum and
// quotient is rounded separately (__fmul_rn, __fadd_rn, __fdiv_rn), the arithmetic of the
// unfused host code, so the words do not depend on fused multiply-add choices.
#include <cuda_fp16.h>

#include "common.cuh"
#include "host_common.h"
#include "kernels.h"
#include "packed.cuh"

namespace sad {

namespace {

// Order-preserving map of floats onto u32, so atomicMin / atomicMax give float min / max.
__device__ __forceinline__ uint32_t order_key(float f) {
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float order_value(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

constexpr int kQuantFields = 5;  // log_tau, radius, r, g, b

// keys[0..4] = min keys, keys[5..9] = max keys
__global__ void quant_init_kernel(uint32_t* __restrict__ keys) {
    int i = threadIdx.x;
    if (i < kQuantFields) {
        keys[i] = 0xFFFFFFFFu;
        keys[kQuantFields + i] = 0u;
    }
}

// Ranges over the active sites (x >= 0 and y >= 0) of the finite values of each field
// (packed_inference.swift:87-130).
__global__ void __launch_bounds__(256) quant_reduce_kernel(const Site* __restrict__ sites, uint32_t n,
                                                           uint32_t* __restrict__ keys) {
    uint32_t lo[kQuantFields], hi[kQuantFields];
#pragma unroll
    for (int f = 0; f < kQuantFields; ++f) {
        lo[f] = 0xFFFFFFFFu;
        hi[f] = 0u;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float2* q = reinterpret_cast<const float2*>(sites + i);
        float2 pos = __ldg(q), tr = __ldg(q + 1), rg = __ldg(q + 2), bd = __ldg(q + 3);
        if (!(pos.x >= 0.0f && pos.y >= 0.0f)) continue;
        float v[kQuantFields] = {tr.x, tr.y, rg.x, rg.y, bd.x};
#pragma unroll
        for (int f = 0; f < kQuantFields; ++f) {
            if (!isfinite(v[f])) continue;
            uint32_t k = order_key(v[f]);
            lo[f] = min(lo[f], k);
            hi[f] = max(hi[f], k);
        }
    }
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int f = 0; f < kQuantFields; ++f) {
        uint32_t a = __reduce_min_sync(0xFFFFFFFFu, lo[f]);
        uint32_t b = __reduce_max_sync(0xFFFFFFFFu, hi[f]);
        if (lane == 0) {
            if (a != 0xFFFFFFFFu) atomicMin(keys + f, a);
            if (b != 0u) atomicMax(keys + kQuantFields + f, b);
        }
    }
}

// Keys -> PackedQuant: an empty range (no active finite value) is [0, 0]; scales are
// max(max - min, 1e-6) (packed_inference.swift:132-162).
__global__ void quant_finalize_kernel(float* quant) {
    const uint32_t* keys = reinterpret_cast<const uint32_t*>(quant);
    if (threadIdx.x != 0) return;
    float out[2 * kQuantFields];
#pragma unroll
    for (int f = 0; f < kQuantFields; ++f) {
        uint32_t a = keys[f], b = keys[kQuantFields + f];
        float mn = 0.0f, mx = 0.0f;
        if (a != 0xFFFFFFFFu && b != 0u) {
            mn = order_value(a);
            mx = order_value(b);
        }
        out[2 * f] = mn;
        out[2 * f + 1] = fmaxf(__fsub_rn(mx, mn), 1.0e-6f);
    }
#pragma unroll
    for (int i = 0; i < 2 * kQuantFields; ++i) quant[i] = out[i];
}

// UInt32(n * levels + 0.5) of n = clamp((v - min) / scale, 0, 1); 0 when scale <= 0.
__device__ __forceinline__ uint32_t pack_unorm(float v, float minv, float scale, float levels) {
    if (scale <= 0.0f) return 0u;
    float n = fminf(fmaxf(__fdiv_rn(__fsub_rn(v, minv), scale), 0.0f), 1.0f);
    return static_cast<uint32_t>(__fadd_rn(__fmul_rn(n, levels), 0.5f));
}

// As pack_unorm over [0, max_value].
__device__ __forceinline__ uint32_t pack_unorm_max(float v, float max_value, float levels) {
    if (max_value <= 0.0f) return 0u;
    float n = fminf(fmaxf(__fdiv_rn(v, max_value), 0.0f), 1.0f);
    return static_cast<uint32_t>(__fadd_rn(__fmul_rn(n, levels), 0.5f));
}

// Direction -> unorm16 of its angle in [-pi, pi] (packAngle / normalizedDir,
// packed_inference.swift:33-38, 79-85).
__device__ __forceinline__ uint32_t pack_angle(float dx, float dy) {
    float len2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
    float ux = 1.0f, uy = 0.0f;
    if (!(len2 < 1.0e-8f)) {
        float inv = __fdiv_rn(1.0f, __fsqrt_rn(len2));
        ux = __fmul_rn(dx, inv);
        uy = __fmul_rn(dy, inv);
    }
    const float pi = 3.14159265358979f;  // Float.pi
    float angle = atan2f(uy, ux);
    float n = fminf(fmaxf(__fdiv_rn(__fadd_rn(angle, pi), __fmul_rn(pi, 2.0f)), 0.0f), 1.0f);
    return static_cast<uint32_t>(__fadd_rn(__fmul_rn(n, 65535.0f), 0.5f));
}

__global__ void __launch_bounds__(256) pack_sites_kernel(const Site* __restrict__ sites, uint32_t n,
                                                         const float* __restrict__ quant, float max_x,
                                                         float max_y, uint4* __restrict__ packed) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const PackedQuant q = load_packed_quant(quant);
    const float2* src = reinterpret_cast<const float2*>(sites + i);
    float2 pos = __ldg(src), tr = __ldg(src + 1), rg = __ldg(src + 2), bd = __ldg(src + 3),
           ea = __ldg(src + 4);
    bool active = pos.x >= 0.0f && pos.y >= 0.0f;
    float x = fminf(fmaxf(pos.x, 0.0f), max_x);
    float y = fminf(fmaxf(pos.y, 0.0f), max_y);
    uint32_t w0 = pack_unorm_max(x, max_x, 32767.0f) | (pack_unorm_max(y, max_y, 32767.0f) << 15);
    w0 = (w0 & 0x3fffffffu) | ((active ? 0u : 1u) << 30);
    uint32_t w1 = pack_unorm(rg.x, q.r_min, q.r_scale, 2047.0f) |
                  (pack_unorm(rg.y, q.g_min, q.g_scale, 2047.0f) << 11) |
                  (pack_unorm(bd.x, q.b_min, q.b_scale, 1023.0f) << 22);
    float log_tau = isfinite(tr.x) ? tr.x : q.log_tau_min;
    float radius = isfinite(tr.y) ? tr.y : q.radius_min;
    uint32_t w2 = pack_unorm(log_tau, q.log_tau_min, q.log_tau_scale, 65535.0f) |
                  (pack_unorm(radius, q.radius_min, q.radius_scale, 65535.0f) << 16);
    float log_aniso = isfinite(ea.y) ? ea.y : 0.0f;
    uint32_t half_bits = __half_as_ushort(__float2half_rn(log_aniso));
    uint32_t w3 = (pack_angle(bd.y, ea.x) & 0xffffu) | (half_bits << 16);
    packed[i] = make_uint4(w0, w1, w2, w3);
}

__global__ void __launch_bounds__(256) unpack_sites_kernel(const uint4* __restrict__ packed, uint32_t n,
                                                           const float* __restrict__ quant, float dim_x,
                                                           float dim_y, Site* __restrict__ sites) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const PackedQuant q = load_packed_quant(quant);
    uint4 w = __ldg(packed + i);
    Site s = decode_packed_site(w, q, dim_x, dim_y);
    if (!packed_active(w.x)) s.px = s.py = -1.0f;
    float2* d = reinterpret_cast<float2*>(sites + i);
    d[0] = make_float2(s.px, s.py);
    d[1] = make_float2(s.log_tau, s.radius);
    d[2] = make_float2(s.r, s.g);
    d[3] = make_float2(s.b, s.dx);
    d[4] = make_float2(s.dy, s.log_aniso);
}

}  // namespace

// Ranges then words.  The range reduction works on order keys stored in the quant buffer
// itself (ten u32), which the finalize kernel turns into the ten floats in place.
void launch_pack_inference(const Site* sites, uint32_t n, int w, int h, float* quant, uint32_t* packed,
                           cudaStream_t st) {
    uint32_t* keys = reinterpret_cast<uint32_t*>(quant);
    quant_init_kernel<<<1, 32, 0, st>>>(keys);
    if (n > 0) {
        unsigned blocks = std::min<unsigned>(blocks_for(n, 256), 152u * 4u);
        quant_reduce_kernel<<<blocks, 256, 0, st>>>(sites, n, keys);
    }
    quant_finalize_kernel<<<1, 32, 0, st>>>(quant);
    note_launches(n > 0 ? 3 : 2);
    if (n == 0) return;
    pack_sites_kernel<<<blocks_for(n, 256), 256, 0, st>>>(
        sites, n, quant, static_cast<float>(std::max(w - 1, 0)), static_cast<float>(std::max(h - 1, 0)),
        reinterpret_cast<uint4*>(packed));
    note_launches(1);
}

void launch_unpack_inference(const uint32_t* packed, const float* quant, uint32_t n, int w, int h, Site* sites,
                             cudaStream_t st) {
    if (n == 0) return;
    unpack_sites_kernel<<<blocks_for(n, 256), 256, 0, st>>>(reinterpret_cast<const uint4*>(packed), n, quant,
                                                           static_cast<float>(w - 1), static_cast<float>(h - 1),
                                                           sites);
    note_launches(1);
}

}  // namespace sad

using namespace sad;

namespace {

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

extern "C" sad_status_t sad_pack_inference_sites(const float* sites, uint32_t site_count, int width,
                                                 int height, uint32_t* packed, sad_packed_quant_t* quant,
                                                 sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_pack_inference_sites: invalid size");
    SAD_REQUIRE(width <= 32768 && height <= 32768, "sad_pack_inference_sites: image side above 32768");
    SAD_REQUIRE(quant && (site_count == 0 || (sites && packed)), "sad_pack_inference_sites: null buffer");
    launch_pack_inference(reinterpret_cast<const Site*>(sites), site_count, width, height,
                          reinterpret_cast<float*>(quant), packed, as_stream(stream));
    return check_launch("sad_pack_inference_sites");
}

extern "C" sad_status_t sad_unpack_inference_sites(const uint32_t* packed, const sad_packed_quant_t* quant,
                                                   uint32_t site_count, int width, int height, float* sites,
                                                   sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_unpack_inference_sites: invalid size");
    SAD_REQUIRE(site_count == 0 || (packed && quant && sites), "sad_unpack_inference_sites: null buffer");
    launch_unpack_inference(packed, reinterpret_cast<const float*>(quant), site_count, width, height,
                            reinterpret_cast<Site*>(sites), as_stream(stream));
    return check_launch("sad_unpack_inference_sites");
}

extern "C" sad_status_t sad_render_packed(const uint32_t* cand0, const uint32_t* cand1, float* out_rgb,
                                          const uint32_t* packed, const sad_packed_quant_t* quant,
                                          float inv_scale_sq, uint32_t site_count, int width, int height,
                                          int cand_width, int cand_height, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height) && image_size_ok(cand_width, cand_height),
                "sad_render_packed: invalid size");
    SAD_REQUIRE(cand0 && cand1 && out_rgb && quant && (site_count == 0 || packed),
                "sad_render_packed: null buffer");
    launch_render_packed(cand0, cand1, out_rgb, packed, reinterpret_cast<const float*>(quant), inv_scale_sq,
                         site_count, width, height, cand_width, cand_height, as_stream(stream));
    return check_launch("sad_render_packed");
}

extern "C" size_t sad_render_packed_scratch_bytes(uint32_t site_count, int width, int height,
                                                  int cand_downscale) {
    return 256 + align256(static_cast<size_t>(site_count) * sizeof(Site)) +
           sad_render_scratch_bytes(site_count, width, height, cand_downscale);
}

// The candidate field is built from the decoded sites: the reference's packed JFA / VPT
// encoders decode each site with the same decodePackedSite before using it
// (packed_renderer.swift:15-135), so decoding once gives the same field.
extern "C" sad_status_t sad_render_packed_from_sites(const sad_render_config_t* cfg, const uint32_t* packed,
                                                     const sad_packed_quant_t* quant, uint32_t site_count,
                                                     int width, int height, float* out_rgb, void* scratch,
                                                     size_t scratch_bytes, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(cfg, "sad_render_packed_from_sites: null config");
    SAD_REQUIRE(image_size_ok(width, height), "sad_render_packed_from_sites: invalid size");
    SAD_REQUIRE(site_count > 0 && packed && quant && out_rgb && scratch,
                "sad_render_packed_from_sites: null buffer or no sites");
    SAD_REQUIRE(scratch_bytes >= sad_render_packed_scratch_bytes(site_count, width, height, cfg->cand_downscale),
                "sad_render_packed_from_sites: scratch smaller than sad_render_packed_scratch_bytes()");
    uintptr_t base = (reinterpret_cast<uintptr_t>(scratch) + 255) & ~uintptr_t(255);
    size_t lead = base - reinterpret_cast<uintptr_t>(scratch);
    size_t site_bytes = align256(static_cast<size_t>(site_count) * sizeof(Site));
    SAD_REQUIRE(scratch_bytes >= lead + site_bytes, "sad_render_packed_from_sites: scratch too small");
    float* decoded = reinterpret_cast<float*>(base);
    launch_unpack_inference(packed, reinterpret_cast<const float*>(quant), site_count, width, height,
                            reinterpret_cast<Site*>(decoded), as_stream(stream));
    SAD_TRY(check_launch("sad_render_packed_from_sites"));
    return sad_render_from_sites(cfg, decoded, site_count, width, height, out_rgb,
                                 reinterpret_cast<char*>(base) + site_bytes, scratch_bytes - lead - site_bytes,
                                 stream);
}
