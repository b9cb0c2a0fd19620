// packed.cuh -- the 16-byte quantised inference site (the Metal backend's serving format)
// and its decode, shared by the unpack kernel and the packed render source.
//
// Word layout (backends/metal/sources/utils/packed_inference.swift:164-196):
//   w0: x (unorm15 of [0, W-1]) | y (unorm15 of [0, H-1]) << 15 | inactive << 30
//   w1: r (unorm11) | g (unorm11) << 11 | b (unorm10) << 22, each over the active sites'
//       [min, min + scale] range of that channel
//   w2: log_tau (unorm16) | radius (unorm16) << 16, over their active ranges
//   w3: direction angle atan2(dy, dx) as unorm16 of [-pi, pi] | log_aniso as f16 << 16
// The decode restates backends/metal/shaders/sad_common.metal:71-120.  Every product and
// sum is rounded separately (__fmul_rn / __fadd_rn), so the decoded floats do not depend
// on the compiler's fused multiply-add choices.
#pragma once

#include <cuda_fp16.h>

#include "common.cuh"

namespace sad {

// Quantisation ranges of one packed site set (PackedSiteQuant, packed_inference.swift:7-18).
struct PackedQuant {
    float log_tau_min, log_tau_scale;
    float radius_min, radius_scale;
    float r_min, r_scale;
    float g_min, g_scale;
    float b_min, b_scale;
};
static_assert(sizeof(PackedQuant) == 40, "PackedQuant is 10 floats");

constexpr float kInvUnorm16 = 1.0f / 65535.0f;
constexpr float kInvUnorm15 = 1.0f / 32767.0f;
constexpr float kInvUnorm11 = 1.0f / 2047.0f;
constexpr float kInvUnorm10 = 1.0f / 1023.0f;
constexpr float kPackedPi = 3.14159265f;
constexpr float kPackedTwoPi = 6.2831853f;

__device__ __forceinline__ bool packed_active(uint32_t w0) { return ((w0 >> 30) & 1u) == 0u; }

__device__ __forceinline__ float unpack_unorm(uint32_t v, float inv_levels, float minv, float scale) {
    return __fadd_rn(minv, __fmul_rn(__fmul_rn(static_cast<float>(v), inv_levels), fmaxf(scale, 0.0f)));
}

// Decoded fields in Site order; dim_x / dim_y are W-1 and H-1 of the image.
__device__ __forceinline__ Site decode_packed_site(uint4 w, const PackedQuant& q, float dim_x, float dim_y) {
    Site s;
    s.px = __fmul_rn(__fmul_rn(static_cast<float>(w.x & 0x7fffu), kInvUnorm15), fmaxf(dim_x, 0.0f));
    s.py = __fmul_rn(__fmul_rn(static_cast<float>((w.x >> 15) & 0x7fffu), kInvUnorm15), fmaxf(dim_y, 0.0f));
    s.r = unpack_unorm(w.y & 0x7ffu, kInvUnorm11, q.r_min, q.r_scale);
    s.g = unpack_unorm((w.y >> 11) & 0x7ffu, kInvUnorm11, q.g_min, q.g_scale);
    s.b = unpack_unorm((w.y >> 22) & 0x3ffu, kInvUnorm10, q.b_min, q.b_scale);
    s.log_tau = unpack_unorm(w.z & 0xffffu, kInvUnorm16, q.log_tau_min, q.log_tau_scale);
    s.radius = unpack_unorm(w.z >> 16, kInvUnorm16, q.radius_min, q.radius_scale);
    float angle = __fsub_rn(__fmul_rn(__fmul_rn(static_cast<float>(w.w & 0xffffu), kInvUnorm16), kPackedTwoPi),
                            kPackedPi);
    s.dx = cosf(angle);
    s.dy = sinf(angle);
    s.log_aniso = __half2float(__ushort_as_half(static_cast<unsigned short>(w.w >> 16)));
    return s;
}

__device__ __forceinline__ PackedQuant load_packed_quant(const float* __restrict__ q) {
    PackedQuant r;
    r.log_tau_min = __ldg(q + 0);
    r.log_tau_scale = __ldg(q + 1);
    r.radius_min = __ldg(q + 2);
    r.radius_scale = __ldg(q + 3);
    r.r_min = __ldg(q + 4);
    r.r_scale = __ldg(q + 5);
    r.g_min = __ldg(q + 6);
    r.g_scale = __ldg(q + 7);
    r.b_min = __ldg(q + 8);
    r.b_scale = __ldg(q + 9);
    return r;
}

}  // namespace sad
