// sources.cuh -- where per-pixel kernels read site data from, and the per-candidate
// gradient algebra shared by the autograd adjoint and the fused training kernel.
#pragma once

#include "common.cuh"
#include "packed.cuh"

namespace sad {

// ---------------------------------------------------------------------------
// site sources: raw [N,10] sites (API calls) or prepared SiteGeom/SiteColor (trainer)
// ---------------------------------------------------------------------------
struct RawSites {
    const Site* s;
    __device__ __forceinline__ void load(uint32_t id, SiteGeom& g, float3& c) const {
        const float2* q = reinterpret_cast<const float2*>(s + id);
        float2 a = __ldg(q), b = __ldg(q + 1), cc = __ldg(q + 2), d = __ldg(q + 3), e = __ldg(q + 4);
        // a = (px, py), b = (log_tau, radius), cc = (r, g), d = (b, dx), e = (dy, log_aniso)
        g = make_geom(a.x, a.y, b.x, b.y, d.y, e.x, e.y);
        c = make_float3(cc.x, cc.y, d.x);
    }
    __device__ __forceinline__ float px(uint32_t id) const { return __ldg(&s[id].px); }
    __device__ __forceinline__ void prepare() {}
};

struct PreparedSites {
    const SiteGeom* g;
    const SiteColor* c;
    __device__ __forceinline__ void load(uint32_t id, SiteGeom& geom, float3& col) const {
        geom = load_geom(g, id);
        float4 v = __ldg(reinterpret_cast<const float4*>(c + id));
        col = make_float3(v.x, v.y, v.z);
    }
    __device__ __forceinline__ float px(uint32_t id) const { return __ldg(&g[id].px); }
    __device__ __forceinline__ void prepare() {}
};

// 16-byte quantised sites (packed.cuh), decoded per candidate; an inactive site reads as
// position (-1, -1) so it is skipped like a pruned one (packedActive,
// backends/metal/shaders/sad_common.metal:85-87).  prepare() loads the ranges once per thread.
struct PackedSites {
    const uint4* p;
    const float* quant;  // device PackedQuant
    float dim_x, dim_y;  // W-1, H-1
    PackedQuant q;
    __device__ __forceinline__ void prepare() { q = load_packed_quant(quant); }
    __device__ __forceinline__ void load(uint32_t id, SiteGeom& g, float3& c) const {
        uint4 w = __ldg(p + id);
        Site s = decode_packed_site(w, q, dim_x, dim_y);
        if (!packed_active(w.x)) s.px = s.py = -1.0f;
        g = make_geom(s.px, s.py, s.log_tau, s.radius, s.dx, s.dy, s.log_aniso);
        c = make_float3(s.r, s.g, s.b);
    }
};

// Per-candidate parameter gradients for dL/dpred; out in site order.  clamp_l1 selects
// the fused kernel's l2 = 1 / max(l1, 1e-8) (gradients.cu:383) over 1 / l1
// (sad_bindings.cu:166).
__device__ __forceinline__ void candidate_grads(const SiteGeom& g, float3 col, float ux, float uy,
                                                float inv_s2, float inv_scale, float w,
                                                float3 dLdp, float3 pred, bool clamp_l1,
                                                float (&o)[10]) {
    o[4] = w * dLdp.x;
    o[5] = w * dLdp.y;
    o[6] = w * dLdp.z;
    float dlogit = dLdp.x * w * (col.x - pred.x) + dLdp.y * w * (col.y - pred.y) +
                   dLdp.z * w * (col.z - pred.z);
    float tau = g.tau;
    float dx = ux - g.px, dy = uy - g.py;
    float diff2 = dx * dx + dy * dy;
    float proj = g.dx * dx + g.dy * dy;
    float proj2 = proj * proj;
    float perp2 = fmaxf(diff2 - proj2, 0.0f);
    float l1 = g.l1;
    float l2 = (clamp_l1 && !(l1 >= 1e-8f)) ? 1.0f / 1e-8f : g.l2;
    float d2n = (l1 * proj2 + l2 * perp2) * inv_s2;
    float d2s = fmaxf(d2n, 1e-8f);
    float isq = rsqrtf(d2s);
    float rn = g.radius * inv_scale;
    float dm = d2s * isq - rn;  // sqrt(d2s) from the reciprocal root already at hand
    float gdx = l2 * dx + (l1 - l2) * g.dx * proj;
    float gdy = l2 * dy + (l1 - l2) * g.dy * proj;
    float kpos = tau * inv_s2 * isq;
    o[0] = dlogit * kpos * gdx;
    o[1] = dlogit * kpos * gdy;
    o[2] = dlogit * (-dm) * tau;
    o[3] = dlogit * tau * inv_scale;
    float dla = (l1 * proj2 - l2 * perp2) * inv_s2;
    float kang = dlogit * (-tau) * (0.5f * isq);
    float kdir = 2.0f * (l1 - l2) * proj * inv_s2;
    o[7] = kang * (kdir * dx);
    o[8] = kang * (kdir * dy);
    o[9] = kang * dla;
}

}  // namespace sad
