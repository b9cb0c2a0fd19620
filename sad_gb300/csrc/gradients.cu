// gradients.cu -- fused training gradient: forward softmax, dL/dpred of the MSE (+ SSIM)
// loss, per-site parameter gradients and the prune removal delta, accumulated per 16x16
// tile in a shared-memory table (accum.cuh): float for API calls, 64-bit fixed point
// (bitwise reproducible) for the trainer.
//
// Semantics follow backends/cuda/src/gradients.cu:103-486 (computeGradientsTiledKernel):
//   * masked pixels (mask <= 0) contribute nothing (the reference returns before its
//     barrier; here they simply carry no keys, so every thread reaches the barrier);
//   * a pixel whose candidates are all invalid contributes nothing;
//   * l2 = 1 / max(l1, 1e-8) in the gradient algebra (gradients.cu:383);
//   * the removal delta of a site is taken once per pixel with the site's summed weight
//     over duplicate slots (gradients.cu:295-350).
//
// Tile mapping: 256 threads = 8 warps, each warp an 8x4 pixel patch, so the lanes of a
// warp share most candidates and register each site with one CAS per warp.
#include "accum.cuh"
#include "common.cuh"
#include "host_common.h"
#include "kernels.h"
#include "sources.cuh"

#include <atomic>
#include <type_traits>

namespace sad {

constexpr int kGradSlots = 512;  // hash slots (and values) of the in-kernel registration table
constexpr float kRemovalSentinel = 1.0e6f;  // removal delta of a pixel the site dominates

__device__ __forceinline__ float luma(const float* __restrict__ p) {
    return __ldg(p) * 0.299f + __ldg(p + 1) * 0.587f + __ldg(p + 2) * 0.114f;
}

// SSIM term of dL/dpred, backends/cuda/src/gradients.cu:258-292 (3x3 window, clamped taps)
__device__ float ssim_dloss(const float* __restrict__ ren, const float* __restrict__ tgt, int x,
                            int y, int w, int h) {
    float mux = 0.f, muy = 0.f, ex2 = 0.f, ey2 = 0.f, exy = 0.f;
    for (int dy = -1; dy <= 1; ++dy) {
        int yy = clampi(y + dy, 0, h - 1);
        for (int dx = -1; dx <= 1; ++dx) {
            int xx = clampi(x + dx, 0, w - 1);
            int i = 3 * (yy * w + xx);
            float xv = luma(ren + i), yv = luma(tgt + i);
            mux += xv;
            muy += yv;
            ex2 += xv * xv;
            ey2 += yv * yv;
            exy += xv * yv;
        }
    }
    const float invn = 0.111111111f;
    mux *= invn; muy *= invn; ex2 *= invn; ey2 *= invn; exy *= invn;
    float sx2 = fmaxf(ex2 - mux * mux, 0.0f);
    float sy2 = fmaxf(ey2 - muy * muy, 0.0f);
    float sxy = exy - mux * muy;
    float A = 2.0f * mux * muy + 0.0001f;
    float B = 2.0f * sxy + 0.0009f;
    float C = mux * mux + muy * muy + 0.0001f;
    float D = sx2 + sy2 + 0.0009f;
    float den = fmaxf(C * D, 1e-8f);
    float num = A * B;
    int p = 3 * (y * w + x);
    float xk = luma(ren + p), yk = luma(tgt + p);
    float dA = 2.0f * muy * invn;
    float dB = 2.0f * (invn * (yk - muy));
    float dC = 2.0f * mux * invn;
    float dD = (2.0f * invn) * (xk - mux);
    return (dA * B + A * dB) / den - num * (dC * D + C * dD) / (den * den);
}

// Global fallback: float SoA arrays (API, accumulated like the reference) or the trainer's
// [N][12] fixed-point records (slot 10 = removal delta, 11 = sentinel count).
template <bool kFix, int NV>
__device__ __forceinline__ void global_add(const GradParams& p, uint32_t key, const float (&v)[NV]) {
    if constexpr (kFix) {
        long long* o = p.fix12 + static_cast<size_t>(key) * 12;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const long long x = to_fix(v[k]);
            if (x != 0) fix_add_global(o + k, x);  // a zero word leaves the sum as it is
        }
    } else {
#pragma unroll
        for (int k = 0; k < 10; ++k) atomicAdd(p.soa[k] + key, v[k]);
        if constexpr (NV > 10) {
            if (v[10] != 0.0f) atomicAdd(p.removal + key, v[10]);
        }
    }
}

template <bool kFix, int NV, class Table>
__device__ __forceinline__ void flush_slot(const GradParams& p, const Table& table, int s) {
    const uint32_t key = table.key_at(s);
    if constexpr (kFix) {
        long long* o = p.fix12 + static_cast<size_t>(key) * 12;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            long long v = table.fixed(k, s);
            if (v != 0) fix_add_global(o + k, v);
        }
    } else {
#pragma unroll
        for (int k = 0; k < 10; ++k) atomicAdd(p.soa[k] + key, table.value(k, s));
        if constexpr (NV > 10) {
            float r = table.value(10, s);
            if (r != 0.0f) atomicAdd(p.removal + key, r);
        }
    }
}

// Values per table slot: 10 gradients, + removal delta (float path), + removal delta and
// count of "keep < 1e-4" pixels (fixed-point path; each such pixel adds the reference's
// 1e6 sentinel, kept as an exact integer count so the fixed-point sum cannot overflow).
template <bool kFix, bool kRemoval>
struct GradLayout {
    static constexpr int NV = kRemoval ? (kFix ? 12 : 11) : 10;
    using Mode = typename std::conditional<kFix, AccSplit, AccFloat>::type;
    using Table = TileTable<NV, kGradSlots, Mode>;
    // precomputed registration (trainer): the tile's values, keys and staged sites, and
    // each thread's candidate weights (and removal deltas) for the accumulation loop
    struct Pre {
        union {
            TileWords<NV> vals;   // lo words per pixel row (narrow tiles) or row parity (wide)
            LaneWords<NV> lanes;  // words per warp lane (tiles of at most kLaneKeys entries)
        };
        uint32_t dkey[kTileKeys];
        // staged site records of the first kNarrowKeys entries (the entries of a wide tile
        // beyond them read their site from global memory)
        float4 g0[kNarrowKeys];  // px, py, tau, radius
        float4 g1[kNarrowKeys];  // dx, dy, l1, l2
        float4 col[kNarrowKeys];  // r, g, b, -
        float wts[kCand][256];
        float rem[kRemoval ? kCand : 1][256];
    };
    static_assert(sizeof(LaneWords<NV>) <= sizeof(TileWords<NV>), "the lane words reuse the tile words' memory");
};

// Forward of one pixel: softmax over the 8 candidates, pred, dL/dpred (+ SSIM term) and,
// with kRemoval, the removal delta on the first slot of each distinct valid site.
// site(i, g, col) supplies candidate i's data.  Semantics of
// backends/cuda/src/gradients.cu:103-300.
template <bool kRemoval, bool kSSIM, class SiteFn>
__device__ __forceinline__ void pixel_forward(const GradParams& prm, int x, int y, float ux,
                                              float uy, float inv_s2, float inv_scale,
                                              const uint32_t (&ids)[kCand], float3 tgt,
                                              SiteFn site, float (&wts)[kCand],
                                              float (&rem)[kCand], uint32_t& valid,
                                              float3& pred, float3& dLdp) {
    const uint32_t n = prm.site_count;
    uint32_t blend = 0;
    float logits[kCand];
    float3 cols[kCand];
    float mx = -INFINITY;
#pragma unroll
    for (int i = 0; i < kCand; ++i) {
        logits[i] = -INFINITY;
        cols[i] = make_float3(0.f, 0.f, 0.f);
        if (ids[i] >= n) continue;
        SiteGeom g;
        site(i, g, cols[i]);
        if (g.px < 0.0f) continue;
        valid |= 1u << i;
        if (g.px >= 0.0f) blend |= 1u << i;
        float tau = g.tau;
        float d = dmix2(g, ux, uy, inv_s2, inv_scale);
        logits[i] = -tau * d;
        mx = fmaxf(mx, logits[i]);
    }
    if (isinf(mx) && mx < 0.0f) {
        valid = 0;
        return;
    }
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
    dLdp = make_float3(2.0f * (pred.x - tgt.x), 2.0f * (pred.y - tgt.y), 2.0f * (pred.z - tgt.z));
    if constexpr (kSSIM) {
        float ds = ssim_dloss(prm.rendered, prm.target, x, y, prm.width, prm.height);
        float k = -prm.ssim_weight * ds;
        dLdp.x += k * 0.299f;
        dLdp.y += k * 0.587f;
        dLdp.z += k * 0.114f;
    }
    if constexpr (kRemoval) {
#pragma unroll
        for (int i = 0; i < kCand; ++i) {
            if (!(valid >> i & 1u)) continue;
            bool first = true;
#pragma unroll
            for (int j = 0; j < i; ++j) first &= !((valid >> j & 1u) && ids[j] == ids[i]);
            if (!first) continue;
            float wt = 0.0f;
#pragma unroll
            for (int j = i; j < kCand; ++j)
                if ((valid >> j & 1u) && ids[j] == ids[i]) wt += wts[j];
            if (!(wt > 0.0f)) continue;
            float keep = 1.0f - wt;
            float delta;
            if (keep < 1e-4f) {
                delta = kRemovalSentinel;
            } else {
                float3 c = cols[i];
                float3 pk = make_float3((pred.x - wt * c.x) / keep, (pred.y - wt * c.y) / keep,
                                        (pred.z - wt * c.z) / keep);
                float3 df = make_float3(pred.x - tgt.x, pred.y - tgt.y, pred.z - tgt.z);
                float3 dk = make_float3(pk.x - tgt.x, pk.y - tgt.y, pk.z - tgt.z);
                delta = (dk.x * dk.x + dk.y * dk.y + dk.z * dk.z) -
                        (df.x * df.x + df.y * df.y + df.z * df.z);
            }
            rem[i] = delta;
        }
    }
}

// The 10 (+ removal) values one candidate adds; the removal slots follow the table mode.
template <bool kFix, int NV>
__device__ __forceinline__ void candidate_values(const SiteGeom& g, float3 col, float ux, float uy,
                                                 float inv_s2, float inv_scale, float w, float3 dLdp,
                                                 float3 pred, float rem, float removal_fix_mul,
                                                 float (&v)[NV]) {
    float o[10];
    candidate_grads(g, col, ux, uy, inv_s2, inv_scale, w, dLdp, pred, true, o);
#pragma unroll
    for (int k = 0; k < 10; ++k) v[k] = o[k];
    if constexpr (NV > 10) {
        if constexpr (kFix) {
            bool sentinel = rem == kRemovalSentinel;
            v[10] = sentinel ? 0.0f : rem * removal_fix_mul;
            v[11] = sentinel ? kFixInvScale : 0.0f;  // adds exactly 1
        } else {
            v[10] = rem;
        }
    }
}

// One 16x16 tile per 256-thread block, each warp an 8x4 pixel patch, so the lanes of a
// warp share most candidates.  Keys are registered here: one CAS per (warp, site).
template <class Src, bool kFix, bool kRemoval, bool kSSIM>
__global__ void __launch_bounds__(256, 3) fused_gradients_kernel(GradParams prm, Src src) {
    using L = GradLayout<kFix, kRemoval>;
    constexpr int NV = L::NV;
    auto& table = shared_table<typename L::Table>();
    const int tid = threadIdx.x;
    table.init(tid, 256);
    __syncthreads();

    const int lane = tid & 31, warp = tid >> 5;
    const int x = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
    const int y = blockIdx.y * 16 + (warp >> 1) * 4 + (lane >> 3);
    const int w = prm.width, h = prm.height;
    const float inv_s2 = prm.inv_scale_sq;
    const float inv_scale = sqrtf(inv_s2);
    const float ux = static_cast<float>(x), uy = static_cast<float>(y);

    uint32_t ids[kCand];
    float wts[kCand];
    float rem[kCand];
    uint32_t valid = 0;
    float3 pred = make_float3(0.f, 0.f, 0.f), dLdp = make_float3(0.f, 0.f, 0.f);
#pragma unroll
    for (int i = 0; i < kCand; ++i) {
        ids[i] = kEmpty;
        wts[i] = 0.0f;
        rem[i] = 0.0f;
    }
    bool live = x < w && y < h;
    const int pix = live ? y * w + x : 0;
    if (live && prm.mask) live = __ldg(prm.mask + pix) > 0.0f;
    if (live) {
        int ci = cand_index_for_pixel(x, y, w, h, prm.cand_width, prm.cand_height);
        uint4 a = __ldg(reinterpret_cast<const uint4*>(prm.cand0) + ci);
        uint4 b = __ldg(reinterpret_cast<const uint4*>(prm.cand1) + ci);
        ids[0] = a.x; ids[1] = a.y; ids[2] = a.z; ids[3] = a.w;
        ids[4] = b.x; ids[5] = b.y; ids[6] = b.z; ids[7] = b.w;
        const float* t = prm.target + 3 * pix;
        float3 tgt = make_float3(__ldg(t), __ldg(t + 1), __ldg(t + 2));
        pixel_forward<kRemoval, kSSIM>(prm, x, y, ux, uy, inv_s2, inv_scale, ids, tgt,
                                       [&](int i, SiteGeom& g, float3& c) { src.load(ids[i], g, c); },
                                       wts, rem, valid, pred, dLdp);
    }

    // 1. registration: one CAS per (warp, site)
    int slots[kCand];
#pragma unroll
    for (int i = 0; i < kCand; ++i)
        slots[i] = register_key(table, (valid >> i & 1u) ? ids[i] : kEmpty);

    // 2. accumulate in a lane-rotated candidate order; the loop is kept rolled (the arrays
    // shift down one entry per step) so the kernel body stays small in the instruction cache
    const uint32_t r = lane_rotation();
    rotate8(ids, r);
    rotate8(wts, r);
    rotate8(slots, r);
    if constexpr (kRemoval) rotate8(rem, r);
    uint32_t vr = rotate_mask8(valid, r);
#pragma unroll 1
    for (int j = 0; j < kCand; ++j) {
        if (vr & 1u) {
            SiteGeom g;
            float3 col;
            src.load(ids[0], g, col);
            float v[NV];
            candidate_values<kFix, NV>(g, col, ux, uy, inv_s2, inv_scale, wts[0], dLdp, pred, rem[0],
                                       prm.removal_fix_mul, v);
            if (slots[0] >= 0)
                table.add(slots[0], v);
            else
                global_add<kFix, NV>(prm, ids[0], v);
        }
        vr >>= 1;
        shift8(ids);
        shift8(wts);
        shift8(slots);
        if constexpr (kRemoval) shift8(rem);
    }
    __syncthreads();
    const int used = table.size();
    for (int d = tid; d < used; d += 256) flush_slot<kFix, NV>(prm, table, d);
}

// Trainer form with the candidate field's registration precomputed (register_tiles_kernel):
// the tile's keys are known before the first pixel is touched, so their values are
// cleared and their sites staged in shared memory in one pass, and the accumulation loop
// reads each candidate's table index, weight and site data by index instead of carrying
// rotated register arrays.
template <class Src, bool kRemoval, bool kSSIM>
__device__ __forceinline__ void grad_pre_tile(const GradParams& prm, const Src& src, int bx, int by, int tiles_x);

template <class Src, bool kRemoval, bool kSSIM>
__global__ void __launch_bounds__(256, 4) fused_gradients_pre_kernel(GradParams prm, Src src) {
    pdl_wait();
    grad_pre_tile<Src, kRemoval, kSSIM>(prm, src, blockIdx.x, blockIdx.y, gridDim.x);
}

// Batched form: one launch over the tiles of up to kBatchLaunchItems images, passed by
// value.  Every thread finds its block's image in the constant bank, and grad_pre_tile
// reads that image's parameters from there.
template <class Src, bool kRemoval, bool kSSIM>
__global__ void __launch_bounds__(256, 4)
    fused_gradients_batch_kernel(const __grid_constant__ BatchArgs<GradBatchItem> a) {
    pdl_wait();
    const uint32_t i = a.item_of(blockIdx.x);
    const GradBatchItem& it = a.items[i];
    const int local = static_cast<int>(blockIdx.x - a.block_prefix[i]);
    grad_pre_tile<Src, kRemoval, kSSIM>(it.p, Src{it.geom, it.color}, local % it.tiles_x, local / it.tiles_x,
                                        it.tiles_x);
}

template <class Src, bool kRemoval, bool kSSIM>
__device__ __forceinline__ void grad_pre_tile(const GradParams& prm, const Src& src, int bx, int by, int tiles_x) {
    using L = GradLayout<true, kRemoval>;
    constexpr int NV = L::NV;
    auto& sm = shared_table<typename L::Pre>();
    const int tid = threadIdx.x;
    const int tile = by * tiles_x + bx;
    const int tile_word = prm.tile_count[tile];
    const bool wide = (tile_word & kTileWideFlag) != 0;  // uniform over the block
    // a narrow tile keeps its first kNarrowKeys entries; slot_of() sends the rest global
    const int used = wide ? tile_word & ~kTileWideFlag : min(tile_word, kNarrowKeys);
    // the lane-word shape (uniform over the block; every shape gives the same sums)
    const bool lanes = !wide && tile_word <= kLaneKeys;
    if (lanes) sm.lanes.zero(used, tid);
    {
        const uint32_t* keys = prm.tile_keys + static_cast<size_t>(tile) * kTileKeys;
        for (int d = tid; d < used; d += 256) {
            const uint32_t key = keys[d];
            sm.dkey[d] = key;
            if (!lanes) sm.vals.zero(d, wide);
            if (d < kNarrowKeys) {
                SiteGeom g;
                float3 c;
                src.load(key, g, c);
                sm.g0[d] = make_float4(g.px, g.py, g.tau, g.radius);
                sm.g1[d] = make_float4(g.dx, g.dy, g.l1, g.l2);
                sm.col[d] = make_float4(c.x, c.y, c.z, 0.0f);
            }
        }
    }
    __syncthreads();

    const int lane = tid & 31, warp = tid >> 5;
    const int x = bx * 16 + (warp & 1) * 8 + (lane & 7);
    const int y = by * 16 + (warp >> 1) * 4 + (lane >> 3);
    const int w = prm.width, h = prm.height;
    const float inv_s2 = prm.inv_scale_sq;
    const float inv_scale = sqrtf(inv_s2);
    const float ux = static_cast<float>(x), uy = static_cast<float>(y);

    // table index of each candidate, 8 x u16 packed in 4 words (0xFFFF: not in the table)
    uint32_t pm[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
    auto slot_of = [&pm, used](int i) {
        uint32_t word = (i >> 1) == 0 ? pm[0] : (i >> 1) == 1 ? pm[1] : (i >> 1) == 2 ? pm[2] : pm[3];
        uint32_t sidx = (word >> ((i & 1) << 4)) & 0xFFFFu;
        return sidx >= static_cast<uint32_t>(used) ? -1 : static_cast<int>(sidx);
    };
    auto site_at = [&](uint32_t id, int slot, SiteGeom& g, float3& c) {
        if (static_cast<unsigned>(slot) < static_cast<unsigned>(kNarrowKeys)) {
            float4 a = sm.g0[slot], b = sm.g1[slot], q = sm.col[slot];
            g.px = a.x; g.py = a.y; g.tau = a.z; g.radius = a.w;
            g.dx = b.x; g.dy = b.y; g.l1 = b.z; g.l2 = b.w;
            c = make_float3(q.x, q.y, q.z);
        } else {
            src.load(id, g, c);  // not staged: read directly
        }
    };

    uint32_t valid = 0;
    float3 pred = make_float3(0.f, 0.f, 0.f), dLdp = make_float3(0.f, 0.f, 0.f);
    bool live = x < w && y < h;
    const int pix = live ? y * w + x : 0;
    int ci = 0;
    if (live && prm.mask) live = __ldg(prm.mask + pix) > 0.0f;
    if (live) {
        uint4 m = __ldg(prm.slot_map + pix);
        pm[0] = m.x; pm[1] = m.y; pm[2] = m.z; pm[3] = m.w;
        ci = cand_index_for_pixel(x, y, w, h, prm.cand_width, prm.cand_height);
        uint32_t ids[kCand];
        uint4 a = __ldg(reinterpret_cast<const uint4*>(prm.cand0) + ci);
        uint4 b = __ldg(reinterpret_cast<const uint4*>(prm.cand1) + ci);
        ids[0] = a.x; ids[1] = a.y; ids[2] = a.z; ids[3] = a.w;
        ids[4] = b.x; ids[5] = b.y; ids[6] = b.z; ids[7] = b.w;
        const float* t = prm.target + 3 * pix;
        float3 tgt = make_float3(__ldg(t), __ldg(t + 1), __ldg(t + 2));
        float wts[kCand], rem[kCand];
#pragma unroll
        for (int i = 0; i < kCand; ++i) {
            wts[i] = 0.0f;
            rem[i] = 0.0f;
        }
        pixel_forward<kRemoval, kSSIM>(prm, x, y, ux, uy, inv_s2, inv_scale, ids, tgt,
                                       [&](int i, SiteGeom& g, float3& c) { site_at(ids[i], slot_of(i), g, c); },
                                       wts, rem, valid, pred, dLdp);
#pragma unroll
        for (int i = 0; i < kCand; ++i) {
            sm.wts[i][tid] = wts[i];
            if constexpr (kRemoval) sm.rem[i][tid] = rem[i];
        }
    }

    // accumulate in a lane-rotated candidate order (spreads the row copies' adds over the
    // banks), or with lane words in the same order in every lane (broadcast record loads)
    const uint32_t r = lanes ? 0u : lane_rotation();
    const int rbits = TileWords<NV>::row_bits(lane >> 3, wide);
#pragma unroll 1
    for (int j = 0; j < kCand; ++j) {
        const int c = static_cast<int>((j + r) & 7u);
        if (!(valid >> c & 1u)) continue;
        const float wt = sm.wts[c][tid];
        const float rv = kRemoval ? sm.rem[kRemoval ? c : 0][tid] : 0.0f;
        // A candidate whose softmax weight underflowed to 0 and that carries no removal
        // term adds only zero words (every parameter term is a product with its weight):
        // skipping it leaves every integer sum unchanged.  Far candidates of the random
        // initial lists are almost all of this kind.
        if (wt == 0.0f && rv == 0.0f) continue;
        const int slot = slot_of(c);
        uint32_t id = kEmpty;
        if (slot < 0)
            id = (c < 4 ? prm.cand0 : prm.cand1)[4 * static_cast<size_t>(ci) + (c & 3)];
        else if (slot >= kNarrowKeys)
            id = sm.dkey[slot];  // a wide tile's entry without a staged site
        SiteGeom g;
        float3 col;
        site_at(id, slot, g, col);
        float v[NV];
        candidate_values<true, NV>(g, col, ux, uy, inv_s2, inv_scale, wt, dLdp, pred, rv, prm.removal_fix_mul, v);
        if (slot < 0)
            global_add<true, NV>(prm, id, v);
        else if (lanes)
            sm.lanes.add(slot, lane, v, prm.fix12, sm.dkey);
        else
            sm.vals.add_unique(slot, TileWords<NV>::block_of(slot, rbits), v);
    }
    __syncthreads();
    if (lanes) {
        sm.lanes.flush(used, tid, prm.fix12, sm.dkey);
        return;
    }
    for (int d = tid; d < used; d += 256) {
        long long* o = prm.fix12 + static_cast<size_t>(sm.dkey[d]) * 12;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const long long x = sm.vals.fixed(k, d, wide);
            if (x != 0) fix_add_global(o + k, x);
        }
    }
}

// Tile registration of a candidate field: the table index of each (pixel, candidate)
// and each tile's key list, with the gradient kernel's tiling (16x16 tiles, 8x4 warp
// patches) and its registration (one CAS per warp and site).  Every candidate id below
// n is registered; inactive sites simply receive no value.
__device__ __forceinline__ void register_tile(const uint4* __restrict__ c0, const uint4* __restrict__ c1,
                                              uint32_t n, int w, int h, int cw, int ch, const TileMap& map,
                                              int bx, int by, int tiles_x);

__global__ void __launch_bounds__(256) register_tiles_kernel(const uint4* __restrict__ c0,
                                                             const uint4* __restrict__ c1, uint32_t n,
                                                             int w, int h, int cw, int ch, TileMap map) {
    pdl_wait();
    register_tile(c0, c1, n, w, h, cw, ch, map, blockIdx.x, blockIdx.y, gridDim.x);
}

// Batched form over the tiles of up to kBatchLaunchItems images (by value, as the gradient
// kernel's); one thread copies the block's image into shared memory, which measured faster
// here than constant-bank reads.
__global__ void __launch_bounds__(256) register_tiles_batch_kernel(const __grid_constant__ BatchArgs<RegisterBatchItem> a) {
    pdl_wait();
    __shared__ RegisterBatchItem s_it;
    __shared__ int s_local;
    if (threadIdx.x == 0) {
        const uint32_t i = a.item_of(blockIdx.x);
        s_it = a.items[i];
        s_local = static_cast<int>(blockIdx.x - a.block_prefix[i]);
    }
    __syncthreads();
    const int tx = s_it.tiles_x;
    register_tile(reinterpret_cast<const uint4*>(s_it.c0), reinterpret_cast<const uint4*>(s_it.c1), s_it.n, s_it.w,
                  s_it.h, s_it.cw, s_it.ch, s_it.map, s_local % tx, s_local / tx, tx);
}

__device__ __forceinline__ void register_tile(const uint4* __restrict__ c0, const uint4* __restrict__ c1,
                                              uint32_t n, int w, int h, int cw, int ch, const TileMap& map,
                                              int bx, int by, int tiles_x) {
    __shared__ KeyTable<512> table;
    __shared__ int s_far;  // the tile's references to far entries
    const int tid = threadIdx.x;
    table.init_keys(tid, 256);
    if (tid == 0) s_far = 0;
    __syncthreads();
    const int lane = tid & 31, warp = tid >> 5;
    const int x = bx * 16 + (warp & 1) * 8 + (lane & 7);
    const int y = by * 16 + (warp >> 1) * 4 + (lane >> 3);
    const bool inside = x < w && y < h;
    uint32_t ids[kCand];
    if (inside) {
        int ci = cand_index_for_pixel(x, y, w, h, cw, ch);
        uint4 a = __ldg(c0 + ci), b = __ldg(c1 + ci);
        ids[0] = a.x; ids[1] = a.y; ids[2] = a.z; ids[3] = a.w;
        ids[4] = b.x; ids[5] = b.y; ids[6] = b.z; ids[7] = b.w;
    } else {
#pragma unroll
        for (int i = 0; i < kCand; ++i) ids[i] = kEmpty;
    }
    const int far = __reduce_add_sync(0xffffffffu, register_tile_pixel(table, ids, n, x, y, w, inside, map));
    if (lane == 0 && far != 0) atomicAdd(&s_far, far);
    __syncthreads();
    const int rule = map.wide_far_refs ? *map.wide_far_refs : kWideFarRefs;
    write_tile_keys(table, tid, by * tiles_x + bx, s_far, rule, map);
}

size_t tile_map_words(int w, int h) {
    size_t tiles = static_cast<size_t>((w + 15) / 16) * ((h + 15) / 16);
    return static_cast<size_t>(w) * h * 4 + tiles * kTileKeys + tiles;
}

TileMap tile_map_at(uint32_t* base, int w, int h) {
    size_t tiles = static_cast<size_t>((w + 15) / 16) * ((h + 15) / 16);
    TileMap m;
    m.slot_map = reinterpret_cast<uint4*>(base);
    m.tile_keys = base + static_cast<size_t>(w) * h * 4;
    m.tile_count = reinterpret_cast<int*>(m.tile_keys + tiles * kTileKeys);
    m.wide_far_refs = nullptr;
    return m;
}

void launch_register_tiles(const uint32_t* c0, const uint32_t* c1, uint32_t n, int w, int h,
                           int cw, int ch, const TileMap& map, cudaStream_t st) {
    dim3 grid((w + 15) / 16, (h + 15) / 16);
    launch_pdl(register_tiles_kernel, grid, dim3(256), 0, st, reinterpret_cast<const uint4*>(c0),
               reinterpret_cast<const uint4*>(c1), n, w, h, cw, ch, map);
    note_launches(1);
}

void launch_register_tiles_batch(const RegisterBatchItem* items, const uint32_t* tile_prefix, uint32_t n_items,
                                 cudaStream_t st) {
    for_each_batch_launch(items, tile_prefix, n_items, [&](const BatchArgs<RegisterBatchItem>& a, uint32_t tiles) {
        launch_pdl(register_tiles_batch_kernel, dim3(tiles), dim3(256), 0, st, a);
        note_launches(1);
    });
}

template <class Src, bool kFix, bool kRemoval, bool kSSIM>
static void launch_fused(const GradParams& p, Src src, cudaStream_t st) {
    dim3 grid((p.width + 15) / 16, (p.height + 15) / 16);
    if constexpr (kFix) {
        if (p.slot_map) {
            launch_pdl(fused_gradients_pre_kernel<Src, kRemoval, kSSIM>, grid, dim3(256),
                       sizeof(typename GradLayout<true, kRemoval>::Pre), st, p, src);
            return;
        }
    }
    fused_gradients_kernel<Src, kFix, kRemoval, kSSIM>
        <<<grid, 256, sizeof(typename GradLayout<kFix, kRemoval>::Table), st>>>(p, src);
}

cudaError_t prepare_gradient_kernels();

// Opt-in of the >48 KB shared-memory launches, once per device (an attribute set, not a
// stream operation).
static void ensure_gradient_kernels() {
    static std::atomic<unsigned long long> done{0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return;
    unsigned long long bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return;
    if (prepare_gradient_kernels() == cudaSuccess) done.fetch_or(bit, std::memory_order_release);
}

template <class Src, bool kFix>
static void dispatch_gradients(const GradParams& p, Src src, cudaStream_t st) {
    ensure_gradient_kernels();
    bool rem = p.compute_removal != 0;
    bool ssim = p.ssim_weight > 0.0f;
    if (rem && ssim)
        launch_fused<Src, kFix, true, true>(p, src, st);
    else if (rem)
        launch_fused<Src, kFix, true, false>(p, src, st);
    else if (ssim)
        launch_fused<Src, kFix, false, true>(p, src, st);
    else
        launch_fused<Src, kFix, false, false>(p, src, st);
    note_launches(1);
}

template <class Src, bool kFix, bool kRemoval>
static cudaError_t allow_variant() {
    size_t smem = sizeof(typename GradLayout<kFix, kRemoval>::Table);
    cudaError_t e = allow_dynamic_smem(fused_gradients_kernel<Src, kFix, kRemoval, false>, smem);
    if (e == cudaSuccess) e = allow_dynamic_smem(fused_gradients_kernel<Src, kFix, kRemoval, true>, smem);
    if constexpr (kFix) {
        size_t pre = sizeof(typename GradLayout<true, kRemoval>::Pre);
        if (e == cudaSuccess) e = allow_dynamic_smem(fused_gradients_pre_kernel<Src, kRemoval, false>, pre);
        if (e == cudaSuccess) e = allow_dynamic_smem(fused_gradients_pre_kernel<Src, kRemoval, true>, pre);
        if constexpr (std::is_same<Src, PreparedSites>::value) {
            if (e == cudaSuccess) e = allow_dynamic_smem(fused_gradients_batch_kernel<Src, kRemoval, false>, pre);
            if (e == cudaSuccess) e = allow_dynamic_smem(fused_gradients_batch_kernel<Src, kRemoval, true>, pre);
        }
    }
    return e;
}

cudaError_t prepare_gradient_kernels() {
    cudaError_t e = allow_variant<RawSites, false, true>();
    if (e == cudaSuccess) e = allow_variant<PreparedSites, false, true>();
    if (e == cudaSuccess) e = allow_variant<PreparedSites, true, false>();
    if (e == cudaSuccess) e = allow_variant<PreparedSites, true, true>();
    return e;
}

void launch_gradients_raw(const GradParams& p, const Site* sites, cudaStream_t st) {
    dispatch_gradients<RawSites, false>(p, RawSites{sites}, st);
}

void launch_gradients_prepared(const GradParams& p, const SiteGeom* geom, const SiteColor* color,
                               cudaStream_t st) {
    if (p.fix12)
        dispatch_gradients<PreparedSites, true>(p, PreparedSites{geom, color}, st);
    else
        dispatch_gradients<PreparedSites, false>(p, PreparedSites{geom, color}, st);
}

template <bool kRemoval, bool kSSIM>
static void launch_batch_variant(const BatchArgs<GradBatchItem>& a, uint32_t tiles, cudaStream_t st) {
    launch_pdl(fused_gradients_batch_kernel<PreparedSites, kRemoval, kSSIM>, dim3(tiles), dim3(256),
               sizeof(typename GradLayout<true, kRemoval>::Pre), st, a);
}

void launch_gradients_batch(const GradBatchItem* items, const uint32_t* tile_prefix, uint32_t n_items,
                            bool removal, bool ssim, cudaStream_t st) {
    ensure_gradient_kernels();
    for_each_batch_launch(items, tile_prefix, n_items, [&](const BatchArgs<GradBatchItem>& a, uint32_t tiles) {
        if (removal && ssim)
            launch_batch_variant<true, true>(a, tiles, st);
        else if (removal)
            launch_batch_variant<true, false>(a, tiles, st);
        else if (ssim)
            launch_batch_variant<false, true>(a, tiles, st);
        else
            launch_batch_variant<false, false>(a, tiles, st);
        note_launches(1);
    });
}

}  // namespace sad

using namespace sad;

extern "C" sad_status_t sad_compute_gradients_tiled(
    const uint32_t* cand0, const uint32_t* cand1, const float* target, const float* rendered,
    const float* mask, float* grad_pos_x, float* grad_pos_y, float* grad_log_tau,
    float* grad_radius, float* grad_color_r, float* grad_color_g, float* grad_color_b,
    float* grad_dir_x, float* grad_dir_y, float* grad_log_aniso, const float* sites,
    float inv_scale_sq, uint32_t site_count, float* removal_delta, uint32_t compute_removal,
    float ssim_weight, int width, int height, int cand_width, int cand_height,
    sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_compute_gradients_tiled: invalid image size");
    SAD_REQUIRE(image_size_ok(cand_width, cand_height), "sad_compute_gradients_tiled: invalid cand size");
    SAD_REQUIRE(cand0 && cand1 && target, "sad_compute_gradients_tiled: null input");
    SAD_REQUIRE(ssim_weight <= 0.0f || rendered, "sad_compute_gradients_tiled: SSIM needs rendered");
    SAD_REQUIRE(grad_pos_x && grad_pos_y && grad_log_tau && grad_radius && grad_color_r &&
                    grad_color_g && grad_color_b && grad_dir_x && grad_dir_y && grad_log_aniso,
                "sad_compute_gradients_tiled: null gradient array");
    SAD_REQUIRE(!compute_removal || removal_delta, "sad_compute_gradients_tiled: null removal_delta");
    SAD_REQUIRE(sites || site_count == 0, "sad_compute_gradients_tiled: null sites");
    GradParams p{};
    p.cand0 = cand0;
    p.cand1 = cand1;
    p.target = target;
    p.rendered = rendered;
    p.mask = mask;
    p.inv_scale_sq = inv_scale_sq;
    p.site_count = site_count;
    p.ssim_weight = ssim_weight;
    p.width = width;
    p.height = height;
    p.cand_width = cand_width;
    p.cand_height = cand_height;
    float* g[10] = {grad_pos_x, grad_pos_y, grad_log_tau, grad_radius, grad_color_r,
                    grad_color_g, grad_color_b, grad_dir_x, grad_dir_y, grad_log_aniso};
    for (int k = 0; k < 10; ++k) p.soa[k] = g[k];
    p.removal = removal_delta;
    p.fix12 = nullptr;
    p.compute_removal = compute_removal ? 1 : 0;
    launch_gradients_raw(p, reinterpret_cast<const Site*>(sites), as_stream(stream));
    return check_launch("sad_compute_gradients_tiled");
}

extern "C" size_t sad_compute_gradients_fixed_scratch_bytes(uint32_t site_count, int width, int height) {
    if (!image_size_ok(width, height)) return 0;
    auto a256 = [](size_t x) { return (x + 255) & ~size_t(255); };
    return 256 + a256(size_t(site_count) * sizeof(SiteGeom)) + a256(size_t(site_count) * sizeof(SiteColor)) +
           a256(tile_map_words(width, height) * sizeof(uint32_t));
}

extern "C" sad_status_t sad_compute_gradients_fixed(
    const uint32_t* cand0, const uint32_t* cand1, const float* target, const float* rendered,
    const float* mask, const float* sites, float inv_scale_sq, uint32_t site_count,
    uint32_t compute_removal, float ssim_weight, int width, int height, int cand_width,
    int cand_height, long long* fix12_out, float* removal_scale_out, void* scratch,
    size_t scratch_bytes, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_compute_gradients_fixed: invalid image size");
    SAD_REQUIRE(image_size_ok(cand_width, cand_height), "sad_compute_gradients_fixed: invalid cand size");
    SAD_REQUIRE(cand0 && cand1 && target && fix12_out, "sad_compute_gradients_fixed: null input");
    SAD_REQUIRE(ssim_weight <= 0.0f || rendered, "sad_compute_gradients_fixed: SSIM needs rendered");
    SAD_REQUIRE(sites || site_count == 0, "sad_compute_gradients_fixed: null sites");
    SAD_REQUIRE(scratch && scratch_bytes >= sad_compute_gradients_fixed_scratch_bytes(site_count, width, height),
                "sad_compute_gradients_fixed: scratch too small");
    const float scale = removal_fix_mul(width, height);
    if (removal_scale_out) *removal_scale_out = scale;
    cudaStream_t st = as_stream(stream);
    auto a256 = [](size_t x) { return (x + 255) & ~size_t(255); };
    char* p = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(scratch) + 255) & ~uintptr_t(255));
    SiteGeom* geom = reinterpret_cast<SiteGeom*>(p);
    p += a256(size_t(site_count) * sizeof(SiteGeom));
    SiteColor* color = reinterpret_cast<SiteColor*>(p);
    p += a256(size_t(site_count) * sizeof(SiteColor));
    TileMap map = tile_map_at(reinterpret_cast<uint32_t*>(p), width, height);
    launch_prepare_sites(reinterpret_cast<const Site*>(sites), geom, color, site_count, st);
    launch_register_tiles(cand0, cand1, site_count, width, height, cand_width, cand_height, map, st);
    GradParams g{};
    g.cand0 = cand0;
    g.cand1 = cand1;
    g.target = target;
    g.rendered = rendered;
    g.mask = mask;
    g.inv_scale_sq = inv_scale_sq;
    g.site_count = site_count;
    g.ssim_weight = ssim_weight;
    g.width = width;
    g.height = height;
    g.cand_width = cand_width;
    g.cand_height = cand_height;
    g.fix12 = fix12_out;
    g.removal_fix_mul = scale;
    g.compute_removal = compute_removal ? 1 : 0;
    g.slot_map = map.slot_map;
    g.tile_keys = map.tile_keys;
    g.tile_count = map.tile_count;
    launch_gradients_prepared(g, geom, color, st);
    return check_launch("sad_compute_gradients_fixed");
}
