// topology.cu -- site-set changes and per-site statistics: densify/prune scoring, index
// selection, prune, split, site statistics, Hilbert ordering, quality metrics and the
// gradient-weighted initialisation.
#include "accum.cuh"
#include "common.cuh"
#include "host_common.h"
#include "kernels.h"

#include <cmath>
#include <type_traits>
#include "sources.cuh"

#include <vector>

namespace sad {

// ---------------------------------------------------------------------------
// score pairs (backends/cuda/src/densify_prune.cu:223-281)
// ---------------------------------------------------------------------------
__global__ void densify_pairs_kernel(const Site* __restrict__ sites, const float* __restrict__ mass,
                                     const float* __restrict__ energy, uint2* __restrict__ pairs,
                                     uint32_t n, float min_mass, float alpha, uint32_t pc) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pc) return;
    uint2 o = make_uint2(kEmpty, kEmpty);
    if (i < n) {
        float m = mass[i], e = energy[i];
        bool active = sites[i].px >= 0.0f;
        if (active && m > min_mass && isfinite(e)) {
            float den = powf(fmaxf(m, 1e-8f), alpha);
            float score = fmaxf(e, 0.0f) / den;
            o = make_uint2(0xFFFFFFFFu - __float_as_uint(score), i);
        }
    }
    pairs[i] = o;
}

void launch_densify_pairs(const Site* sites, const float* mass, const float* energy,
                          uint32_t* pairs, uint32_t n, float min_mass, float alpha,
                          uint32_t pair_count, cudaStream_t st) {
    if (pair_count == 0) return;
    densify_pairs_kernel<<<blocks_for(pair_count, 256), 256, 0, st>>>(
        sites, mass, energy, reinterpret_cast<uint2*>(pairs), n, min_mass, alpha, pair_count);
    note_launches(1);
}

// removal values are read with a stride (12 inside the trainer's gradient records, where
// the slot is cleared after reading so the next prune iteration starts from zero)
__global__ void prune_pairs_kernel(const Site* __restrict__ sites, float* __restrict__ removal,
                                   int stride, int clear, uint2* __restrict__ pairs, uint32_t n,
                                   float delta_norm, uint32_t pc) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pc) return;
    uint2 o = make_uint2(kEmpty, kEmpty);
    if (i < n) {
        bool active = sites[i].px >= 0.0f;
        float* r = removal + static_cast<size_t>(i) * stride;
        float delta = *r * delta_norm;
        if (clear) *r = 0.0f;
        if (active && isfinite(delta)) o = make_uint2(__float_as_uint(fmaxf(delta, 0.0f)), i);
    }
    pairs[i] = o;
}

void launch_prune_pairs(const Site* sites, const float* removal, int removal_stride,
                        uint32_t* pairs, uint32_t n, float delta_norm, uint32_t pair_count,
                        cudaStream_t st) {
    if (pair_count == 0) return;
    prune_pairs_kernel<<<blocks_for(pair_count, 256), 256, 0, st>>>(
        sites, const_cast<float*>(removal), removal_stride, removal_stride != 1,
        reinterpret_cast<uint2*>(pairs), n, delta_norm, pair_count);
    note_launches(1);
}

__global__ void prune_pairs_fixed_kernel(const Site* __restrict__ sites, long long* __restrict__ fix12,
                                         float inv_mul, uint2* __restrict__ pairs, uint32_t n,
                                         float delta_norm, uint32_t pc) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pc) return;
    uint2 o = make_uint2(kEmpty, kEmpty);
    if (i < n) {
        bool active = sites[i].px >= 0.0f;
        longlong2* r = reinterpret_cast<longlong2*>(fix12 + static_cast<size_t>(i) * 12 + 10);
        longlong2 v = *r;
        *r = make_longlong2(0, 0);
        float removal = static_cast<float>(v.y) * 1.0e6f + from_fix(v.x) * inv_mul;
        float delta = removal * delta_norm;
        if (active && isfinite(delta)) o = make_uint2(__float_as_uint(fmaxf(delta, 0.0f)), i);
    }
    pairs[i] = o;
}

// Trainer form over the compacted active list (grid-stride; any grid size is correct):
// pair j is (key, alive[j]) for the n_alive listed sites (the same sorted prefix as pairs over every slot, where inactive
// slots key 0xFFFFFFFF), and their removal records are consumed.
__global__ void prune_pairs_alive_kernel(long long* __restrict__ fix12, float inv_mul,
                                         uint2* __restrict__ pairs, const uint32_t* __restrict__ alive,
                                         const DevState* __restrict__ state, float delta_norm) {
    pdl_wait();
    const uint32_t n_alive = state->n_alive;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_alive; j += gridDim.x * blockDim.x) {
        const uint32_t i = alive[j];
        longlong2* r = reinterpret_cast<longlong2*>(fix12 + static_cast<size_t>(i) * 12 + 10);
        longlong2 v = *r;
        *r = make_longlong2(0, 0);
        float removal = static_cast<float>(v.y) * 1.0e6f + from_fix(v.x) * inv_mul;
        float delta = removal * delta_norm;
        pairs[j] = isfinite(delta) ? make_uint2(__float_as_uint(fmaxf(delta, 0.0f)), i)
                                   : make_uint2(kEmpty, kEmpty);
    }
}

__global__ void __launch_bounds__(256) prune_pairs_batch_kernel(const SiteBatchItem* __restrict__ items,
                                                                const uint32_t* __restrict__ prefix,
                                                                uint32_t n_items) {
    pdl_wait();
    __shared__ uint32_t s_prefix[kMaxBatchItems + 1];
    const uint32_t total = load_site_prefix(s_prefix, prefix, n_items);
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const uint32_t k = batch_item_of(s_prefix, n_items, g);
        const SiteBatchItem& it = items[k];
        const uint32_t j = g - s_prefix[k];
        const uint32_t i = it.alive[j];
        longlong2* r = reinterpret_cast<longlong2*>(it.grads + static_cast<size_t>(i) * 12 + 10);
        longlong2 v = *r;
        *r = make_longlong2(0, 0);
        float removal = static_cast<float>(v.y) * 1.0e6f + from_fix(v.x) * it.removal_inv_mul;
        float delta = removal * it.delta_norm;
        reinterpret_cast<uint2*>(it.pairs)[j] = isfinite(delta) ? make_uint2(__float_as_uint(fmaxf(delta, 0.0f)), i)
                                                                : make_uint2(kEmpty, kEmpty);
    }
}

void launch_prune_pairs_batch(const SiteBatchItem* items, const uint32_t* site_prefix, uint32_t n_items,
                              uint32_t grid_threads, cudaStream_t st) {
    launch_pdl(prune_pairs_batch_kernel, dim3(std::max(1u, blocks_for(grid_threads, 256))), dim3(256), 0, st, items,
               site_prefix, n_items);
    note_launches(1);
}

void launch_prune_pairs_alive(long long* fix12, float fix_mul, uint32_t* pairs, const uint32_t* alive,
                              const DevState* state, uint32_t max_alive, float delta_norm, cudaStream_t st) {
    if (max_alive == 0) return;
    launch_pdl(prune_pairs_alive_kernel, dim3(blocks_for(max_alive, 256)), dim3(256), 0, st, fix12,
               1.0f / fix_mul, reinterpret_cast<uint2*>(pairs), alive, state, delta_norm);
    note_launches(1);
}

void launch_prune_pairs_fixed(const Site* sites, long long* fix12, float fix_mul, uint32_t* pairs,
                              uint32_t n, float delta_norm, uint32_t pair_count, cudaStream_t st) {
    if (pair_count == 0) return;
    prune_pairs_fixed_kernel<<<blocks_for(pair_count, 256), 256, 0, st>>>(
        sites, fix12, 1.0f / fix_mul, reinterpret_cast<uint2*>(pairs), n, delta_norm, pair_count);
    note_launches(1);
}

__global__ void write_indices_kernel(const uint2* __restrict__ pairs, uint32_t* __restrict__ idx,
                                     uint32_t k) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < k) idx[i] = pairs[i].y;
}

void launch_write_indices(const uint32_t* pairs, uint32_t* idx, uint32_t k, cudaStream_t st) {
    if (k == 0) return;
    write_indices_kernel<<<blocks_for(k, 256), 256, 0, st>>>(reinterpret_cast<const uint2*>(pairs),
                                                             idx, k);
    note_launches(1);
}

__global__ void prune_by_index_kernel(Site* __restrict__ sites, const uint32_t* __restrict__ idx,
                                      uint32_t k) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k) return;
    uint32_t s = idx[i];
    if (s == kEmpty) return;
    sites[s].px = -1.0f;
    sites[s].py = -1.0f;
}

void launch_prune_by_index(Site* sites, const uint32_t* idx, uint32_t k, cudaStream_t st) {
    if (k == 0) return;
    prune_by_index_kernel<<<blocks_for(k, 256), 256, 0, st>>>(sites, idx, k);
    note_launches(1);
}

// Trainer form: write-indices + prune fused; the count comes from the host-planned
// per-iteration table (the schedule is fixed before the fit starts).
// The pruned sites are marked inactive in the site records, the prepared geometry and
// the VPT geometry (the refresh repacks only listed sites).
__global__ void prune_sorted_kernel(Site* __restrict__ sites, SiteGeom* __restrict__ geom,
                                    SiteGeom* __restrict__ vgeom, const uint2* __restrict__ pairs,
                                    const uint32_t* __restrict__ prune_k,
                                    const DevState* __restrict__ state) {
    pdl_wait();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t k = prune_k[state->iter];
    if (i >= k) return;
    uint32_t s = pairs[i].y;
    if (s == kEmpty) return;
    sites[s].px = -1.0f;
    sites[s].py = -1.0f;
    geom[s].px = -1.0f;
    geom[s].py = -1.0f;
    vgeom[s].px = -1.0f;
    vgeom[s].py = -1.0f;
}

// Batched form: blockIdx.y is the image; each marks the first prune_k[iter] of its pairs.
__global__ void prune_sorted_batch_kernel(const SiteBatchItem* __restrict__ items) {
    pdl_wait();
    const SiteBatchItem& it = items[blockIdx.y];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t k = it.prune_k[it.state->iter];
    if (i >= k) return;
    const uint32_t s = reinterpret_cast<const uint2*>(it.pairs)[i].y;
    if (s == kEmpty) return;
    it.sites[s].px = -1.0f;
    it.sites[s].py = -1.0f;
    it.geom[s].px = -1.0f;
    it.geom[s].py = -1.0f;
    it.vgeom[s].px = -1.0f;
    it.vgeom[s].py = -1.0f;
}

void launch_prune_sorted_batch(const SiteBatchItem* items, uint32_t n_items, uint32_t max_k, cudaStream_t st) {
    if (max_k == 0 || n_items == 0) return;
    launch_pdl(prune_sorted_batch_kernel, dim3(blocks_for(max_k, 256), n_items), dim3(256), 0, st, items);
    note_launches(1);
}

void launch_prune_sorted_train(Site* sites, SiteGeom* geom, SiteGeom* vgeom, const uint32_t* pairs,
                               const uint32_t* prune_k, const DevState* state, uint32_t max_k,
                               cudaStream_t st) {
    if (max_k == 0) return;
    launch_pdl(prune_sorted_kernel, dim3(blocks_for(max_k, 256)), dim3(256), 0, st, sites, geom, vgeom,
               reinterpret_cast<const uint2*>(pairs), prune_k, state);
    note_launches(1);
}

// ---------------------------------------------------------------------------
// split (backends/cuda/src/densify_prune.cu:86-220)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float lum_at(const float* __restrict__ t, int w, int h, int x, int y) {
    x = clampi(x, 0, w - 1);
    y = clampi(y, 0, h - 1);
    const float* p = t + 3 * (y * w + x);
    return 0.299f * p[0] + 0.587f * p[1] + 0.114f * p[2];
}

struct SplitStats {
    const float* mass;
    const float* ew;
    const float* ewx;
    const float* ewy;
    const float* ewxx;
    const float* ewxy;
    const float* ewyy;
};

__global__ void split_kernel(Site* __restrict__ sites, float* __restrict__ adam,
                             const uint32_t* __restrict__ split_idx, uint32_t num, SplitStats st,
                             uint32_t cur, const float* __restrict__ target, int w, int h) {
    uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= num) return;
    uint32_t pi = split_idx[gid];
    Site par = sites[pi];
    if (par.px < 0.0f) return;
    float ew = st.ew[pi];
    float ax = par.dx, ay = par.dy, cx = par.px, cy = par.py;
    float la = par.log_aniso * 0.8f;
    if (ew > 1e-3f) {
        float mx = st.ewx[pi] / ew, my = st.ewy[pi] / ew;
        cx = 0.4f * par.px + 0.6f * mx;
        cy = 0.4f * par.py + 0.6f * my;
        float exx = st.ewxx[pi] / ew - mx * mx;
        float exy = st.ewxy[pi] / ew - mx * my;
        float eyy = st.ewyy[pi] / ew - my * my;
        exx = fmaxf(exx, 1e-4f);
        eyy = fmaxf(eyy, 1e-4f);
        float th = 0.5f * atan2f(2.0f * exy, exx - eyy);
        ax = cosf(th);
        ay = sinf(th);
        float tr = exx + eyy;
        float disc = sqrtf(fmaxf(0.0f, 0.25f * (exx - eyy) * (exx - eyy) + exy * exy));
        float l1 = fmaxf(1e-4f, 0.5f * tr + disc);
        float l2 = fmaxf(1e-4f, 0.5f * tr - disc);
        la = clampf(-0.5f * logf(l1 / l2), -2.0f, 2.0f);
    } else {
        int ix = clampi(static_cast<int>(par.px), 0, w - 1);
        int iy = clampi(static_cast<int>(par.py), 0, h - 1);
        float TL = lum_at(target, w, h, ix - 1, iy - 1), T = lum_at(target, w, h, ix, iy - 1),
              TR = lum_at(target, w, h, ix + 1, iy - 1);
        float L = lum_at(target, w, h, ix - 1, iy), R = lum_at(target, w, h, ix + 1, iy);
        float BL = lum_at(target, w, h, ix - 1, iy + 1), B = lum_at(target, w, h, ix, iy + 1),
              BR = lum_at(target, w, h, ix + 1, iy + 1);
        float gx = (-TL + TR - 2.0f * L + 2.0f * R - BL + BR) / 4.0f;
        float gy = (-TL - 2.0f * T - TR + BL + 2.0f * B + BR) / 4.0f;
        float g2 = gx * gx + gy * gy;
        if (g2 > 1e-8f) {
            float len = sqrtf(gx * gx + gy * gy);
            if (len > 1e-8f) {
                ax = gx / len;
                ay = gy / len;
            } else {
                ax = 1.0f;
                ay = 0.0f;
            }
        }
    }
    float m = fmaxf(st.mass[pi], 1.0f);
    float od = clampf(sqrtf(m) * 0.5f, 1.5f, 48.0f);
    float ox = ax * od, oy = ay * od;
    float pax = clampf(cx + ox, 0.0f, static_cast<float>(w - 1));
    float pay = clampf(cy + oy, 0.0f, static_cast<float>(h - 1));
    float pbx = clampf(cx - ox, 0.0f, static_cast<float>(w - 1));
    float pby = clampf(cy - oy, 0.0f, static_cast<float>(h - 1));
    const float* ca = target + 3 * (static_cast<int>(pay) * w + static_cast<int>(pax));
    const float* cb = target + 3 * (static_cast<int>(pby) * w + static_cast<int>(pbx));
    uint32_t ci = cur + gid;
    if (ci == pi) return;
    Site c0 = par, c1 = par;
    c0.px = pax; c0.py = pay;
    c1.px = pbx; c1.py = pby;
    c0.r = ca[0]; c0.g = ca[1]; c0.b = ca[2];
    c1.r = cb[0]; c1.g = cb[1]; c1.b = cb[2];
    c0.log_tau = par.log_tau - 0.25f;
    c1.log_tau = par.log_tau - 0.25f;
    c0.radius = par.radius * 0.85f;
    c1.radius = par.radius * 0.85f;
    c0.dx = ax; c0.dy = ay; c1.dx = ax; c1.dy = ay;
    c0.log_aniso = la;
    c1.log_aniso = la;
    sites[pi] = c0;
    sites[ci] = c1;
    float4* a0 = reinterpret_cast<float4*>(adam + static_cast<size_t>(pi) * 20);
    float4* a1 = reinterpret_cast<float4*>(adam + static_cast<size_t>(ci) * 20);
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        a0[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        a1[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

void launch_split(Site* sites, float* adam, const uint32_t* split_idx, uint32_t num,
                  const float* const stats[7], uint32_t cur, const float* target, int w, int h,
                  cudaStream_t st) {
    if (num == 0) return;
    SplitStats s{stats[0], stats[1], stats[2], stats[3], stats[4], stats[5], stats[6]};
    split_kernel<<<blocks_for(num, 256), 256, 0, st>>>(sites, adam, split_idx, num, s, cur, target,
                                                       w, h);
    note_launches(1);
}

// ---------------------------------------------------------------------------
// site statistics (backends/cuda/src/utils.cu:106-231)
// ---------------------------------------------------------------------------
struct StatOut {
    float* o[8];       // float path: accumulate into caller arrays
    long long* fix;    // fixed-point path: [8][stride] records, 2^32 * mul[k] units
    size_t stride;
    float mul[8];      // per-statistic pre-scale (power of two <= 1), sized to the image
};

constexpr int kStatSlots = 512;

template <bool kFix>
__global__ void __launch_bounds__(256) site_stats_kernel(const uint4* __restrict__ c0,
                                                         const uint4* __restrict__ c1,
                                                         const float* __restrict__ target,
                                                         const float* __restrict__ mask,
                                                         RawSites src, float inv_s2, uint32_t n,
                                                         StatOut out, int w, int h, int cw,
                                                         int ch) {
    using Table = TileTable<8, kStatSlots, typename std::conditional<kFix, AccSplit, AccFloat>::type>;
    auto& table = shared_table<Table>();
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    table.init(tid, 256);
    __syncthreads();

    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    bool live = x < w && y < h;
    int p = live ? y * w + x : 0;
    if (live && mask) live = mask[p] > 0.0f;
    float ux = static_cast<float>(x), uy = static_cast<float>(y);
    float inv_scale = sqrtf(inv_s2);
    uint32_t ids[kCand];
    float wts[kCand];
    uint32_t valid = 0, blend = 0;
    float err = 0.0f;
#pragma unroll
    for (int i = 0; i < kCand; ++i) {
        ids[i] = kEmpty;
        wts[i] = 0.0f;
    }
    if (live) {
        int ci = cand_index_for_pixel(x, y, w, h, cw, ch);
        uint4 a = __ldg(c0 + ci), b = __ldg(c1 + ci);
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
        if (isinf(mx) && mx < 0.0f) {
            valid = 0;
        } else {
            float sum = 0.0f;
#pragma unroll
            for (int i = 0; i < kCand; ++i) {
                wts[i] = expf(logits[i] - mx);
                sum += wts[i];
            }
            float inv = 1.0f / fmaxf(sum, 1e-8f);
            float3 pr = make_float3(0.f, 0.f, 0.f);
#pragma unroll
            for (int i = 0; i < kCand; ++i) {
                wts[i] *= inv;
                if (blend >> i & 1u) {
                    pr.x += wts[i] * cols[i].x;
                    pr.y += wts[i] * cols[i].y;
                    pr.z += wts[i] * cols[i].z;
                }
            }
            const float* t = target + 3 * p;
            float d0 = pr.x - t[0], d1 = pr.y - t[1], d2 = pr.z - t[2];
            err = d0 * d0 + d1 * d1 + d2 * d2;
        }
    }
    // unique valid sites of the pixel, each with its weight summed over duplicate slots
    float wsum[kCand];
    uint32_t uniq = 0;
#pragma unroll
    for (int i = 0; i < kCand; ++i) {
        bool first = (valid >> i & 1u) != 0u;
#pragma unroll
        for (int j = 0; j < i; ++j) first &= !((valid >> j & 1u) && ids[j] == ids[i]);
        float wt = 0.0f;
        if (first) {
#pragma unroll
            for (int j = i; j < kCand; ++j)
                if ((valid >> j & 1u) && ids[j] == ids[i]) wt += wts[j];
        }
        wsum[i] = wt;
        if (first && wt > 0.0f) uniq |= 1u << i;
    }
    int slots[kCand];
#pragma unroll
    for (int i = 0; i < kCand; ++i)
        slots[i] = register_key(table, (uniq >> i & 1u) ? ids[i] : kEmpty);
    const uint32_t r = lane_rotation();
    rotate8(ids, r);
    rotate8(wsum, r);
    rotate8(slots, r);
    const uint32_t ur = rotate_mask8(uniq, r);
    const float ef = fminf(err, 1.0f);
#pragma unroll
    for (int j = 0; j < kCand; ++j) {
        if (!(ur >> j & 1u)) continue;
        float wt = wsum[j];
        float we = wt * ef;
        float v[8] = {wt, wt * err, we, we * ux, we * uy, we * ux * ux, we * ux * uy, we * uy * uy};
        if constexpr (kFix) {
#pragma unroll
            for (int k = 0; k < 8; ++k) v[k] *= out.mul[k];
        }
        if (slots[j] >= 0) {
            table.add(slots[j], v);
        } else {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if constexpr (kFix)
                    fix_add_global(out.fix + k * out.stride + ids[j], to_fix(v[k]));
                else
                    atomicAdd(out.o[k] + ids[j], v[k]);
            }
        }
    }
    __syncthreads();
    const int used = table.size();
    for (int s = tid; s < used; s += 256) {
        const uint32_t key = table.key_at(s);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if constexpr (kFix) {
                long long v = table.fixed(k, s);
                if (v != 0) fix_add_global(out.fix + k * out.stride + key, v);
            } else {
                atomicAdd(out.o[k] + key, table.value(k, s));
            }
        }
    }
}

// fixed-point statistics -> float arrays; clears the records for the next use
__global__ void stats_finalize_kernel(StatOut out, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        long long* f = out.fix + k * out.stride + i;
        out.o[k][i] = from_fix(*f) / out.mul[k];
        *f = 0;
    }
}

static dim3 stats_grid(int w, int h) { return dim3((w + 31) / 32, (h + 7) / 8); }

void launch_site_stats(const uint32_t* c0, const uint32_t* c1, const float* target,
                       const float* mask, const Site* sites, float inv_s2, uint32_t n,
                       float* const out[8], int w, int h, int cw, int ch, cudaStream_t st) {
    StatOut o{};
    for (int k = 0; k < 8; ++k) o.o[k] = out[k];
    site_stats_kernel<false><<<stats_grid(w, h), dim3(32, 8), sizeof(TileTable<8, kStatSlots, AccFloat>), st>>>(
        reinterpret_cast<const uint4*>(c0), reinterpret_cast<const uint4*>(c1), target, mask,
        RawSites{sites}, inv_s2, n, o, w, h, cw, ch);
    note_launches(1);
}

// Power-of-two pre-scale keeping a fixed-point value exact with the most fractional bits:
// the largest mul (up to 2^30) with a tile's sum below 2^27 (the split shared words, 256
// pixel terms of at most per_pixel each) and a site's total below 2^39 (the 64-bit record,
// npix terms).  Values far below 1 (removal deltas, weights) so keep a resolution far finer
// than the 2^-24 of an unscaled term.
static float fix_mul_for_bound(double per_pixel, double npix) {
    float mul = 0x1p30f;
    while (mul > 0x1p-60f &&
           (256.0 * per_pixel * mul >= 0x1p27 || npix * per_pixel * mul >= 0x1p39))
        mul *= 0.5f;
    return mul;
}

float removal_fix_mul(int w, int h) {
    // per pixel |delta| <= 3: a difference of two squared colour errors, colours in [0, 1]
    return fix_mul_for_bound(4.0, static_cast<double>(w) * h);
}

void launch_site_stats_fixed(const uint32_t* c0, const uint32_t* c1, const float* target,
                             const float* mask, const Site* sites, float inv_s2, uint32_t n,
                             long long* fix, size_t stride, float* const out[8], int w, int h,
                             int cw, int ch, cudaStream_t st) {
    StatOut o{};
    for (int k = 0; k < 8; ++k) o.o[k] = out[k];
    o.fix = fix;
    o.stride = stride;
    const double np = static_cast<double>(w) * h, fw = w, fh = h;
    // weights <= 1, squared colour errors <= 3, positions below the image size
    const double per_pixel[8] = {1.0, 4.0, 1.0, fw, fh, fw * fw, fw * fh, fh * fh};
    for (int k = 0; k < 8; ++k) o.mul[k] = fix_mul_for_bound(per_pixel[k], np);
    site_stats_kernel<true><<<stats_grid(w, h), dim3(32, 8), sizeof(TileTable<8, kStatSlots, AccSplit>), st>>>(
        reinterpret_cast<const uint4*>(c0), reinterpret_cast<const uint4*>(c1), target, mask,
        RawSites{sites}, inv_s2, n, o, w, h, cw, ch);
    stats_finalize_kernel<<<blocks_for(n, 256), 256, 0, st>>>(o, n);
    note_launches(2);
}

// ---------------------------------------------------------------------------
// Hilbert order (backends/cuda/src/sad_cuda.cu:1512-1584)
// ---------------------------------------------------------------------------
__host__ __device__ inline uint32_t hilbert_index(uint32_t x, uint32_t y, int bits) {
    uint32_t xi = x, yi = y, index = 0;
    uint32_t mask = bits >= 32 ? 0xFFFFFFFFu : ((1u << bits) - 1u);
    for (int i = bits - 1; i >= 0; --i) {
        uint32_t s = static_cast<uint32_t>(i);
        uint32_t rx = (xi >> s) & 1u, ry = (yi >> s) & 1u;
        index |= ((3u * rx) ^ ry) << (2u * s);
        if (ry == 0u) {
            if (rx == 1u) {
                xi = mask - xi;
                yi = mask - yi;
            }
            uint32_t t = xi;
            xi = yi;
            yi = t;
        }
    }
    return index;
}

__global__ void hilbert_pairs_kernel(const Site* __restrict__ sites, uint2* __restrict__ pairs,
                                     uint32_t n, uint32_t padded, int w, int h, int bits) {
    pdl_wait();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= padded) return;
    if (i < n) {
        int px = static_cast<int>(sites[i].px), py = static_cast<int>(sites[i].py);
        px = px < 0 ? 0 : (px >= w ? w - 1 : px);
        py = py < 0 ? 0 : (py >= h ? h - 1 : py);
        pairs[i] = make_uint2(hilbert_index(px, py, bits), i);
    } else {
        pairs[i] = make_uint2(0xFFFFFFFFu, 0u);
    }
}

void launch_hilbert_pairs(const Site* sites, uint32_t* pairs, uint32_t n, uint32_t padded, int w,
                          int h, int bits, cudaStream_t st) {
    if (padded == 0) return;
    launch_pdl(hilbert_pairs_kernel, dim3(blocks_for(padded, 256)), dim3(256), 0, st, sites,
               reinterpret_cast<uint2*>(pairs), n, padded, w, h, bits);
    note_launches(1);
}

__global__ void hilbert_order_kernel(const uint2* __restrict__ pairs, uint32_t* __restrict__ order,
                                     uint32_t* __restrict__ pos, uint32_t n) {
    pdl_wait();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t s = pairs[i].y;
    order[i] = s;
    pos[s] = i;
}

void launch_hilbert_order(const uint32_t* pairs, uint32_t* order, uint32_t* pos, uint32_t n,
                          cudaStream_t st) {
    if (n == 0) return;
    launch_pdl(hilbert_order_kernel, dim3(blocks_for(n, 256)), dim3(256), 0, st,
               reinterpret_cast<const uint2*>(pairs), order, pos, n);
    note_launches(1);
}

// ---------------------------------------------------------------------------
// metrics (backends/cuda/src/utils.cu:5-101): one atomic per block after a block sum
// ---------------------------------------------------------------------------
__device__ __forceinline__ float block_sum(float v) {
    __shared__ float ws[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int tid = threadIdx.y * blockDim.x + threadIdx.x;
    int nw = (blockDim.x * blockDim.y + 31) / 32;
    if ((tid & 31) == 0) ws[tid >> 5] = v;
    __syncthreads();
    float s = 0.0f;
    if (tid == 0)
        for (int i = 0; i < nw; ++i) s += ws[i];
    return s;
}

__global__ void mse_kernel(const float* __restrict__ ren, const float* __restrict__ tgt,
                           const float* __restrict__ mask, float* __restrict__ acc, int w, int h) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    float v = 0.0f;
    if (x < w && y < h) {
        int p = y * w + x;
        if (!mask || mask[p] > 0.0f) {
            float d0 = ren[3 * p] - tgt[3 * p], d1 = ren[3 * p + 1] - tgt[3 * p + 1],
                  d2 = ren[3 * p + 2] - tgt[3 * p + 2];
            v = d0 * d0 + d1 * d1 + d2 * d2;
        }
    }
    float s = block_sum(v);
    if (threadIdx.x == 0 && threadIdx.y == 0) atomicAdd(acc, s);
}

void launch_mse(const float* ren, const float* tgt, const float* mask, float* acc, int w, int h,
                cudaStream_t st) {
    mse_kernel<<<dim3((w + 31) / 32, (h + 7) / 8), dim3(32, 8), 0, st>>>(ren, tgt, mask, acc, w, h);
    note_launches(1);
}

// Reproducible form: each block's sum (fixed order) added as a fixed-point integer.
__global__ void mse_fixed_kernel(const float* __restrict__ ren, const float* __restrict__ tgt,
                                 const float* __restrict__ mask, long long* __restrict__ acc, int w,
                                 int h) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    float v = 0.0f;
    if (x < w && y < h) {
        int p = y * w + x;
        if (!mask || mask[p] > 0.0f) {
            float d0 = ren[3 * p] - tgt[3 * p], d1 = ren[3 * p + 1] - tgt[3 * p + 1],
                  d2 = ren[3 * p + 2] - tgt[3 * p + 2];
            v = d0 * d0 + d1 * d1 + d2 * d2;
        }
    }
    float s = block_sum(v);
    if (threadIdx.x == 0 && threadIdx.y == 0) fix_add_global(acc, to_fix(s));
}

void launch_mse_fixed(const float* ren, const float* tgt, const float* mask, long long* acc, int w,
                      int h, cudaStream_t st) {
    mse_fixed_kernel<<<dim3((w + 31) / 32, (h + 7) / 8), dim3(32, 8), 0, st>>>(ren, tgt, mask, acc, w, h);
    note_launches(1);
}

__global__ void ssim_kernel(const float* __restrict__ ren, const float* __restrict__ tgt,
                            const float* __restrict__ mask, float* __restrict__ acc, int w, int h) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    float v = 0.0f;
    if (x < w && y < h && (!mask || mask[y * w + x] > 0.0f)) {
        float mux = 0, muy = 0, ex2 = 0, ey2 = 0, exy = 0;
        for (int dy = -1; dy <= 1; ++dy) {
            int yy = clampi(y + dy, 0, h - 1);
            for (int dx = -1; dx <= 1; ++dx) {
                int xx = clampi(x + dx, 0, w - 1);
                int i = 3 * (yy * w + xx);
                float xv = ren[i] * 0.299f + ren[i + 1] * 0.587f + ren[i + 2] * 0.114f;
                float yv = tgt[i] * 0.299f + tgt[i + 1] * 0.587f + tgt[i + 2] * 0.114f;
                mux += xv; muy += yv; ex2 += xv * xv; ey2 += yv * yv; exy += xv * yv;
            }
        }
        const float invn = 0.111111111f;
        mux *= invn; muy *= invn; ex2 *= invn; ey2 *= invn; exy *= invn;
        float sx2 = fmaxf(ex2 - mux * mux, 0.0f), sy2 = fmaxf(ey2 - muy * muy, 0.0f);
        float sxy = exy - mux * muy;
        float A = 2.0f * mux * muy + 0.0001f, B = 2.0f * sxy + 0.0009f;
        float C = mux * mux + muy * muy + 0.0001f, D = sx2 + sy2 + 0.0009f;
        v = (A * B) / fmaxf(C * D, 1e-8f);
    }
    float s = block_sum(v);
    if (threadIdx.x == 0 && threadIdx.y == 0) atomicAdd(acc, s);
}

void launch_ssim(const float* ren, const float* tgt, const float* mask, float* acc, int w, int h,
                 cudaStream_t st) {
    ssim_kernel<<<dim3((w + 31) / 32, (h + 7) / 8), dim3(32, 8), 0, st>>>(ren, tgt, mask, acc, w, h);
    note_launches(1);
}

// ---------------------------------------------------------------------------
// stream compaction of the active set: the ascending list of the active sites of [0, n)
// and its length (in DevState), rebuilt after init, densify and every prune.  The site
// records themselves stay in place: candidate fields, tile maps and the Hilbert order
// keep naming sites by their slot, and the per-site kernels walk the list.
// ---------------------------------------------------------------------------
constexpr int kCompactThreads = 256;
constexpr int kCompactPer = 4;  // sites per thread
constexpr int kCompactBlock = kCompactThreads * kCompactPer;

uint32_t compact_blocks(uint32_t n) { return (n + kCompactBlock - 1) / kCompactBlock; }
__device__ __forceinline__ uint32_t compact_blocks_dev(uint32_t n) { return (n + kCompactBlock - 1) / kCompactBlock; }

// Active flags of sites base .. base+3: px[i * stride] >= 0 (stride in floats: 8 for the
// prepared geometry, 10 for site records).
__device__ __forceinline__ uint32_t compact_flags(const float* __restrict__ px, uint32_t stride, uint32_t n,
                                                  uint32_t base) {
    uint32_t f = 0;
#pragma unroll
    for (int k = 0; k < kCompactPer; ++k) {
        const uint32_t i = base + k;
        if (i < n && __ldg(px + static_cast<size_t>(i) * stride) >= 0.0f) f |= 1u << k;
    }
    return f;
}

// Active count of compaction block b into counts[b].
__device__ __forceinline__ void compact_count_block(const float* __restrict__ px, uint32_t stride, uint32_t n,
                                                    uint32_t* __restrict__ counts, uint32_t b) {
    __shared__ uint32_t warp_sums[kCompactThreads / 32];
    const uint32_t base = b * kCompactBlock + threadIdx.x * kCompactPer;
    uint32_t c = __popc(compact_flags(px, stride, n, base));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
#pragma unroll
        for (int w = 0; w < kCompactThreads / 32; ++w) t += warp_sums[w];
        counts[b] = t;
    }
}

__global__ void __launch_bounds__(kCompactThreads) compact_count_kernel(const float* __restrict__ px,
                                                                        uint32_t stride, uint32_t n,
                                                                        uint32_t* __restrict__ counts) {
    pdl_wait();
    compact_count_block(px, stride, n, counts, blockIdx.x);
}

// Compaction block blk of nb: sums the counts of the blocks before it (a few hundred
// words even at a million sites), scans its own flags and writes its slots in order; the
// last block also writes the total.
__device__ __forceinline__ void compact_write_block(const float* __restrict__ px, uint32_t stride, uint32_t n,
                                                    const uint32_t* __restrict__ counts, uint32_t* __restrict__ alive,
                                                    uint32_t* __restrict__ n_alive, uint32_t blk, uint32_t nb) {
    __shared__ uint32_t warp_sums[kCompactThreads / 32];
    __shared__ uint32_t s_before;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    {
        uint32_t b = 0;
        for (uint32_t k = tid; k < blk; k += kCompactThreads) b += counts[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) b += __shfl_down_sync(0xffffffffu, b, o);
        if (lane == 0) warp_sums[warp] = b;
        __syncthreads();
        if (tid == 0) {
            uint32_t t = 0;
#pragma unroll
            for (int w = 0; w < kCompactThreads / 32; ++w) t += warp_sums[w];
            s_before = t;
            if (blk == nb - 1) *n_alive = t + counts[blk];
        }
        __syncthreads();
    }
    const uint32_t base = blk * kCompactBlock + tid * kCompactPer;
    const uint32_t f = compact_flags(px, stride, n, base);
    const uint32_t c = __popc(f);
    uint32_t x = c;  // inclusive scan over the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += t;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    uint32_t before = s_before;
#pragma unroll
    for (int w = 0; w < kCompactThreads / 32; ++w)
        if (w < warp) before += warp_sums[w];
    uint32_t out = before + x - c;
#pragma unroll
    for (int k = 0; k < kCompactPer; ++k)
        if (f >> k & 1u) alive[out++] = base + k;
}

__global__ void __launch_bounds__(kCompactThreads) compact_write_kernel(const float* __restrict__ px,
                                                                        uint32_t stride, uint32_t n,
                                                                        const uint32_t* __restrict__ counts,
                                                                        uint32_t* __restrict__ alive,
                                                                        uint32_t* __restrict__ n_alive) {
    pdl_wait();
    compact_write_block(px, stride, n, counts, alive, n_alive, blockIdx.x, gridDim.x);
}

// Batched compaction: blockIdx.y is the image (its prepared geometry over [0, n)); blocks
// beyond an image's own number of compaction blocks return at once.
__global__ void __launch_bounds__(kCompactThreads) compact_count_batch_kernel(const SiteBatchItem* __restrict__ items) {
    pdl_wait();
    const SiteBatchItem& it = items[blockIdx.y];
    if (blockIdx.x >= max(1u, compact_blocks_dev(it.n))) return;
    compact_count_block(reinterpret_cast<const float*>(it.geom), 8u, it.n, it.alive_blocks, blockIdx.x);
}

__global__ void __launch_bounds__(kCompactThreads) compact_write_batch_kernel(const SiteBatchItem* __restrict__ items) {
    pdl_wait();
    const SiteBatchItem& it = items[blockIdx.y];
    const uint32_t nb = max(1u, compact_blocks_dev(it.n));
    if (blockIdx.x >= nb) return;
    compact_write_block(reinterpret_cast<const float*>(it.geom), 8u, it.n, it.alive_blocks, it.alive,
                        &it.state->n_alive, blockIdx.x, nb);
}

void launch_compact_batch(const SiteBatchItem* items, uint32_t n_items, uint32_t max_blocks, cudaStream_t st) {
    if (n_items == 0) return;
    const dim3 grid(std::max(1u, max_blocks), n_items);
    launch_pdl(compact_count_batch_kernel, grid, dim3(kCompactThreads), 0, st, items);
    launch_pdl(compact_write_batch_kernel, grid, dim3(kCompactThreads), 0, st, items);
    note_launches(2);
}

static void launch_compact(const float* px, uint32_t stride, uint32_t n, uint32_t* block_counts,
                           uint32_t* alive, uint32_t* n_alive, cudaStream_t st) {
    const uint32_t blocks = std::max(1u, compact_blocks(n));
    launch_pdl(compact_count_kernel, dim3(blocks), dim3(kCompactThreads), 0, st, px, stride, n, block_counts);
    launch_pdl(compact_write_kernel, dim3(blocks), dim3(kCompactThreads), 0, st, px, stride, n,
               static_cast<const uint32_t*>(block_counts), alive, n_alive);
    note_launches(2);
}

void launch_compact_active(const SiteGeom* geom, uint32_t n, uint32_t* block_counts, uint32_t* alive,
                           uint32_t* n_alive, cudaStream_t st) {
    launch_compact(reinterpret_cast<const float*>(geom), 8u, n, block_counts, alive, n_alive, st);
}

void launch_compact_sites(const Site* sites, uint32_t n, uint32_t* block_counts, uint32_t* alive,
                          uint32_t* n_alive, cudaStream_t st) {
    launch_compact(reinterpret_cast<const float*>(sites), 10u, n, block_counts, alive, n_alive, st);
}

__global__ void count_active_kernel(const Site* __restrict__ sites, uint32_t* __restrict__ count,
                                    uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool a = i < n && sites[i].px >= 0.0f;
    uint32_t b = __ballot_sync(0xffffffffu, a);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(count, __popc(b));
}

void launch_count_active(const Site* sites, uint32_t* count, uint32_t n, cudaStream_t st) {
    if (n == 0) return;
    count_active_kernel<<<blocks_for(n, 256), 256, 0, st>>>(sites, count, n);
    note_launches(1);
}

// ---------------------------------------------------------------------------
// gradient-weighted init (backends/cuda/src/densify_prune.cu:5-83)
//
// The reference hands out R2 seeds from one atomic counter, so which site gets which
// seed depends on scheduling.  Here the seeds are handed out in site order: site k keeps
// drawing until a seed is accepted or max_attempts are used.  Between two accepted
// seeds A[j-1] < A[j] lie gap_j rejected seeds, which fail floor(gap_j / max_attempts)
// whole sites before the next site takes A[j]; site index of A[j] = j + sum_{i<=j}
// floor(gap_i / max_attempts).  Accept flags are evaluated in batches, compacted in
// seed order, and the index formula is one prefix sum.  The luminance and gradient
// magnitude use explicit FMAs so the CPU restatement reproduces them bit for bit.
// ---------------------------------------------------------------------------
struct InitCtx {
    const float* target;
    const float* mask;
    float thr;
    int w, h;
};

__device__ __forceinline__ float init_lum(const float* __restrict__ t, int w, int h, int x, int y) {
    x = clampi(x, 0, w - 1);
    y = clampi(y, 0, h - 1);
    const float* p = t + 3 * (y * w + x);
    return __fmaf_rn(0.114f, p[2], __fmaf_rn(0.299f, p[0], __fmul_rn(0.587f, p[1])));
}

// returns the acceptance gradient (> thr) or -1 when rejected; position/texel out
__device__ __forceinline__ float init_try(const InitCtx& c, uint32_t seed, float& px, float& py,
                                          int& ix, int& iy, float& mval) {
    const float g = 1.32471795724474602596f;
    const float a1 = 1.0f / g;
    const float a2 = 1.0f / (g * g);
    float u = fmodf(__fmaf_rn(static_cast<float>(seed), a1, 0.5f), 1.0f);
    float v = fmodf(__fmaf_rn(static_cast<float>(seed), a2, 0.5f), 1.0f);
    px = __fmul_rn(u, static_cast<float>(c.w - 1));
    py = __fmul_rn(v, static_cast<float>(c.h - 1));
    ix = static_cast<int>(px);
    iy = static_cast<int>(py);
    mval = c.mask ? c.mask[iy * c.w + ix] : 1.0f;
    if (mval <= 0.0f) return -1.0f;
    const float* t = c.target;
    float TL = init_lum(t, c.w, c.h, ix - 1, iy - 1), T = init_lum(t, c.w, c.h, ix, iy - 1),
          TR = init_lum(t, c.w, c.h, ix + 1, iy - 1);
    float L = init_lum(t, c.w, c.h, ix - 1, iy), R = init_lum(t, c.w, c.h, ix + 1, iy);
    float BL = init_lum(t, c.w, c.h, ix - 1, iy + 1), B = init_lum(t, c.w, c.h, ix, iy + 1),
          BR = init_lum(t, c.w, c.h, ix + 1, iy + 1);
    // 2*x is exact, so these sums round the same with or without contraction
    float gx = __fmul_rn(__fadd_rn(__fsub_rn(__fadd_rn(__fsub_rn(__fadd_rn(-TL, TR), 2.0f * L), 2.0f * R), BL), BR), 0.25f);
    float gy = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fsub_rn(__fsub_rn(-TL, 2.0f * T), TR), BL), 2.0f * B), BR), 0.25f);
    float grad = __fmul_rn(sqrtf(__fmaf_rn(gx, gx, __fmul_rn(gy, gy))), mval);
    return grad > c.thr ? grad : -1.0f;
}

// flags: one ballot word per warp (8 per block); block_counts: accepted seeds per block
__global__ void init_flags_kernel(InitCtx c, uint32_t seed0, uint32_t count,
                                  uint32_t* __restrict__ block_counts, uint32_t* __restrict__ flags) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool acc = false;
    if (i < count) {
        float px, py, m;
        int ix, iy;
        acc = init_try(c, seed0 + i, px, py, ix, iy, m) > 0.0f;
    }
    uint32_t b = __ballot_sync(0xffffffffu, acc);
    if ((threadIdx.x & 31) == 0) flags[i >> 5] = b;
    __shared__ uint32_t cnt;
    if (threadIdx.x == 0) cnt = 0;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) atomicAdd(&cnt, __popc(b));
    __syncthreads();
    if (threadIdx.x == 0) block_counts[blockIdx.x] = cnt;
}

// write accepted seeds in seed order: block offset (scanned) + warp prefix + lane rank
__global__ void init_compact_kernel(const uint32_t* __restrict__ flags,
                                    const uint32_t* __restrict__ block_offs, uint32_t seed0,
                                    uint32_t count, uint32_t* __restrict__ accepted,
                                    uint32_t out_base, uint32_t out_cap) {
    __shared__ uint32_t wsum[8];
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t b = flags[(blockIdx.x * blockDim.x >> 5) + warp];
    if (lane == 0) wsum[warp] = __popc(b);
    __syncthreads();
    uint32_t off = block_offs[blockIdx.x];
    for (int k = 0; k < warp; ++k) off += wsum[k];
    if (i < count && (b >> lane & 1u)) {
        uint32_t pos = out_base + off + __popc(b & ((1u << lane) - 1u));
        if (pos < out_cap) accepted[pos] = seed0 + i;
    }
}

// floor(gap / max_attempts) per accepted seed
__global__ void init_fail_counts_kernel(const uint32_t* __restrict__ accepted, uint32_t na,
                                        uint32_t max_attempts, uint32_t* __restrict__ fails) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= na) return;
    uint32_t start = j == 0 ? 0u : accepted[j - 1] + 1u;
    fails[j] = (accepted[j] - start) / max_attempts;
}

__global__ void init_default_kernel(Site* __restrict__ sites, uint32_t n, float init_log_tau,
                                    float init_radius) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Site s;
    s.px = -1.0f; s.py = -1.0f;
    s.log_tau = init_log_tau + powf(0.0f, 0.25f) * 2.0f;
    s.radius = init_radius;
    s.r = 0.5f; s.g = 0.5f; s.b = 0.5f;
    s.dx = 1.0f; s.dy = 0.0f;
    s.log_aniso = 0.0f;
    sites[i] = s;
}

// fails[] holds the exclusive scan of the per-seed failure counts
__global__ void init_assign_kernel(InitCtx c, const uint32_t* __restrict__ accepted,
                                   const uint32_t* __restrict__ fail_scan,
                                   const uint32_t* __restrict__ fail_raw, uint32_t na,
                                   Site* __restrict__ sites, uint32_t n, float init_log_tau,
                                   float init_radius) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= na) return;
    uint64_t k = static_cast<uint64_t>(j) + fail_scan[j] + fail_raw[j];
    if (k >= n) return;
    float px, py, m;
    int ix, iy;
    float g = init_try(c, accepted[j], px, py, ix, iy, m);
    const float* col = c.target + 3 * (iy * c.w + ix);
    Site s;
    s.px = px; s.py = py;
    s.log_tau = __fmaf_rn(powf(g, 0.25f), 2.0f, init_log_tau);
    s.radius = init_radius;
    s.r = col[0]; s.g = col[1]; s.b = col[2];
    s.dx = 1.0f; s.dy = 0.0f;
    s.log_aniso = 0.0f;
    sites[k] = s;
}

// exclusive scan of u32 with temp (block sums): 3 launches
__global__ void block_reduce_kernel(const uint32_t* __restrict__ in, uint32_t n,
                                    uint32_t* __restrict__ sums) {
    uint32_t i = blockIdx.x * 1024 + threadIdx.x;
    uint32_t v = i < n ? in[i] : 0u;
    v = __reduce_add_sync(0xffffffffu, v);
    __shared__ uint32_t ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t s = __reduce_add_sync(0xffffffffu, ws[threadIdx.x]);
        if (threadIdx.x == 0) sums[blockIdx.x] = s;
    }
}

__global__ void block_scan_kernel(const uint32_t* __restrict__ in, uint32_t n,
                                  const uint32_t* __restrict__ offs, uint32_t* __restrict__ out) {
    uint32_t i = blockIdx.x * 1024 + threadIdx.x;
    uint32_t v = i < n ? in[i] : 0u;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += t;
    }
    __shared__ uint32_t ws[32];
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        ws[lane] = s;
    }
    __syncthreads();
    if (i < n) out[i] = offs[blockIdx.x] + (warp > 0 ? ws[warp - 1] : 0u) + x - v;
}


// out[i] = sum_{k<i} in[k]; tmp holds ceil(n/1024) + 1 words
static void exclusive_scan_u32(const uint32_t* in, uint32_t n, uint32_t* out, uint32_t* tmp,
                               cudaStream_t st) {
    uint32_t blocks = (n + 1023) / 1024;
    block_reduce_kernel<<<blocks, 1024, 0, st>>>(in, n, tmp);
    launch_scan_single(tmp, blocks, nullptr, st);
    block_scan_kernel<<<blocks, 1024, 0, st>>>(in, n, tmp, out);
    note_launches(2);
}

static inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

static uint32_t init_batch(uint32_t n) { return std::max<uint32_t>(4u * n, 1u << 18); }

size_t init_temp_bytes(uint32_t n) {
    size_t batch = init_batch(n);
    size_t cap = static_cast<size_t>(n) + batch;  // accepted seeds kept
    size_t nblk = (batch + 255) / 256;
    return align256(cap * 4) * 3 + align256(nblk * 8 * 4) + align256((nblk + 1) * 4) +
           align256(((cap + 1023) / 1024 + 2) * 4) + 256;
}

cudaError_t run_init_gradient_weighted(Site* sites, uint32_t n, const float* target,
                                       const float* mask, float thr, uint32_t max_attempts,
                                       float init_log_tau, float init_radius, int w, int h,
                                       void* temp, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    if (max_attempts == 0) max_attempts = 1;
    uint32_t batch = init_batch(n);
    size_t cap = static_cast<size_t>(n) + batch;
    char* t = static_cast<char*>(temp);
    uint32_t* accepted = reinterpret_cast<uint32_t*>(t);
    t += align256(cap * 4);
    uint32_t* fails = reinterpret_cast<uint32_t*>(t);
    t += align256(cap * 4);
    uint32_t* fail_scan = reinterpret_cast<uint32_t*>(t);
    t += align256(cap * 4);
    uint32_t nblk = (batch + 255) / 256;
    uint32_t* flags = reinterpret_cast<uint32_t*>(t);
    t += align256(static_cast<size_t>(nblk) * 8 * 4);
    uint32_t* boffs = reinterpret_cast<uint32_t*>(t);
    t += align256((nblk + 1) * 4);
    uint32_t* scan_tmp = reinterpret_cast<uint32_t*>(t);

    InitCtx c{target, mask, thr, w, h};
    uint64_t total_seeds = static_cast<uint64_t>(n) * max_attempts;
    uint64_t seed0 = 0;
    uint32_t na = 0;
    uint32_t* d_total = scan_tmp;  // batch total (scan_tmp is free until the final scan)
    std::vector<uint32_t> host_total(1);
    while (na < n && seed0 < total_seeds) {
        uint32_t count = static_cast<uint32_t>(std::min<uint64_t>(batch, total_seeds - seed0));
        uint32_t blocks = (count + 255) / 256;
        init_flags_kernel<<<blocks, 256, 0, st>>>(c, static_cast<uint32_t>(seed0), count, boffs, flags);
        launch_scan_single(boffs, blocks, d_total, st);
        init_compact_kernel<<<blocks, 256, 0, st>>>(flags, boffs, static_cast<uint32_t>(seed0), count,
                                                    accepted, na, static_cast<uint32_t>(cap));
        note_launches(2);
        cudaError_t e = cudaMemcpyAsync(host_total.data(), d_total, 4, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return e;
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
        na += std::min<uint32_t>(host_total[0], static_cast<uint32_t>(cap) - na);
        seed0 += count;
    }
    init_default_kernel<<<blocks_for(n, 256), 256, 0, st>>>(sites, n, init_log_tau, init_radius);
    note_launches(1);
    if (na > 0) {
        init_fail_counts_kernel<<<blocks_for(na, 256), 256, 0, st>>>(accepted, na, max_attempts, fails);
        note_launches(1);
        exclusive_scan_u32(fails, na, fail_scan, scan_tmp, st);
        init_assign_kernel<<<blocks_for(na, 256), 256, 0, st>>>(c, accepted, fail_scan, fails, na,
                                                                sites, n, init_log_tau, init_radius);
        note_launches(1);
    }
    return cudaGetLastError();
}

}  // namespace sad

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace sad;

extern "C" sad_status_t sad_compute_densify_score_pairs(const float* sites, const float* mass,
                                                        const float* energy, uint32_t* pairs,
                                                        uint32_t site_count, float min_mass,
                                                        float score_alpha, uint32_t pair_count,
                                                        sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(pair_count == 0 || pairs, "sad_compute_densify_score_pairs: null pairs");
    SAD_REQUIRE(site_count <= pair_count, "sad_compute_densify_score_pairs: site_count > pair_count");
    SAD_REQUIRE(site_count == 0 || (sites && mass && energy), "sad_compute_densify_score_pairs: null input");
    launch_densify_pairs(reinterpret_cast<const Site*>(sites), mass, energy, pairs, site_count,
                         min_mass, score_alpha, pair_count, as_stream(stream));
    return check_launch("sad_compute_densify_score_pairs");
}

extern "C" sad_status_t sad_compute_prune_score_pairs(const float* sites, const float* removal_delta,
                                                      uint32_t* pairs, uint32_t site_count,
                                                      float delta_norm, uint32_t pair_count,
                                                      sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(pair_count == 0 || pairs, "sad_compute_prune_score_pairs: null pairs");
    SAD_REQUIRE(site_count <= pair_count, "sad_compute_prune_score_pairs: site_count > pair_count");
    SAD_REQUIRE(site_count == 0 || (sites && removal_delta), "sad_compute_prune_score_pairs: null input");
    launch_prune_pairs(reinterpret_cast<const Site*>(sites), removal_delta, 1, pairs, site_count,
                       delta_norm, pair_count, as_stream(stream));
    return check_launch("sad_compute_prune_score_pairs");
}

extern "C" sad_status_t sad_write_split_indices(const uint32_t* pairs, uint32_t* indices,
                                                uint32_t k, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(k == 0 || (pairs && indices), "sad_write_split_indices: null buffer");
    launch_write_indices(pairs, indices, k, as_stream(stream));
    return check_launch("sad_write_split_indices");
}

extern "C" sad_status_t sad_prune_sites(float* sites, const uint32_t* indices, uint32_t count,
                                        sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(count == 0 || (sites && indices), "sad_prune_sites: null buffer");
    launch_prune_by_index(reinterpret_cast<Site*>(sites), indices, count, as_stream(stream));
    return check_launch("sad_prune_sites");
}

extern "C" sad_status_t sad_split_sites(float* sites, float* adam, const uint32_t* split_indices,
                                        uint32_t num_to_split, const float* mass,
                                        const float* err_w, const float* err_wx,
                                        const float* err_wy, const float* err_wxx,
                                        const float* err_wxy, const float* err_wyy,
                                        uint32_t current_site_count, const float* target,
                                        int width, int height, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_split_sites: invalid image size");
    SAD_REQUIRE(num_to_split == 0 || (sites && adam && split_indices && mass && err_w && err_wx &&
                                      err_wy && err_wxx && err_wxy && err_wyy && target),
                "sad_split_sites: null buffer");
    SAD_REQUIRE((reinterpret_cast<uintptr_t>(adam) & 15u) == 0, "sad_split_sites: adam must be 16-byte aligned");
    const float* st[7] = {mass, err_w, err_wx, err_wy, err_wxx, err_wxy, err_wyy};
    launch_split(reinterpret_cast<Site*>(sites), adam, split_indices, num_to_split, st,
                 current_site_count, target, width, height, as_stream(stream));
    return check_launch("sad_split_sites");
}

extern "C" sad_status_t sad_compute_site_stats(const uint32_t* cand0, const uint32_t* cand1,
                                               const float* target, const float* mask,
                                               const float* sites, float inv_scale_sq,
                                               uint32_t site_count, float* mass, float* energy,
                                               float* err_w, float* err_wx, float* err_wy,
                                               float* err_wxx, float* err_wxy, float* err_wyy,
                                               int width, int height, int cand_width,
                                               int cand_height, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height) && image_size_ok(cand_width, cand_height),
                "sad_compute_site_stats: invalid size");
    SAD_REQUIRE(cand0 && cand1 && target && (sites || site_count == 0),
                "sad_compute_site_stats: null input");
    SAD_REQUIRE(mass && energy && err_w && err_wx && err_wy && err_wxx && err_wxy && err_wyy,
                "sad_compute_site_stats: null output");
    float* out[8] = {mass, energy, err_w, err_wx, err_wy, err_wxx, err_wxy, err_wyy};
    launch_site_stats(cand0, cand1, target, mask, reinterpret_cast<const Site*>(sites),
                      inv_scale_sq, site_count, out, width, height, cand_width, cand_height,
                      as_stream(stream));
    return check_launch("sad_compute_site_stats");
}

extern "C" size_t sad_init_temp_bytes(uint32_t site_count) { return init_temp_bytes(site_count); }

extern "C" sad_status_t sad_init_gradient_weighted(float* sites, uint32_t site_count,
                                                   const float* target, const float* mask,
                                                   float grad_threshold, uint32_t max_attempts,
                                                   float init_log_tau, float init_radius,
                                                   int width, int height, void* temp,
                                                   size_t temp_bytes, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_init_gradient_weighted: invalid image size");
    SAD_REQUIRE(site_count == 0 || (sites && target && temp), "sad_init_gradient_weighted: null buffer");
    SAD_REQUIRE(site_count == 0 || temp_bytes >= init_temp_bytes(site_count),
                "sad_init_gradient_weighted: temp smaller than sad_init_temp_bytes(site_count)");
    cudaError_t e = run_init_gradient_weighted(reinterpret_cast<Site*>(sites), site_count, target,
                                               mask, grad_threshold, max_attempts, init_log_tau,
                                               init_radius, width, height, temp, as_stream(stream));
    return check_cuda(e, "sad_init_gradient_weighted");
}

extern "C" int sad_hilbert_bits_for_size(int width, int height) {
    int m = width > height ? width : height;
    int n = 1, bits = 0;
    while (n < m) {
        n <<= 1;
        ++bits;
    }
    return bits > 1 ? bits : 1;
}

extern "C" sad_status_t sad_hilbert_pairs(const float* sites, uint32_t* pairs, uint32_t site_count,
                                          uint32_t padded_count, int width, int height, int bits,
                                          sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(site_count <= padded_count, "sad_hilbert_pairs: site_count > padded_count");
    SAD_REQUIRE(padded_count == 0 || pairs, "sad_hilbert_pairs: null pairs");
    SAD_REQUIRE(site_count == 0 || sites, "sad_hilbert_pairs: null sites");
    launch_hilbert_pairs(reinterpret_cast<const Site*>(sites), pairs, site_count, padded_count,
                         width, height, bits, as_stream(stream));
    return check_launch("sad_hilbert_pairs");
}

extern "C" sad_status_t sad_write_hilbert_order(const uint32_t* sorted_pairs, uint32_t* order,
                                                uint32_t* pos, uint32_t site_count,
                                                sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(site_count == 0 || (sorted_pairs && order && pos), "sad_write_hilbert_order: null buffer");
    launch_hilbert_order(sorted_pairs, order, pos, site_count, as_stream(stream));
    return check_launch("sad_write_hilbert_order");
}

extern "C" sad_status_t sad_compute_mse(const float* rendered, const float* target,
                                        const float* mask, float* mse_accum, int width,
                                        int height, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_compute_mse: invalid size");
    SAD_REQUIRE(rendered && target && mse_accum, "sad_compute_mse: null buffer");
    launch_mse(rendered, target, mask, mse_accum, width, height, as_stream(stream));
    return check_launch("sad_compute_mse");
}

extern "C" sad_status_t sad_compute_ssim(const float* rendered, const float* target,
                                         const float* mask, float* ssim_accum, int width,
                                         int height, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_compute_ssim: invalid size");
    SAD_REQUIRE(rendered && target && ssim_accum, "sad_compute_ssim: null buffer");
    launch_ssim(rendered, target, mask, ssim_accum, width, height, as_stream(stream));
    return check_launch("sad_compute_ssim");
}

extern "C" sad_status_t sad_count_active_sites(const float* sites, uint32_t* count,
                                               uint32_t site_count, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(count && (sites || site_count == 0), "sad_count_active_sites: null buffer");
    launch_count_active(reinterpret_cast<const Site*>(sites), count, site_count, as_stream(stream));
    return check_launch("sad_count_active_sites");
}

extern "C" size_t sad_compact_active_scratch_bytes(uint32_t site_count) {
    return (static_cast<size_t>(std::max(1u, compact_blocks(site_count))) * 4 + 255) & ~size_t(255);
}

extern "C" sad_status_t sad_compact_active(const float* sites, uint32_t site_count, uint32_t* alive_out,
                                           uint32_t* count_dev, void* scratch, size_t scratch_bytes,
                                           sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(count_dev, "sad_compact_active: null count");
    SAD_REQUIRE(site_count == 0 || (sites && alive_out), "sad_compact_active: null buffer");
    SAD_REQUIRE(scratch && scratch_bytes >= sad_compact_active_scratch_bytes(site_count),
                "sad_compact_active: scratch smaller than sad_compact_active_scratch_bytes(site_count)");
    launch_compact_sites(reinterpret_cast<const Site*>(sites), site_count, static_cast<uint32_t*>(scratch),
                         alive_out, count_dev, as_stream(stream));
    return check_launch("sad_compact_active");
}
