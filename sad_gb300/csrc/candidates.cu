// candidates.cu -- per-pixel candidate lists: f16 site packing, jump flooding (top-4) and
// the VPT propagation pass (top-8).
//
// Candidate distances are the reference's: tau_c * dmix2 with tau_c = max(exp(log_tau),
// 1e-4) (backends/cuda/src/jfa.cu:14-63, 150-174), evaluated on f16-rounded site values in
// the VPT pass.  The insertion rule is the reference's: a candidate already in the list
// is skipped, otherwise it takes the first slot whose distance is strictly larger.  Lists
// live in registers; insertion is a branch-free compare/select network.
#include "accum.cuh"
#include "common.cuh"
#include "host_common.h"
#include "kernels.h"

namespace sad {

// ---------------------------------------------------------------------------
// f16 packing (backends/cuda/src/candidate_pack.cu:3-28)
// ---------------------------------------------------------------------------
__global__ void pack_sites_kernel(const Site* __restrict__ sites, uint4* __restrict__ packed,
                                  uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2* q = reinterpret_cast<const float2*>(sites + i);
    float2 a = q[0], b = q[1], d = q[3], e = q[4];
    __half2 h0, h1, h2, h3;
    if (a.x < 0.0f) {
        __half neg = __float2half(-1.0f), z = __float2half(0.0f);
        h0 = __halves2half2(neg, neg);
        h1 = h2 = h3 = __halves2half2(z, z);
    } else {
        h0 = __halves2half2(__float2half(a.x), __float2half(a.y));
        h1 = __halves2half2(__float2half(b.x), __float2half(b.y));
        h2 = __halves2half2(__float2half(d.y), __float2half(e.x));
        h3 = __halves2half2(__float2half(e.y), __float2half(0.0f));
    }
    uint4 o;
    o.x = *reinterpret_cast<uint32_t*>(&h0);
    o.y = *reinterpret_cast<uint32_t*>(&h1);
    o.z = *reinterpret_cast<uint32_t*>(&h2);
    o.w = *reinterpret_cast<uint32_t*>(&h3);
    packed[i] = o;
}

void launch_pack_sites(const Site* sites, uint16_t* packed, uint32_t n, cudaStream_t st) {
    if (n == 0) return;
    pack_sites_kernel<<<blocks_for(n, 256), 256, 0, st>>>(sites, reinterpret_cast<uint4*>(packed), n);
    note_launches(1);
}

// Metric record of an f16 packed site: tau field = max(exp(log_tau), 1e-4).
__device__ __forceinline__ SiteGeom geom_from_packed(uint4 v) {
    __half2 h0 = *reinterpret_cast<__half2*>(&v.x);
    __half2 h1 = *reinterpret_cast<__half2*>(&v.y);
    __half2 h2 = *reinterpret_cast<__half2*>(&v.z);
    __half2 h3 = *reinterpret_cast<__half2*>(&v.w);
    float2 pos = __half22float2(h0), tr = __half22float2(h1), dir = __half22float2(h2),
           an = __half22float2(h3);
    SiteGeom g = make_geom(pos.x, pos.y, tr.x, tr.y, dir.x, dir.y, an.x);
    g.tau = fmaxf(g.tau, 1e-4f);
    return g;
}

// Trainer form: the same record built once per site per refresh (32-byte gathers in the
// pass instead of 16-byte gathers plus two expf and a division per visit).
__device__ __forceinline__ void pack_geom_one(const Site* __restrict__ sites, SiteGeom* __restrict__ out,
                                              uint32_t i);

__global__ void pack_geom_kernel(const Site* __restrict__ sites, SiteGeom* __restrict__ out,
                                 uint32_t n) {
    pdl_wait();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pack_geom_one(sites, out, i);
}

// The trainer's refresh: only the listed (active) sites; a pruned site's record is marked
// inactive by the prune itself.
__global__ void pack_geom_alive_kernel(const Site* __restrict__ sites, SiteGeom* __restrict__ out,
                                       const uint32_t* __restrict__ alive, const DevState* __restrict__ state) {
    pdl_wait();
    const uint32_t n_alive = state->n_alive;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_alive; j += gridDim.x * blockDim.x)
        pack_geom_one(sites, out, alive[j]);
}

__device__ __forceinline__ void pack_geom_one(const Site* __restrict__ sites, SiteGeom* __restrict__ out,
                                              uint32_t i) {
    const float2* q = reinterpret_cast<const float2*>(sites + i);
    float2 a = q[0], b = q[1], d = q[3], e = q[4];
    uint4 v;
    if (a.x < 0.0f) {
        __half neg = __float2half(-1.0f), z = __float2half(0.0f);
        __half2 h0 = __halves2half2(neg, neg), hz = __halves2half2(z, z);
        v.x = *reinterpret_cast<uint32_t*>(&h0);
        v.y = v.z = v.w = *reinterpret_cast<uint32_t*>(&hz);
    } else {
        __half2 h0 = __halves2half2(__float2half(a.x), __float2half(a.y));
        __half2 h1 = __halves2half2(__float2half(b.x), __float2half(b.y));
        __half2 h2 = __halves2half2(__float2half(d.y), __float2half(e.x));
        __half2 h3 = __halves2half2(__float2half(e.y), __float2half(0.0f));
        v.x = *reinterpret_cast<uint32_t*>(&h0);
        v.y = *reinterpret_cast<uint32_t*>(&h1);
        v.z = *reinterpret_cast<uint32_t*>(&h2);
        v.w = *reinterpret_cast<uint32_t*>(&h3);
    }
    store_geom(out, i, geom_from_packed(v));
}

void launch_pack_geom(const Site* sites, SiteGeom* out, uint32_t n, cudaStream_t st) {
    if (n == 0) return;
    launch_pdl(pack_geom_kernel, dim3(blocks_for(n, 256)), dim3(256), 0, st, sites, out, n);
    note_launches(1);
}

__global__ void __launch_bounds__(256) pack_geom_batch_kernel(const SiteBatchItem* __restrict__ items,
                                                              const uint32_t* __restrict__ prefix,
                                                              uint32_t n_items) {
    pdl_wait();
    __shared__ uint32_t s_prefix[kMaxBatchItems + 1];
    const uint32_t total = load_site_prefix(s_prefix, prefix, n_items);
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const uint32_t k = batch_item_of(s_prefix, n_items, g);
        const SiteBatchItem& it = items[k];
        pack_geom_one(it.sites, it.vgeom, it.alive[g - s_prefix[k]]);
    }
}

void launch_pack_geom_batch(const SiteBatchItem* items, const uint32_t* site_prefix, uint32_t n_items,
                            uint32_t grid_threads, cudaStream_t st) {
    launch_pdl(pack_geom_batch_kernel, dim3(std::max(1u, blocks_for(grid_threads, 256))), dim3(256), 0, st, items,
               site_prefix, n_items);
    note_launches(1);
}

void launch_pack_geom_alive(const Site* sites, SiteGeom* out, const uint32_t* alive, const DevState* state,
                            uint32_t max_alive, cudaStream_t st) {
    if (max_alive == 0) return;
    launch_pdl(pack_geom_alive_kernel, dim3(blocks_for(max_alive, 256)), dim3(256), 0, st, sites, out, alive,
               state);
    note_launches(1);
}

struct PackedHalfSites {
    const uint4* p;
    __device__ __forceinline__ SiteGeom load(uint32_t id) const { return geom_from_packed(__ldg(p + id)); }
};
struct PackedGeomSites {
    const SiteGeom* g;
    __device__ __forceinline__ SiteGeom load(uint32_t id) const { return load_geom(g, id); }
};

// ---------------------------------------------------------------------------
// sorted top-L lists
// ---------------------------------------------------------------------------
template <int L>
__device__ __forceinline__ void sorted_insert(uint32_t (&bi)[L], float (&bd)[L], uint32_t id,
                                              float d) {
    if (!(d < bd[L - 1])) return;  // not better than the last entry: no slot takes it
#pragma unroll
    for (int j = L - 1; j > 0; --j) {
        bool before_prev = d < bd[j - 1];
        bool before_this = d < bd[j];
        float nd = before_prev ? bd[j - 1] : (before_this ? d : bd[j]);
        uint32_t ni = before_prev ? bi[j - 1] : (before_this ? id : bi[j]);
        bd[j] = nd;
        bi[j] = ni;
    }
    if (d < bd[0]) {
        bd[0] = d;
        bi[0] = id;
    }
}

template <int L>
__device__ __forceinline__ bool in_list(const uint32_t (&bi)[L], uint32_t id) {
    bool hit = false;
#pragma unroll
    for (int j = 0; j < L; ++j) hit |= bi[j] == id;
    return hit;
}

// VPT insertion: insertClosest8Packed, backends/cuda/src/jfa.cu:176-248
template <class Src>
__device__ __forceinline__ void vpt_insert(uint32_t (&bi)[8], float (&bd)[8], uint32_t id, float ux,
                                           float uy, const Src& src, uint32_t n, float inv_s2,
                                           float inv_scale) {
    if (id >= n) return;
    if (in_list<8>(bi, id)) return;
    SiteGeom g = src.load(id);
    float d = g.px < 0.0f ? INFINITY : g.tau * dmix2(g, ux, uy, inv_s2, inv_scale);
    sorted_insert<8>(bi, bd, id, d);
}

template <class Src>
__device__ __forceinline__ void vpt_merge(uint32_t (&bi)[8], float (&bd)[8], uint4 c0, uint4 c1,
                                          float ux, float uy, const Src& src, uint32_t n,
                                          float inv_s2, float inv_scale) {
    vpt_insert(bi, bd, c0.x, ux, uy, src, n, inv_s2, inv_scale);
    vpt_insert(bi, bd, c0.y, ux, uy, src, n, inv_s2, inv_scale);
    vpt_insert(bi, bd, c0.z, ux, uy, src, n, inv_s2, inv_scale);
    vpt_insert(bi, bd, c0.w, ux, uy, src, n, inv_s2, inv_scale);
    vpt_insert(bi, bd, c1.x, ux, uy, src, n, inv_s2, inv_scale);
    vpt_insert(bi, bd, c1.y, ux, uy, src, n, inv_s2, inv_scale);
    vpt_insert(bi, bd, c1.z, ux, uy, src, n, inv_s2, inv_scale);
    vpt_insert(bi, bd, c1.w, ux, uy, src, n, inv_s2, inv_scale);
}

// Jump schedule on the device (jumpStepForIndex/packJumpStep, sad_cuda.cu:1157-1183);
// pow2 and stages depend only on the field size and come from the host.
__device__ __forceinline__ uint32_t device_pack_jump(uint32_t idx, uint32_t pow2, uint32_t stages) {
    uint32_t jump = 1;
    if (pow2 > 1u) {
        uint32_t stage = idx >= stages ? stages - 1u : idx;
        jump = max(pow2 >> (stage + 1u), 1u);
    }
    jump = min(jump, 0xffffu);
    return (jump << 16) | (idx & 0xffffu);
}

// One VPT pass, backends/cuda/src/jfa.cu:271-386.
// One VPT pass at candidate-field texel (x, y) (in range): writes the new list to
// prm.out0/out1 and returns it in out.  backends/cuda/src/jfa.cu:271-386.
template <class Src>
__device__ __forceinline__ void vpt_pixel(const VptParams& prm, const Src& src, int x, int y,
                                          uint32_t (&out)[8]) {

    const int w = prm.width, h = prm.height;
    uint32_t step = prm.step, step_high = prm.step_high;
    if (prm.state) {
        uint32_t idx = prm.state->vpt_pass + prm.pass_offset;
        step = device_pack_jump(idx, prm.pow2, prm.stages);
        step_high = idx >> 16;
    }
    const uint32_t n = prm.site_count;
    uint32_t step_index = step & 0xffffu;
    uint32_t jump = step >> 16;
    if (jump == 0u) jump = 1u;
    uint32_t full_step = (step_high << 16) | step_index;
    float ux = fminf(static_cast<float>(x) * static_cast<float>(prm.cand_downscale),
                     static_cast<float>(prm.target_width - 1));
    float uy = fminf(static_cast<float>(y) * static_cast<float>(prm.cand_downscale),
                     static_cast<float>(prm.target_height - 1));
    const float inv_s2 = prm.inv_scale_sq;
    const float inv_scale = sqrtf(inv_s2);
    const uint4* in0 = reinterpret_cast<const uint4*>(prm.in0);
    const uint4* in1 = reinterpret_cast<const uint4*>(prm.in1);
    int p = y * w + x;

    uint32_t bi[8];
    float bd[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        bi[i] = kEmpty;
        bd[i] = INFINITY;
    }
    vpt_merge(bi, bd, __ldg(in0 + p), __ldg(in1 + p), ux, uy, src, n, inv_s2, inv_scale);
    const int off[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int nx = clampi(x + off[k][0] * static_cast<int>(jump), 0, w - 1);
        int ny = clampi(y + off[k][1] * static_cast<int>(jump), 0, h - 1);
        int q = ny * w + nx;
        vpt_merge(bi, bd, __ldg(in0 + q), __ldg(in1 + q), ux, uy, src, n, inv_s2, inv_scale);
    }
    if (prm.radius_probes > 0u) {
        float rad = prm.radius_scale * (static_cast<float>(w) / 1024.0f);
        uint32_t st = (static_cast<uint32_t>(x) * 73856093u) ^ (static_cast<uint32_t>(y) * 19349663u) ^
                      ((step_index + jump) * 83492791u);
        for (uint32_t r = 0; r < prm.radius_probes; ++r) {
            st = xorshift32(st);
            float a = static_cast<float>(st) * (1.0f / 4294967296.0f) * 6.2831853f;
            int ddx = static_cast<int>(cosf(a) * rad);
            int ddy = static_cast<int>(sinf(a) * rad);
            int px = clampi(x + ddx, 0, w - 1), py = clampi(y + ddy, 0, h - 1);
            if (px == x && py == y) continue;
            int q = py * w + px;
            vpt_merge(bi, bd, __ldg(in0 + q), __ldg(in1 + q), ux, uy, src, n, inv_s2, inv_scale);
        }
    }
    if (prm.hilbert_probes > 0u && prm.hilbert_window > 0u) {
        uint32_t best = bi[0];
        if (best < n) {
            uint32_t pos = __ldg(prm.hilbert_pos + best);
            uint32_t span = prm.hilbert_window * 2u + 1u;
            uint32_t hs = (static_cast<uint32_t>(x) * 2654435761u) ^
                          (static_cast<uint32_t>(y) * 1597334677u) ^ (full_step * 374761393u);
            for (uint32_t i = 0; i < prm.hilbert_probes; ++i) {
                hs = xorshift32(hs + i);
                int o = static_cast<int>(hs % span) - static_cast<int>(prm.hilbert_window);
                int idx = clampi(static_cast<int>(pos) + o, 0, static_cast<int>(n - 1));
                vpt_insert(bi, bd, __ldg(prm.hilbert_order + idx), ux, uy, src, n, inv_s2, inv_scale);
            }
        }
    }
    uint32_t is = (static_cast<uint32_t>(x) * 1664525u) ^ (static_cast<uint32_t>(y) * 1013904223u) ^
                  (full_step * 374761393u);
    for (uint32_t i = 0; i < prm.inject_count; ++i) {
        is = xorshift32(is + i);
        vpt_insert(bi, bd, is % n, ux, uy, src, n, inv_s2, inv_scale);
    }
    reinterpret_cast<uint4*>(prm.out0)[p] = make_uint4(bi[0], bi[1], bi[2], bi[3]);
    reinterpret_cast<uint4*>(prm.out1)[p] = make_uint4(bi[4], bi[5], bi[6], bi[7]);
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = bi[i];
}

template <class Src>
__global__ void __launch_bounds__(256, 5) vpt_kernel(VptParams prm, Src src) {
    pdl_wait();
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= prm.width || y >= prm.height) return;
    uint32_t out[8];
    vpt_pixel(prm, src, x, y, out);
}

// Batched form over the 32x8-pixel blocks of every image of a batch (the trainer's
// refresh pass on the f16-rounded geometry).
// The pass reads its parameters throughout each pixel's merges; one thread copies the
// block's image from the kernel parameters into shared memory (measured 3% faster than
// reading them from the constant bank, unlike the gradient kernel, whose shared-memory
// pipe is busy with the tile table's atomics).
__global__ void __launch_bounds__(256, 5) vpt_batch_kernel(const __grid_constant__ BatchArgs<VptBatchItem> a) {
    pdl_wait();
    __shared__ VptParams s_p;
    __shared__ const SiteGeom* s_g;
    __shared__ int s_local, s_bx;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        const uint32_t i = a.item_of(blockIdx.x);
        s_p = a.items[i].p;
        s_g = a.items[i].vgeom;
        s_bx = a.items[i].blocks_x;
        s_local = static_cast<int>(blockIdx.x - a.block_prefix[i]);
    }
    __syncthreads();
    const int x = (s_local % s_bx) * 32 + threadIdx.x;
    const int y = (s_local / s_bx) * 8 + threadIdx.y;
    if (x >= s_p.width || y >= s_p.height) return;
    uint32_t out[8];
    vpt_pixel(s_p, PackedGeomSites{s_g}, x, y, out);
}

void launch_vpt_batch(const VptBatchItem* items, const uint32_t* block_prefix, uint32_t n_items, cudaStream_t st) {
    for_each_batch_launch(items, block_prefix, n_items, [&](const BatchArgs<VptBatchItem>& a, uint32_t blocks) {
        launch_pdl(vpt_batch_kernel, dim3(blocks), dim3(32, 8), 0, st, a);
        note_launches(1);
    });
}

static dim3 pixel_grid(int w, int h) { return dim3((w + 31) / 32, (h + 7) / 8); }

void launch_vpt_packed(const VptParams& prm, const uint16_t* packed, cudaStream_t st) {
    launch_pdl(vpt_kernel<PackedHalfSites>, pixel_grid(prm.width, prm.height), dim3(32, 8), 0, st,
        prm, PackedHalfSites{reinterpret_cast<const uint4*>(packed)});
    note_launches(1);
}

void launch_vpt_geom(const VptParams& prm, const SiteGeom* geom, cudaStream_t st) {
    launch_pdl(vpt_kernel<PackedGeomSites>, pixel_grid(prm.width, prm.height), dim3(32, 8), 0, st,
        prm, PackedGeomSites{geom});
    note_launches(1);
}

// ---------------------------------------------------------------------------
// JFA (backends/cuda/src/jfa.cu:66-144)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int seed_texel(float px, float py, int w, int h, int ds) {
    float inv = 1.0f / fmaxf(static_cast<float>(ds), 1.0f);
    int x = clampi(static_cast<int>(px * inv), 0, w - 1);
    int y = clampi(static_cast<int>(py * inv), 0, h - 1);
    return y * w + x;
}

// Two phases give a deterministic winner (the lowest id) where sites share a texel.
__global__ void jfa_seed_mark_kernel(uint32_t* __restrict__ cand0, const Site* __restrict__ sites,
                                     uint32_t n, int w, int h, int ds) {
    pdl_wait();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float px = sites[i].px;
    if (px < 0.0f) return;
    cand0[4 * seed_texel(px, sites[i].py, w, h, ds)] = kEmpty;
}

__global__ void jfa_seed_min_kernel(uint32_t* __restrict__ cand0, const Site* __restrict__ sites,
                                    uint32_t n, int w, int h, int ds) {
    pdl_wait();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float px = sites[i].px;
    if (px < 0.0f) return;
    atomicMin(&cand0[4 * seed_texel(px, sites[i].py, w, h, ds)], i);
}

void launch_jfa_seed(uint32_t* cand0, const Site* sites, uint32_t n, int w, int h, int ds,
                     cudaStream_t st) {
    if (n == 0) return;
    launch_pdl(jfa_seed_mark_kernel, dim3(blocks_for(n, 256)), dim3(256), 0, st, cand0, sites, n, w, h, ds);
    launch_pdl(jfa_seed_min_kernel, dim3(blocks_for(n, 256)), dim3(256), 0, st, cand0, sites, n, w, h, ds);
    note_launches(2);
}

struct RawGeomSites {
    const Site* s;
    __device__ __forceinline__ SiteGeom load(uint32_t id) const {
        const float2* q = reinterpret_cast<const float2*>(s + id);
        float2 a = __ldg(q), b = __ldg(q + 1), d = __ldg(q + 3), e = __ldg(q + 4);
        return make_geom(a.x, a.y, b.x, b.y, d.y, e.x, e.y);
    }
};
struct FullGeomSites {
    const SiteGeom* g;
    __device__ __forceinline__ SiteGeom load(uint32_t id) const { return load_geom(g, id); }
};

template <class Src>
__device__ __forceinline__ void jfa_insert(uint32_t (&bi)[4], float (&bd)[4], uint32_t id, float ux,
                                           float uy, const Src& src, uint32_t n, float inv_s2,
                                           float inv_scale) {
    if (id >= n) return;
    if (in_list<4>(bi, id)) return;
    SiteGeom g = src.load(id);
    if (g.px < 0.0f) return;
    float dm = dmix2(g, ux, uy, inv_s2, inv_scale);
    float tau = fmaxf(g.tau, 1e-4f);
    sorted_insert<4>(bi, bd, id, tau * dm);
}

template <class Src>
__global__ void __launch_bounds__(256) jfa_flood_kernel(const uint4* __restrict__ in0,
                                                        uint4* __restrict__ out0, Src src,
                                                        uint32_t n, uint32_t step, float inv_s2,
                                                        int w, int h, int ds, int tw, int th) {
    pdl_wait();
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    float ux = fminf(static_cast<float>(x) * static_cast<float>(ds), static_cast<float>(tw - 1));
    float uy = fminf(static_cast<float>(y) * static_cast<float>(ds), static_cast<float>(th - 1));
    float inv_scale = sqrtf(inv_s2);
    uint32_t bi[4] = {kEmpty, kEmpty, kEmpty, kEmpty};
    float bd[4] = {INFINITY, INFINITY, INFINITY, INFINITY};
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy) {
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
            int sx = clampi(x + dx * static_cast<int>(step), 0, w - 1);
            int sy = clampi(y + dy * static_cast<int>(step), 0, h - 1);
            uint4 c = __ldg(in0 + sy * w + sx);
            jfa_insert(bi, bd, c.x, ux, uy, src, n, inv_s2, inv_scale);
            jfa_insert(bi, bd, c.y, ux, uy, src, n, inv_s2, inv_scale);
            jfa_insert(bi, bd, c.z, ux, uy, src, n, inv_s2, inv_scale);
            jfa_insert(bi, bd, c.w, ux, uy, src, n, inv_s2, inv_scale);
        }
    }
    out0[y * w + x] = make_uint4(bi[0], bi[1], bi[2], bi[3]);
}

void launch_jfa_flood_raw(const uint32_t* in0, uint32_t* out0, const Site* sites, uint32_t n,
                          uint32_t step, float inv_s2, int w, int h, int ds, int tw, int th,
                          cudaStream_t st) {
    launch_pdl(jfa_flood_kernel<RawGeomSites>, pixel_grid(w, h), dim3(32, 8), 0, st,
        reinterpret_cast<const uint4*>(in0), reinterpret_cast<uint4*>(out0), RawGeomSites{sites},
        n, step, inv_s2, w, h, ds, tw, th);
    note_launches(1);
}

void launch_jfa_flood_geom(const uint32_t* in0, uint32_t* out0, const SiteGeom* geom, uint32_t n,
                           uint32_t step, float inv_s2, int w, int h, int ds, int tw, int th,
                           cudaStream_t st) {
    launch_pdl(jfa_flood_kernel<FullGeomSites>, pixel_grid(w, h), dim3(32, 8), 0, st,
        reinterpret_cast<const uint4*>(in0), reinterpret_cast<uint4*>(out0), FullGeomSites{geom},
        n, step, inv_s2, w, h, ds, tw, th);
    note_launches(1);
}

uint32_t host_jump_step_for_index(uint32_t idx, int w, int h) {
    uint32_t maxd = static_cast<uint32_t>(w > h ? w : h);
    uint32_t pow2 = 1;
    while (pow2 < maxd) pow2 <<= 1;
    if (pow2 <= 1) return 1;
    uint32_t stages = 0, t = pow2;
    while (t > 1) {
        t >>= 1;
        ++stages;
    }
    uint32_t stage = idx >= stages ? stages - 1 : idx;
    uint32_t s = pow2 >> (stage + 1);
    return s > 1u ? s : 1u;
}

void jump_schedule_constants(int w, int h, uint32_t* pow2_out, uint32_t* stages_out) {
    uint32_t maxd = static_cast<uint32_t>(w > h ? w : h);
    uint32_t pow2 = 1;
    while (pow2 < maxd) pow2 <<= 1;
    uint32_t stages = 0, t = pow2;
    while (t > 1) {
        t >>= 1;
        ++stages;
    }
    *pow2_out = pow2;
    *stages_out = stages;
}

}  // namespace sad

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace sad;

extern "C" uint32_t sad_jump_step_for_index(uint32_t step_index, int width, int height) {
    return host_jump_step_for_index(step_index, width, height);
}

extern "C" uint32_t sad_pack_jump_step(uint32_t step_index, int width, int height) {
    uint32_t j = host_jump_step_for_index(step_index, width, height);
    if (j > 0xffffu) j = 0xffffu;
    return (j << 16) | (step_index & 0xffffu);
}

extern "C" sad_status_t sad_pack_candidate_sites(const float* sites, uint16_t* packed,
                                                 uint32_t site_count, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(site_count == 0 || (sites && packed), "sad_pack_candidate_sites: null buffer");
    launch_pack_sites(reinterpret_cast<const Site*>(sites), packed, site_count, as_stream(stream));
    return check_launch("sad_pack_candidate_sites");
}

extern "C" sad_status_t sad_jfa_seed(uint32_t* cand0, const float* sites, uint32_t site_count,
                                     int width, int height, int cand_downscale,
                                     sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_jfa_seed: invalid cand size");
    SAD_REQUIRE(cand0 && (sites || site_count == 0), "sad_jfa_seed: null buffer");
    launch_jfa_seed(cand0, reinterpret_cast<const Site*>(sites), site_count, width, height,
                    cand_downscale, as_stream(stream));
    return check_launch("sad_jfa_seed");
}

extern "C" sad_status_t sad_jfa_flood(const uint32_t* in_cand0, uint32_t* out_cand0,
                                      const float* sites, uint32_t site_count, uint32_t step_size,
                                      float inv_scale_sq, int width, int height,
                                      int cand_downscale, int target_width, int target_height,
                                      sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_jfa_flood: invalid cand size");
    SAD_REQUIRE(target_width > 0 && target_height > 0, "sad_jfa_flood: invalid target size");
    SAD_REQUIRE(in_cand0 && out_cand0 && (sites || site_count == 0), "sad_jfa_flood: null buffer");
    SAD_REQUIRE(in_cand0 != out_cand0, "sad_jfa_flood: in and out must differ");
    launch_jfa_flood_raw(in_cand0, out_cand0, reinterpret_cast<const Site*>(sites), site_count,
                         step_size, inv_scale_sq, width, height, cand_downscale, target_width,
                         target_height, as_stream(stream));
    return check_launch("sad_jfa_flood");
}

extern "C" sad_status_t sad_update_candidates(
    const uint32_t* in_cand0, const uint32_t* in_cand1, uint32_t* out_cand0, uint32_t* out_cand1,
    const uint16_t* packed_sites, uint32_t site_count, uint32_t step, float inv_scale_sq,
    uint32_t step_high, float radius_scale, uint32_t radius_probes, uint32_t inject_count,
    const uint32_t* hilbert_order, const uint32_t* hilbert_pos, uint32_t hilbert_probes,
    uint32_t hilbert_window, int cand_downscale, int target_width, int target_height, int width,
    int height, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_update_candidates: invalid cand size");
    SAD_REQUIRE(target_width > 0 && target_height > 0, "sad_update_candidates: invalid target size");
    SAD_REQUIRE(in_cand0 && in_cand1 && out_cand0 && out_cand1, "sad_update_candidates: null field");
    SAD_REQUIRE(in_cand0 != out_cand0 && in_cand1 != out_cand1,
                "sad_update_candidates: in and out fields must differ");
    SAD_REQUIRE(site_count == 0 || packed_sites, "sad_update_candidates: null packed sites");
    bool use_h = hilbert_probes > 0 && hilbert_window > 0;
    SAD_REQUIRE(!use_h || (hilbert_order && hilbert_pos),
                "sad_update_candidates: hilbert probes need hilbert_order and hilbert_pos");
    VptParams prm{};
    prm.in0 = in_cand0;
    prm.in1 = in_cand1;
    prm.out0 = out_cand0;
    prm.out1 = out_cand1;
    prm.site_count = site_count;
    prm.step = step;
    prm.step_high = step_high;
    prm.inv_scale_sq = inv_scale_sq;
    prm.radius_scale = radius_scale;
    prm.radius_probes = radius_probes;
    prm.inject_count = site_count == 0 ? 0u : inject_count;
    prm.hilbert_order = hilbert_order;
    prm.hilbert_pos = hilbert_pos;
    prm.hilbert_probes = use_h ? hilbert_probes : 0u;
    prm.hilbert_window = use_h ? hilbert_window : 0u;
    prm.cand_downscale = cand_downscale;
    prm.target_width = target_width;
    prm.target_height = target_height;
    prm.width = width;
    prm.height = height;
    prm.state = nullptr;
    launch_vpt_packed(prm, packed_sites, as_stream(stream));
    return check_launch("sad_update_candidates");
}
