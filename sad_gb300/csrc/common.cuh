// common.cuh -- shared device definitions for the SAD fit-and-render kernels.
//
// Layout contract with the reference (LuckyIYI/SAD):
//   * Site            : 10 x f32 (40 B), backends/cuda/src/sad_common.cuh:21-31.  This is
//                       also the [N,10] torch layout.
//   * candidate field : two [W*H][4] u32 arrays (slots 0-3 and 4-7), 0xFFFFFFFF empty.
//   * packed f16 site : 8 x f16 (16 B), backends/cuda/src/candidate_pack.cu:3-28.
//
// GB300 additions (internal, never crossing the C ABI):
//   * SiteGeom (32 B, 32-B aligned): per-site constants of the soft Voronoi metric,
//     precomputed once per site instead of once per (pixel, candidate).  Every field is
//     produced by the same single operation the reference performs inline (expf, 1/x), so
//     distances computed from it are bit-identical to the reference's.  The radius is kept
//     raw: the reference's `sqrtf(d2) - radius * inv_scale` is contracted into one FMA by
//     nvcc, and precomputing the product would round it differently.
//     One gather = one 32-B sector.
//   * SiteColor (16 B): r, g, b, pad.
#pragma once

#include <utility>

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace sad {

constexpr int kCand = 8;
constexpr uint32_t kEmpty = 0xFFFFFFFFu;

struct Site {
    float px, py, log_tau, radius, r, g, b, dx, dy, log_aniso;
};
static_assert(sizeof(Site) == 40, "Site must match the [N,10] f32 layout");

struct __align__(32) SiteGeom {
    float px, py;  // position (px < 0: inactive)
    float tau;     // expf(log_tau)
    float radius;  // radius in pixels (normalised in-kernel by sqrtf(inv_scale_sq))
    float dx, dy;  // anisotropy direction
    float l1;      // expf(log_aniso)
    float l2;      // 1 / l1
};
static_assert(sizeof(SiteGeom) == 32, "SiteGeom is one sector");

struct __align__(16) SiteColor {
    float r, g, b, pad;
};

// Device-resident iteration counters of the trainer (read by graph-replayed kernels).
struct DevState {
    uint32_t iter;      // training iteration about to run
    uint32_t vpt_pass;  // global VPT pass index (jumpPassIndex of the reference)
    float adam_c1;      // Adam bias corrections 1 / (1 - beta^t) for t = iter + 1
    float adam_c2;
    uint32_t n_alive;   // length of the compacted active-site list
    int32_t wide_far_refs;  // tile-table shape rule of the tile registration (tuned on the host)
    uint32_t pad[2];
};

// Programmatic dependent launch: a kernel launched with the programmatic-serialization
// attribute may start while the previous kernel in its stream drains; it waits here, before
// reading anything that kernel wrote, for that kernel's completion and memory.  A no-op for a
// normally launched kernel.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Launch with programmatic stream serialization (the kernel must call pdl_wait() first).
template <class... KArgs, class... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

__device__ __forceinline__ int clampi(int x, int a, int b) { return max(a, min(b, x)); }
__device__ __forceinline__ float clampf(float x, float a, float b) { return fmaxf(a, fminf(b, x)); }

// Reference RNG, backends/cuda/src/sad_common.cuh:128-138.
__host__ __device__ __forceinline__ uint32_t xorshift32(uint32_t x) {
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    return x;
}

// Candidate-field texel of an output pixel, backends/cuda/src/sad_common.cuh:113-125.
__device__ __forceinline__ int cand_index_for_pixel(int x, int y, int w, int h, int cw, int ch) {
    int sw = w > 0 ? w : 1;
    int sh = h > 0 ? h : 1;
    int cx = clampi((x * cw) / sw, 0, cw - 1);
    int cy = clampi((y * ch) / sh, 0, ch - 1);
    return cy * cw + cx;
}

// Build the metric constants of one site the way the reference evaluates them inline
// (voronoi_dmix2, backends/cuda/src/sad_common.cuh:141-165).
__device__ __forceinline__ SiteGeom make_geom(float px, float py, float log_tau, float radius,
                                              float dx, float dy, float log_aniso) {
    SiteGeom g;
    g.px = px;
    g.py = py;
    g.tau = expf(log_tau);
    g.radius = radius;
    g.dx = dx;
    g.dy = dy;
    g.l1 = expf(log_aniso);
    g.l2 = 1.0f / g.l1;
    return g;
}

__device__ __forceinline__ SiteGeom load_geom(const SiteGeom* __restrict__ p, uint32_t i) {
    const float4* q = reinterpret_cast<const float4*>(p + i);
    float4 a = __ldg(q);
    float4 b = __ldg(q + 1);
    SiteGeom g;
    g.px = a.x; g.py = a.y; g.tau = a.z; g.radius = a.w;
    g.dx = b.x; g.dy = b.y; g.l1 = b.z; g.l2 = b.w;
    return g;
}

__device__ __forceinline__ void store_geom(SiteGeom* p, uint32_t i, const SiteGeom& g) {
    float4* q = reinterpret_cast<float4*>(p + i);
    q[0] = make_float4(g.px, g.py, g.tau, g.radius);
    q[1] = make_float4(g.dx, g.dy, g.l1, g.l2);
}

// Squared anisotropic distance terms at pixel (ux, uy): the algebra of voronoi_dmix2
// written with the same operand order, so nvcc forms the same fused multiply-adds.
struct MetricTerms {
    float dx, dy;   // uv - position
    float proj;     // dir . diff
    float proj2, perp2;
    float d2_safe;  // max(normalised anisotropic distance^2, 1e-8)
};

__device__ __forceinline__ MetricTerms metric_terms(const SiteGeom& g, float ux, float uy,
                                                    float inv_scale_sq) {
    MetricTerms m;
    m.dx = ux - g.px;
    m.dy = uy - g.py;
    float diff2 = m.dx * m.dx + m.dy * m.dy;
    m.proj = g.dx * m.dx + g.dy * m.dy;
    m.proj2 = m.proj * m.proj;
    m.perp2 = fmaxf(diff2 - m.proj2, 0.0f);
    float d2_aniso = g.l1 * m.proj2 + g.l2 * m.perp2;
    float d2_norm = d2_aniso * inv_scale_sq;
    m.d2_safe = fmaxf(d2_norm, 1e-8f);
    return m;
}

// dmix2 = sqrt(d2_safe) - radius * inv_scale, inv_scale = sqrtf(inv_scale_sq)
__device__ __forceinline__ float dmix2(const SiteGeom& g, float ux, float uy, float inv_scale_sq,
                                       float inv_scale) {
    MetricTerms m = metric_terms(g, ux, uy, inv_scale_sq);
    return sqrtf(m.d2_safe) - g.radius * inv_scale;
}

// Item of flat index g in a batch walked as one list: prefix (shared or global) holds the
// first flat index of each of the n_items items and prefix[n_items] the total.
__device__ __forceinline__ uint32_t batch_item_of(const uint32_t* prefix, uint32_t n_items, uint32_t g) {
    uint32_t lo = 0, hi = n_items;  // prefix[lo] <= g < prefix[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (prefix[mid] <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Largest batch of images a batched launch serves (its flat-list prefix is staged in
// shared memory).
constexpr uint32_t kMaxBatchItems = 1024;

// Loads a flat-list prefix (n_items + 1 words) into shared memory; returns the total.
__device__ __forceinline__ uint32_t load_site_prefix(uint32_t* s_prefix, const uint32_t* __restrict__ prefix,
                                                     uint32_t n_items) {
    for (uint32_t k = threadIdx.x; k <= n_items; k += blockDim.x) s_prefix[k] = prefix[k];
    __syncthreads();
    return s_prefix[n_items];
}

__device__ __forceinline__ uint32_t lane_id() {
    uint32_t l;
    asm volatile("mov.u32 %0, %%laneid;" : "=r"(l));
    return l;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Vector reduction to global memory (sm_90+): one L2 atomic for four floats.
__device__ __forceinline__ void red_add_v4(float* addr, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b),
                 "f"(c), "f"(d)
                 : "memory");
}

__device__ __forceinline__ void red_add(float* addr, float a) { atomicAdd(addr, a); }

}  // namespace sad
