// optim.cu -- per-site optimisation: log-tau gradient diffusion, Adam, gradient clears.
//
// Trainer forms keep every iteration-dependent scalar on the device (DevState), so one
// captured CUDA graph per iteration kind is replayed for the whole fit:
//   * tau diffusion: lambda = 0.05 (0.1 + 0.9 iter / iters), the host formula of
//     backends/cuda/src/sad_cuda.cu:2339-2340, evaluated without contraction like an
//     x86 host build would;
//   * Adam: t = iter + 1 (sad_cuda.cu:2369-2380), fused with the gradient clear
//     (adam.cu:183-209) and with the refresh of the prepared SiteGeom/SiteColor records
//     the per-pixel kernels gather.
#include "accum.cuh"
#include "common.cuh"
#include "host_common.h"
#include "kernels.h"

namespace sad {

// ---------------------------------------------------------------------------
// tau diffusion (backends/cuda/src/tau_diffusion.cu:27-89)
// ---------------------------------------------------------------------------
template <class PosFn, class RawFn, class GinFn>
__device__ __forceinline__ float tau_diffuse_one(uint32_t i, const uint4* __restrict__ c0,
                                                 const uint4* __restrict__ c1, PosFn pos,
                                                 RawFn raw, GinFn gin, uint32_t n, float lambda,
                                                 int w, int h, int ds) {
    float2 sp = pos(i);
    if (lambda <= 0.0f || sp.x < 0.0f) return gin(i);
    float inv = 1.0f / fmaxf(static_cast<float>(ds), 1.0f);
    int px = clampi(static_cast<int>(sp.x * inv + 0.5f), 0, w - 1);
    int py = clampi(static_cast<int>(sp.y * inv + 0.5f), 0, h - 1);
    int p = py * w + px;
    uint4 a = __ldg(c0 + p), b = __ldg(c1 + p);
    uint32_t ids[kCand] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    float sum = 0.0f;
    uint32_t cnt = 0;
#pragma unroll
    for (int k = 0; k < kCand; ++k) {
        uint32_t m = ids[k];
        if (m >= n || m == i) continue;
        bool seen = false;
#pragma unroll
        for (int j = 0; j < k; ++j) seen |= ids[j] == m;
        if (seen) continue;
        if (pos(m).x < 0.0f) continue;
        sum += gin(m);
        cnt += 1;
    }
    float diag = 1.0f + lambda * static_cast<float>(cnt);
    return (raw(i) + lambda * sum) / diag;
}

__global__ void tau_diffuse_raw_kernel(const uint4* __restrict__ c0, const uint4* __restrict__ c1,
                                       const Site* __restrict__ sites, const float* __restrict__ raw,
                                       const float* __restrict__ gin, float* __restrict__ gout,
                                       uint32_t n, float lambda, int w, int h, int ds) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    auto pos = [sites](uint32_t k) { return make_float2(__ldg(&sites[k].px), __ldg(&sites[k].py)); };
    auto rawf = [raw](uint32_t k) { return raw[k]; };
    auto ginf = [gin](uint32_t k) { return gin[k]; };
    gout[i] = tau_diffuse_one(i, c0, c1, pos, rawf, ginf, n, lambda, w, h, ds);
}

void launch_tau_diffuse_raw(const uint32_t* c0, const uint32_t* c1, const Site* sites,
                            const float* raw, const float* gin, float* gout, uint32_t n,
                            float lambda, int w, int h, int ds, cudaStream_t st) {
    if (n == 0) return;
    tau_diffuse_raw_kernel<<<blocks_for(n, 256), 256, 0, st>>>(
        reinterpret_cast<const uint4*>(c0), reinterpret_cast<const uint4*>(c1), sites, raw, gin,
        gout, n, lambda, w, h, ds);
    note_launches(1);
}

__device__ __forceinline__ float tau_lambda(uint32_t iter, int iterations) {
    float blend = __fdiv_rn(static_cast<float>(iter), static_cast<float>(max(1, iterations)));
    return __fmul_rn(0.05f, __fadd_rn(0.1f, __fmul_rn(0.9f, blend)));
}

// Trainer form.  The four Jacobi passes of an iteration share one candidate field and one
// set of positions, so the first pass records each active site's neighbour list (the
// distinct active candidates at its texel, in candidate order) and the raw gradient as a
// float; the middle passes read the list; the last pass runs inside the Adam kernel.
// Every pass walks the compacted list of active sites (state->n_alive entries): an
// inactive site's diffused value is never read (a neighbour must be active, and Adam
// skips inactive sites).
struct TauLists {
    uint4* nbr;            // [n][2] neighbour ids, kEmpty-padded
    float* raw;            // [n] raw log-tau gradient (float)
    const uint32_t* alive; // the compacted active list
};

__device__ __forceinline__ void tau_first_one(const uint4* __restrict__ c0, const uint4* __restrict__ c1,
                                              const SiteGeom* __restrict__ geom,
                                              const long long* __restrict__ fix12, const TauLists& tl,
                                              float* __restrict__ gout, uint32_t n, uint32_t i,
                                              float lambda, int w, int h, int ds);

__global__ void tau_first_pass_kernel(const uint4* __restrict__ c0, const uint4* __restrict__ c1,
                                      const SiteGeom* __restrict__ geom,
                                      const long long* __restrict__ fix12, TauLists tl,
                                      float* __restrict__ gout, uint32_t n,
                                      const DevState* __restrict__ state, int iterations, int w,
                                      int h, int ds) {
    pdl_wait();
    const uint32_t n_alive = state->n_alive;
    const float lambda = tau_lambda(state->iter, iterations);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_alive; j += gridDim.x * blockDim.x) {
        const uint32_t i = tl.alive[j];
        tau_first_one(c0, c1, geom, fix12, tl, gout, n, i, lambda, w, h, ds);
    }
}

__device__ __forceinline__ void tau_first_one(const uint4* __restrict__ c0, const uint4* __restrict__ c1,
                                              const SiteGeom* __restrict__ geom,
                                              const long long* __restrict__ fix12, const TauLists& tl,
                                              float* __restrict__ gout, uint32_t n, uint32_t i,
                                              float lambda, int w, int h, int ds) {
    float2 sp = __ldg(reinterpret_cast<const float2*>(geom + i));
    const float r = from_fix(fix12[static_cast<size_t>(i) * 12 + 2]);
    tl.raw[i] = r;
    float inv = 1.0f / fmaxf(static_cast<float>(ds), 1.0f);
    int px = clampi(static_cast<int>(sp.x * inv + 0.5f), 0, w - 1);
    int py = clampi(static_cast<int>(sp.y * inv + 0.5f), 0, h - 1);
    int p = py * w + px;
    uint4 a = __ldg(c0 + p), b = __ldg(c1 + p);
    uint32_t ids[kCand] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    // every candidate's position and raw gradient are fetched before any is used, so the
    // 16 gathers overlap instead of forming a chain of dependent loads
    float cpx[kCand];
    long long cfix[kCand];
#pragma unroll
    for (int k = 0; k < kCand; ++k) {
        const uint32_t m = ids[k];
        const bool ok = m < n && m != i;
        cpx[k] = ok ? __ldg(&geom[m].px) : -1.0f;
        cfix[k] = ok ? fix12[static_cast<size_t>(m) * 12 + 2] : 0ll;
    }
    uint32_t list[kCand];
    float sum = 0.0f;
    uint32_t cnt = 0;
#pragma unroll
    for (int k = 0; k < kCand; ++k) {
        list[k] = kEmpty;
        uint32_t m = ids[k];
        bool take = cpx[k] >= 0.0f;
#pragma unroll
        for (int j = 0; j < k; ++j) take &= ids[j] != m;
        if (take) {
            sum += from_fix(cfix[k]);
            list[k] = m;
            cnt += 1;
        }
    }
    tl.nbr[2 * i] = make_uint4(list[0], list[1], list[2], list[3]);
    tl.nbr[2 * i + 1] = make_uint4(list[4], list[5], list[6], list[7]);
    if (!(lambda > 0.0f)) {
        gout[i] = r;
        return;
    }
    gout[i] = (r + lambda * sum) / (1.0f + lambda * static_cast<float>(cnt));
}

// One Jacobi pass of an active site from its recorded neighbour list (sum in candidate
// order, as the first pass and the reference's kernel).
__device__ __forceinline__ float tau_list_pass(const TauLists& tl, const float* __restrict__ gin,
                                               uint32_t i, float lambda) {
    const float r = tl.raw[i];
    if (!(lambda > 0.0f)) return gin[i];
    uint4 a = tl.nbr[2 * i], b = tl.nbr[2 * i + 1];
    uint32_t ids[kCand] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    float v[kCand];
#pragma unroll
    for (int k = 0; k < kCand; ++k) v[k] = ids[k] == kEmpty ? 0.0f : gin[ids[k]];  // gathers overlap
    float sum = 0.0f;
    uint32_t cnt = 0;
#pragma unroll
    for (int k = 0; k < kCand; ++k) {
        if (ids[k] == kEmpty) continue;
        sum += v[k];
        cnt += 1;
    }
    return (r + lambda * sum) / (1.0f + lambda * static_cast<float>(cnt));
}

__global__ void tau_list_pass_kernel(TauLists tl, const float* __restrict__ gin,
                                     float* __restrict__ gout, const DevState* __restrict__ state,
                                     int iterations) {
    pdl_wait();
    const uint32_t n_alive = state->n_alive;
    const float lambda = tau_lambda(state->iter, iterations);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_alive; j += gridDim.x * blockDim.x) {
        const uint32_t i = tl.alive[j];
        gout[i] = tau_list_pass(tl, gin, i, lambda);
    }
}

void launch_tau_first_pass(const uint32_t* c0, const uint32_t* c1, const SiteGeom* geom,
                           const long long* fix12, uint32_t* nbr, float* raw, const uint32_t* alive,
                           float* gout, uint32_t n, uint32_t max_alive, const DevState* state,
                           int iterations, int w, int h, int ds, cudaStream_t st) {
    if (max_alive == 0) return;
    TauLists tl{reinterpret_cast<uint4*>(nbr), raw, alive};
    launch_pdl(tau_first_pass_kernel, dim3(blocks_for(max_alive, 256)), dim3(256), 0, st,
               reinterpret_cast<const uint4*>(c0), reinterpret_cast<const uint4*>(c1), geom, fix12, tl, gout, n,
               state, iterations, w, h, ds);
    note_launches(1);
}

void launch_tau_list_pass(const uint32_t* nbr, const float* raw, const uint32_t* alive,
                          const float* gin, float* gout, uint32_t max_alive, const DevState* state,
                          int iterations, cudaStream_t st) {
    if (max_alive == 0) return;
    TauLists tl{reinterpret_cast<uint4*>(const_cast<uint32_t*>(nbr)), const_cast<float*>(raw), alive};
    launch_pdl(tau_list_pass_kernel, dim3(blocks_for(max_alive, 256)), dim3(256), 0, st, tl, gin, gout, state,
               iterations);
    note_launches(1);
}

// ---------------------------------------------------------------------------
// Adam (backends/cuda/src/adam.cu:5-180)
// ---------------------------------------------------------------------------
struct AdamSlots {  // the 20-float per-site state
    float v[20];
};

__device__ __forceinline__ void adam_load(const float* __restrict__ a, uint32_t i, AdamSlots& s) {
    const float4* q = reinterpret_cast<const float4*>(a + static_cast<size_t>(i) * 20);
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        float4 t = q[k];
        s.v[4 * k] = t.x; s.v[4 * k + 1] = t.y; s.v[4 * k + 2] = t.z; s.v[4 * k + 3] = t.w;
    }
}

__device__ __forceinline__ void adam_store(float* __restrict__ a, uint32_t i, const AdamSlots& s) {
    float4* q = reinterpret_cast<float4*>(a + static_cast<size_t>(i) * 20);
#pragma unroll
    for (int k = 0; k < 5; ++k)
        q[k] = make_float4(s.v[4 * k], s.v[4 * k + 1], s.v[4 * k + 2], s.v[4 * k + 3]);
}

// One Adam step of one active site.  g[] = the 10 normalised gradients in site order.
__device__ __forceinline__ void adam_site(Site& s, AdamSlots& a, const float (&g)[10],
                                          const AdamHyper& hp, float c1, float c2, int w, int h) {
    const float b1 = hp.beta1, b2 = hp.beta2, eps = hp.eps;
    // position: isotropic Adam
    a.v[0] = b1 * a.v[0] + (1.0f - b1) * g[0];
    a.v[1] = b1 * a.v[1] + (1.0f - b1) * g[1];
    float g2p = g[0] * g[0] + g[1] * g[1];
    a.v[2] = b2 * a.v[2] + (1.0f - b2) * g2p;
    {
        float mh0 = a.v[0] * c1, mh1 = a.v[1] * c1;
        float vh = a.v[2] * c2;
        float idn = 1.0f / (sqrtf(vh) + eps);
        float st0 = hp.lr_pos * mh0 * idn, st1 = hp.lr_pos * mh1 * idn;
        s.px -= st0;
        s.py -= st1;
        s.px = clampf(s.px, 0.0f, static_cast<float>(w - 1));
        s.py = clampf(s.py, 0.0f, static_cast<float>(h - 1));
    }
    // log_tau
    a.v[3] = b1 * a.v[3] + (1.0f - b1) * g[2];
    a.v[4] = b2 * a.v[4] + (1.0f - b2) * (g[2] * g[2]);
    s.log_tau -= hp.lr_tau * (a.v[3] * c1) / (sqrtf(a.v[4] * c2) + eps);
    // radius
    a.v[5] = b1 * a.v[5] + (1.0f - b1) * g[3];
    a.v[6] = b2 * a.v[6] + (1.0f - b2) * (g[3] * g[3]);
    s.radius -= hp.lr_radius * (a.v[5] * c1) / (sqrtf(a.v[6] * c2) + eps);
    s.radius = clampf(s.radius, 1.0f, 512.0f);
    // colour, per channel
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        a.v[7 + c] = b1 * a.v[7 + c] + (1.0f - b1) * g[4 + c];
        a.v[10 + c] = b2 * a.v[10 + c] + (1.0f - b2) * (g[4 + c] * g[4 + c]);
    }
    float st_r = hp.lr_color * (a.v[7] * c1) / (sqrtf(a.v[10] * c2) + eps);
    float st_g = hp.lr_color * (a.v[8] * c1) / (sqrtf(a.v[11] * c2) + eps);
    float st_b = hp.lr_color * (a.v[9] * c1) / (sqrtf(a.v[12] * c2) + eps);
    s.r = clampf(s.r - st_r, 0.0f, 1.0f);
    s.g = clampf(s.g - st_g, 0.0f, 1.0f);
    s.b = clampf(s.b - st_b, 0.0f, 1.0f);
    // direction: tangent-space isotropic Adam, renormalised
    {
        float dx = s.dx, dy = s.dy;
        float gd = g[7] * dx + g[8] * dy;
        float gtx = g[7] - dx * gd, gty = g[8] - dy * gd;
        a.v[13] = b1 * a.v[13] + (1.0f - b1) * gtx;
        a.v[14] = b1 * a.v[14] + (1.0f - b1) * gty;
        float g2d = gtx * gtx + gty * gty;
        a.v[15] = b2 * a.v[15] + (1.0f - b2) * g2d;
        float mh0 = a.v[13] * c1, mh1 = a.v[14] * c1;
        float vh = a.v[15] * c2;
        float idn = 1.0f / (sqrtf(vh) + eps);
        float nx = dx - hp.lr_dir * mh0 * idn, ny = dy - hp.lr_dir * mh1 * idn;
        float l2 = nx * nx + ny * ny;
        if (l2 < 1e-12f) {
            nx = 1.0f;
            ny = 0.0f;
        } else {
            float il = rsqrtf(l2);
            nx *= il;
            ny *= il;
        }
        s.dx = nx;
        s.dy = ny;
    }
    // log_aniso
    a.v[16] = b1 * a.v[16] + (1.0f - b1) * g[9];
    a.v[17] = b2 * a.v[17] + (1.0f - b2) * (g[9] * g[9]);
    s.log_aniso -= hp.lr_aniso * (a.v[16] * c1) / (sqrtf(a.v[17] * c2) + eps);
    s.log_aniso = clampf(s.log_aniso, -4.0f, 4.0f);
}

__device__ __forceinline__ Site site_load(const Site* __restrict__ sites, uint32_t i) {
    const float2* q = reinterpret_cast<const float2*>(sites + i);
    float2 a = q[0], b = q[1], c = q[2], d = q[3], e = q[4];
    Site s;
    s.px = a.x; s.py = a.y; s.log_tau = b.x; s.radius = b.y; s.r = c.x; s.g = c.y;
    s.b = d.x; s.dx = d.y; s.dy = e.x; s.log_aniso = e.y;
    return s;
}

__device__ __forceinline__ void site_store(Site* __restrict__ sites, uint32_t i, const Site& s) {
    float2* q = reinterpret_cast<float2*>(sites + i);
    q[0] = make_float2(s.px, s.py);
    q[1] = make_float2(s.log_tau, s.radius);
    q[2] = make_float2(s.r, s.g);
    q[3] = make_float2(s.b, s.dx);
    q[4] = make_float2(s.dy, s.log_aniso);
}

struct SoaGrads {
    const float* g[10];
};

__global__ void adam_soa_kernel(Site* __restrict__ sites, float* __restrict__ adam, SoaGrads gr,
                                AdamHyper hp, uint32_t t, uint32_t n, int w, int h) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float norm = 1.0f / static_cast<float>(w * h);
    float g[10];
#pragma unroll
    for (int k = 0; k < 10; ++k) g[k] = gr.g[k][i] * norm;
    Site s = site_load(sites, i);
    if (s.px < 0.0f) return;
    float tt = static_cast<float>(t);
    float c1 = 1.0f / (1.0f - powf(hp.beta1, tt));
    float c2 = 1.0f / (1.0f - powf(hp.beta2, tt));
    AdamSlots a;
    adam_load(adam, i, a);
    adam_site(s, a, g, hp, c1, c2, w, h);
    adam_store(adam, i, a);
    site_store(sites, i, s);
}

void launch_adam_soa(Site* sites, float* adam, const float* const g[10], const AdamHyper& hp,
                     uint32_t t, uint32_t n, int w, int h, cudaStream_t st) {
    if (n == 0) return;
    SoaGrads gr;
    for (int k = 0; k < 10; ++k) gr.g[k] = g[k];
    adam_soa_kernel<<<blocks_for(n, 256), 256, 0, st>>>(sites, adam, gr, hp, t, n, w, h);
    note_launches(1);
}

// Trainer form: the last tau Jacobi pass, then Adam on the fixed-point gradient records,
// which are consumed and cleared (slots 0-9; slots 10-11, the removal delta, belong to the
// prune step), then the refreshed SiteGeom / SiteColor records.  Inactive sites carry no
// gradient and are left untouched.
__device__ __forceinline__ void adam_train_one(Site* __restrict__ sites, float* __restrict__ adam,
                                               long long* __restrict__ fix12, const TauLists& tl,
                                               const float* __restrict__ tau_gin, SiteGeom* __restrict__ geom,
                                               SiteColor* __restrict__ color, const AdamHyper& hp,
                                               const DevState* __restrict__ state, int iterations, int w, int h,
                                               uint32_t i);

__global__ void adam_train_kernel(Site* __restrict__ sites, float* __restrict__ adam,
                                  long long* __restrict__ fix12, TauLists tl,
                                  const float* __restrict__ tau_gin, SiteGeom* __restrict__ geom,
                                  SiteColor* __restrict__ color, AdamHyper hp,
                                  const DevState* __restrict__ state, int iterations, int w, int h) {
    pdl_wait();
    const uint32_t n_alive = state->n_alive;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_alive; j += gridDim.x * blockDim.x)
        adam_train_one(sites, adam, fix12, tl, tau_gin, geom, color, hp, state, iterations, w, h, tl.alive[j]);
}

__device__ __forceinline__ void adam_train_one(Site* __restrict__ sites, float* __restrict__ adam,
                                               long long* __restrict__ fix12, const TauLists& tl,
                                               const float* __restrict__ tau_gin, SiteGeom* __restrict__ geom,
                                               SiteColor* __restrict__ color, const AdamHyper& hp,
                                               const DevState* __restrict__ state, int iterations, int w, int h,
                                               uint32_t i) {
    const float tau_g = tau_list_pass(tl, tau_gin, i, tau_lambda(state->iter, iterations));
    float norm = 1.0f / static_cast<float>(w * h);
    longlong2* gq = reinterpret_cast<longlong2*>(fix12 + static_cast<size_t>(i) * 12);
    longlong2 q[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) q[k] = gq[k];
#pragma unroll
    for (int k = 0; k < 5; ++k) gq[k] = make_longlong2(0, 0);
    float g[10] = {from_fix(q[0].x) * norm, from_fix(q[0].y) * norm, tau_g * norm,
                   from_fix(q[1].y) * norm, from_fix(q[2].x) * norm, from_fix(q[2].y) * norm,
                   from_fix(q[3].x) * norm, from_fix(q[3].y) * norm, from_fix(q[4].x) * norm,
                   from_fix(q[4].y) * norm};
    Site s = site_load(sites, i);
    const float c1 = state->adam_c1, c2 = state->adam_c2;
    AdamSlots a;
    adam_load(adam, i, a);
    adam_site(s, a, g, hp, c1, c2, w, h);
    adam_store(adam, i, a);
    site_store(sites, i, s);
    store_geom(geom, i, make_geom(s.px, s.py, s.log_tau, s.radius, s.dx, s.dy, s.log_aniso));
    reinterpret_cast<float4*>(color)[i] = make_float4(s.r, s.g, s.b, 0.0f);
}

void launch_adam_train(Site* sites, float* adam, long long* fix12, const uint32_t* nbr,
                       const float* raw, const uint32_t* alive, const float* tau_gin,
                       SiteGeom* geom, SiteColor* color, const AdamHyper& hp,
                       const DevState* state, int iterations, uint32_t max_alive, int w, int h,
                       cudaStream_t st) {
    if (max_alive == 0) return;
    TauLists tl{reinterpret_cast<uint4*>(const_cast<uint32_t*>(nbr)), const_cast<float*>(raw), alive};
    launch_pdl(adam_train_kernel, dim3(blocks_for(max_alive, 256)), dim3(256), 0, st, sites, adam, fix12, tl,
               tau_gin, geom, color, hp, state, iterations, w, h);
    note_launches(1);
}

// ---------------------------------------------------------------------------
// clears and the iteration counter
// ---------------------------------------------------------------------------
__global__ void clear_f32_kernel(float* __restrict__ buf, size_t count) {
    size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
    size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (; i < count; i += stride) buf[i] = 0.0f;
}

void launch_clear_f32(float* buf, size_t count, cudaStream_t st) {
    if (count == 0) return;
    unsigned blocks = static_cast<unsigned>(std::min<size_t>((count + 255) / 256, 152 * 16));
    clear_f32_kernel<<<blocks, 256, 0, st>>>(buf, count);
    note_launches(1);
}

__global__ void clear10_kernel(SoaGrads g, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
#pragma unroll
    for (int k = 0; k < 10; ++k) const_cast<float*>(g.g[k])[i] = 0.0f;
}

__device__ __forceinline__ void set_bias_corrections(DevState* state, float beta1, float beta2) {
    float tt = static_cast<float>(state->iter + 1u);  // Adam step t = iter + 1
    state->adam_c1 = 1.0f / (1.0f - powf(beta1, tt));
    state->adam_c2 = 1.0f / (1.0f - powf(beta2, tt));
}

__global__ void reset_state_kernel(DevState* state, float beta1, float beta2) {
    state->iter = 0u;
    state->vpt_pass = 0u;
    state->wide_far_refs = kWideFarRefs;
    set_bias_corrections(state, beta1, beta2);
}

__global__ void advance_state_kernel(DevState* state, uint32_t vpt_passes, float beta1, float beta2) {
    pdl_wait();
    state->iter += 1u;
    state->vpt_pass += vpt_passes;
    set_bias_corrections(state, beta1, beta2);
}

void launch_reset_state(DevState* state, float beta1, float beta2, cudaStream_t st) {
    reset_state_kernel<<<1, 1, 0, st>>>(state, beta1, beta2);
    note_launches(1);
}

__global__ void set_wide_far_refs_kernel(DevState* state, int value) { state->wide_far_refs = value; }

void launch_set_wide_far_refs(DevState* state, int value, cudaStream_t st) {
    set_wide_far_refs_kernel<<<1, 1, 0, st>>>(state, value);
    note_launches(1);
}

void launch_advance_state(DevState* state, uint32_t vpt_passes, float beta1, float beta2,
                          cudaStream_t st) {
    launch_pdl(advance_state_kernel, dim3(1), dim3(1), 0, st, state, vpt_passes, beta1, beta2);
    note_launches(1);
}

// ---------------------------------------------------------------------------
// batched forms: every image of a batch in one launch, over the flat active list
// ---------------------------------------------------------------------------
__global__ void batch_site_prefix_kernel(const SiteBatchItem* __restrict__ items, uint32_t n_items,
                                         uint32_t* __restrict__ prefix) {
    pdl_wait();
    if (threadIdx.x != 0) return;
    uint32_t run = 0;
    for (uint32_t i = 0; i < n_items; ++i) {
        prefix[i] = run;
        run += items[i].state->n_alive;
    }
    prefix[n_items] = run;
}

void launch_batch_site_prefix(const SiteBatchItem* items, uint32_t n_items, uint32_t* site_prefix, cudaStream_t st) {
    launch_pdl(batch_site_prefix_kernel, dim3(1), dim3(32), 0, st, items, n_items, site_prefix);
    note_launches(1);
}

__global__ void __launch_bounds__(256) tau_first_batch_kernel(const SiteBatchItem* __restrict__ items,
                                                              const uint32_t* __restrict__ prefix,
                                                              uint32_t n_items, int field, int iterations) {
    pdl_wait();
    __shared__ uint32_t s_prefix[kMaxBatchItems + 1];
    const uint32_t total = load_site_prefix(s_prefix, prefix, n_items);
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const uint32_t k = batch_item_of(s_prefix, n_items, g);
        const SiteBatchItem& it = items[k];
        TauLists tl{reinterpret_cast<uint4*>(it.tau_nbr), it.tau_raw, it.alive};
        const uint32_t i = it.alive[g - s_prefix[k]];
        tau_first_one(reinterpret_cast<const uint4*>(it.cand0[field]), reinterpret_cast<const uint4*>(it.cand1[field]),
                      it.geom, it.grads, tl, it.tau_a, it.n, i, tau_lambda(it.state->iter, iterations), it.cw,
                      it.ch, it.ds);
    }
}

__global__ void __launch_bounds__(256) tau_list_batch_kernel(const SiteBatchItem* __restrict__ items,
                                                             const uint32_t* __restrict__ prefix,
                                                             uint32_t n_items, int a_to_b, int iterations) {
    pdl_wait();
    __shared__ uint32_t s_prefix[kMaxBatchItems + 1];
    const uint32_t total = load_site_prefix(s_prefix, prefix, n_items);
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const uint32_t k = batch_item_of(s_prefix, n_items, g);
        const SiteBatchItem& it = items[k];
        TauLists tl{reinterpret_cast<uint4*>(it.tau_nbr), it.tau_raw, it.alive};
        const uint32_t i = it.alive[g - s_prefix[k]];
        const float* gin = a_to_b ? it.tau_a : it.tau_b;
        float* gout = a_to_b ? it.tau_b : it.tau_a;
        gout[i] = tau_list_pass(tl, gin, i, tau_lambda(it.state->iter, iterations));
    }
}

__global__ void __launch_bounds__(256) adam_batch_kernel(const SiteBatchItem* __restrict__ items,
                                                         const uint32_t* __restrict__ prefix, uint32_t n_items,
                                                         AdamHyper hp, int iterations) {
    pdl_wait();
    __shared__ uint32_t s_prefix[kMaxBatchItems + 1];
    const uint32_t total = load_site_prefix(s_prefix, prefix, n_items);
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const uint32_t k = batch_item_of(s_prefix, n_items, g);
        const SiteBatchItem& it = items[k];
        TauLists tl{reinterpret_cast<uint4*>(it.tau_nbr), it.tau_raw, it.alive};
        adam_train_one(it.sites, it.adam, it.grads, tl, it.tau_a, it.geom, it.color, hp, it.state, iterations, it.w,
                       it.h, it.alive[g - s_prefix[k]]);
    }
}

__global__ void advance_state_batch_kernel(const SiteBatchItem* __restrict__ items, uint32_t n_items,
                                           uint32_t vpt_passes, float beta1, float beta2) {
    pdl_wait();
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_items) return;
    DevState* state = items[k].state;
    state->iter += 1u;
    state->vpt_pass += vpt_passes;
    set_bias_corrections(state, beta1, beta2);
}

static unsigned batch_grid(uint32_t grid_threads) { return std::max(1u, blocks_for(grid_threads, 256)); }

void launch_tau_first_batch(const SiteBatchItem* items, const uint32_t* site_prefix, uint32_t n_items, int field,
                            int iterations, uint32_t grid_threads, cudaStream_t st) {
    launch_pdl(tau_first_batch_kernel, dim3(batch_grid(grid_threads)), dim3(256), 0, st, items, site_prefix, n_items,
               field, iterations);
    note_launches(1);
}

void launch_tau_list_batch(const SiteBatchItem* items, const uint32_t* site_prefix, uint32_t n_items, bool a_to_b,
                           int iterations, uint32_t grid_threads, cudaStream_t st) {
    launch_pdl(tau_list_batch_kernel, dim3(batch_grid(grid_threads)), dim3(256), 0, st, items, site_prefix, n_items,
               a_to_b ? 1 : 0, iterations);
    note_launches(1);
}

void launch_adam_batch(const SiteBatchItem* items, const uint32_t* site_prefix, uint32_t n_items,
                       const AdamHyper& hp, int iterations, uint32_t grid_threads, cudaStream_t st) {
    launch_pdl(adam_batch_kernel, dim3(batch_grid(grid_threads)), dim3(256), 0, st, items, site_prefix, n_items, hp,
               iterations);
    note_launches(1);
}

void launch_advance_state_batch(const SiteBatchItem* items, uint32_t n_items, uint32_t vpt_passes, float beta1,
                                float beta2, cudaStream_t st) {
    launch_pdl(advance_state_batch_kernel, dim3(blocks_for(n_items, 128)), dim3(128), 0, st, items, n_items,
               vpt_passes, beta1, beta2);
    note_launches(1);
}

}  // namespace sad

using namespace sad;

extern "C" sad_status_t sad_tau_diffuse(const uint32_t* cand0, const uint32_t* cand1,
                                        const float* sites, const float* grad_raw,
                                        const float* grad_in, float* grad_out, uint32_t site_count,
                                        float lambda, int width, int height, int cand_downscale,
                                        sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_tau_diffuse: invalid cand size");
    SAD_REQUIRE(site_count == 0 || (cand0 && cand1 && sites && grad_raw && grad_in && grad_out),
                "sad_tau_diffuse: null buffer");
    SAD_REQUIRE(grad_in != grad_out, "sad_tau_diffuse: grad_in and grad_out must differ");
    launch_tau_diffuse_raw(cand0, cand1, reinterpret_cast<const Site*>(sites), grad_raw, grad_in,
                           grad_out, site_count, lambda, width, height, cand_downscale,
                           as_stream(stream));
    return check_launch("sad_tau_diffuse");
}

extern "C" sad_status_t sad_adam_update(float* sites, float* adam, const float* gpx,
                                        const float* gpy, const float* glt, const float* grad,
                                        const float* gr, const float* gg, const float* gb,
                                        const float* gdx, const float* gdy, const float* gla,
                                        float lr_pos, float lr_tau, float lr_radius,
                                        float lr_color, float lr_dir, float lr_aniso, float beta1,
                                        float beta2, float eps, uint32_t t, uint32_t site_count,
                                        int width, int height, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(image_size_ok(width, height), "sad_adam_update: invalid image size");
    SAD_REQUIRE(site_count == 0 || (sites && adam && gpx && gpy && glt && grad && gr && gg && gb &&
                                    gdx && gdy && gla),
                "sad_adam_update: null buffer");
    SAD_REQUIRE((reinterpret_cast<uintptr_t>(adam) & 15u) == 0, "sad_adam_update: adam must be 16-byte aligned");
    AdamHyper hp{lr_pos, lr_tau, lr_radius, lr_color, lr_dir, lr_aniso, beta1, beta2, eps};
    const float* g[10] = {gpx, gpy, glt, grad, gr, gg, gb, gdx, gdy, gla};
    launch_adam_soa(reinterpret_cast<Site*>(sites), adam, g, hp, t, site_count, width, height,
                    as_stream(stream));
    return check_launch("sad_adam_update");
}

extern "C" sad_status_t sad_clear_gradients(float* g0, float* g1, float* g2, float* g3, float* g4,
                                            float* g5, float* g6, float* g7, float* g8, float* g9,
                                            uint32_t count, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(count == 0 || (g0 && g1 && g2 && g3 && g4 && g5 && g6 && g7 && g8 && g9),
                "sad_clear_gradients: null buffer");
    if (count == 0) return SAD_OK;
    SoaGrads g{{g0, g1, g2, g3, g4, g5, g6, g7, g8, g9}};
    clear10_kernel<<<blocks_for(count, 256), 256, 0, as_stream(stream)>>>(g, count);
    note_launches(1);
    return check_launch("sad_clear_gradients");
}

extern "C" sad_status_t sad_clear_buffer(float* buffer, uint32_t count, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(count == 0 || buffer, "sad_clear_buffer: null buffer");
    launch_clear_f32(buffer, count, as_stream(stream));
    return check_launch("sad_clear_buffer");
}
