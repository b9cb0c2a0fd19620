/*
 * sad_oracle.c -- CPU restatement of SAD's fit-and-render path.
 *
 * TEST INFRASTRUCTURE ONLY (see sad_oracle.h).  Each function follows the
 * reference kernel or host routine named in its comment; file:line refer to the
 * LuckyIYI/SAD project tree.  Written as plain loops: clarity over speed, except
 * for the parts the timed CPU baseline runs (render, gradients, VPT, per-site
 * updates), which use OpenMP over pixel rows / tiles.
 */
#include "sad_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define EMPTY ORC_EMPTY
#define K ORC_K

static inline int clampi(int x, int a, int b) { return x < a ? a : (x > b ? b : x); }
static inline float clampf(float x, float a, float b) { return fmaxf(a, fminf(b, x)); }
static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* scalar helpers                                                            */
/* ------------------------------------------------------------------------ */

/* IEEE binary16 round-to-nearest-even, the rounding __float2half performs
 * (used by backends/cuda/src/candidate_pack.cu:21-25). */
uint16_t orc_f32_to_f16(float f) {
    uint32_t x = f2u(f);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t ax = x & 0x7fffffffu;
    if (ax > 0x7f800000u) return (uint16_t)(sign | 0x7e00u);
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);
    if (ax >= 0x38800000u) {
        uint32_t mant = ax & 0x7fffffu;
        uint32_t e = (ax >> 23) - 127u + 15u;
        uint32_t h = (e << 10) | (mant >> 13);
        uint32_t rem = mant & 0x1fffu;
        if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h += 1u;
        return (uint16_t)(sign | h);
    }
    if (ax < 0x33000000u) return (uint16_t)sign;
    {
        uint32_t e = ax >> 23;
        uint32_t mant = (ax & 0x7fffffu) | 0x800000u;
        uint32_t shift = 126u - e;
        uint32_t h = mant >> shift;
        uint32_t rem = mant & ((1u << shift) - 1u);
        uint32_t half = 1u << (shift - 1u);
        if (rem > half || (rem == half && (h & 1u))) h += 1u;
        return (uint16_t)(sign | h);
    }
}

float orc_f16_to_f32(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1fu;
    uint32_t m = h & 0x3ffu;
    uint32_t out;
    if (e == 0) {
        if (m == 0) {
            out = sign;
        } else {
            float v = (float)m * (1.0f / 16777216.0f);
            out = f2u(v) | sign;
        }
    } else if (e == 31) {
        out = sign | 0x7f800000u | (m << 13);
    } else {
        out = sign | ((e - 15u + 127u) << 23) | (m << 13);
    }
    float f;
    memcpy(&f, &out, 4);
    return f;
}

/* backends/cuda/src/sad_common.cuh:128-133 */
uint32_t orc_xorshift32(uint32_t x) {
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    return x;
}

static inline float orc_rand01(uint32_t* state) {
    *state = orc_xorshift32(*state);
    return (float)(*state) * (1.0f / 4294967296.0f);
}

/* backends/cuda/src/sad_cuda.cu:1157-1178 */
uint32_t orc_jump_step_for_index(uint32_t step_index, int width, int height) {
    uint32_t max_dim = (uint32_t)(width > height ? width : height);
    uint32_t pow2 = 1;
    while (pow2 < max_dim) pow2 <<= 1;
    if (pow2 <= 1) return 1;
    uint32_t stages = 0, tmp = pow2;
    while (tmp > 1) { tmp >>= 1; stages++; }
    uint32_t stage = step_index >= stages ? stages - 1 : step_index;
    uint32_t step = pow2 >> (stage + 1);
    return step > 1u ? step : 1u;
}

/* backends/cuda/src/sad_cuda.cu:1180-1183 */
uint32_t orc_pack_jump_step(uint32_t step_index, int width, int height) {
    uint32_t j = orc_jump_step_for_index(step_index, width, height);
    if (j > 0xffffu) j = 0xffffu;
    return (j << 16) | (step_index & 0xffffu);
}

/* backends/cuda/src/sad_cuda.cu:1512-1545 */
uint32_t orc_hilbert_index(uint32_t x, uint32_t y, int bits) {
    uint32_t xi = x, yi = y, index = 0;
    uint32_t mask = bits >= 32 ? 0xffffffffu : ((1u << bits) - 1u);
    for (int i = bits - 1; i >= 0; --i) {
        uint32_t s = (uint32_t)i;
        uint32_t rx = (xi >> s) & 1u, ry = (yi >> s) & 1u;
        uint32_t d = (3u * rx) ^ ry;
        index |= d << (2u * s);
        if (ry == 0u) {
            if (rx == 1u) { xi = mask - xi; yi = mask - yi; }
            uint32_t t = xi; xi = yi; yi = t;
        }
    }
    return index;
}

/* backends/cuda/src/sad_cuda.cu:1501-1510 */
int orc_hilbert_bits_for_size(int width, int height) {
    int m = width > height ? width : height;
    int n = 1, bits = 0;
    while (n < m) { n <<= 1; bits++; }
    return bits > 1 ? bits : 1;
}

/* backends/cuda/src/sad_common.cuh:141-165 (voronoi_dmix2) */
float orc_dmix2(const orc_site* s, float ux, float uy, float inv_scale_sq) {
    float dx = ux - s->px, dy = uy - s->py;
    float diff2 = dx * dx + dy * dy;
    float proj = s->dx * dx + s->dy * dy;
    float proj2 = proj * proj;
    float perp2 = fmaxf(diff2 - proj2, 0.0f);
    float l1 = expf(s->log_aniso);
    float l2 = 1.0f / l1;
    float d2a = l1 * proj2 + l2 * perp2;
    float d2n = d2a * inv_scale_sq;
    float d2s = fmaxf(d2n, 1e-8f);
    float inv_scale = sqrtf(inv_scale_sq);
    float rn = s->radius * inv_scale;
    return sqrtf(d2s) - rn;
}

static double orc_dmix2_d(const orc_site_d* s, double ux, double uy, double inv_scale_sq) {
    double dx = ux - s->px, dy = uy - s->py;
    double diff2 = dx * dx + dy * dy;
    double proj = s->dx * dx + s->dy * dy;
    double proj2 = proj * proj;
    double perp2 = fmax(diff2 - proj2, 0.0);
    double l1 = exp(s->log_aniso);
    double l2 = 1.0 / l1;
    double d2n = (l1 * proj2 + l2 * perp2) * inv_scale_sq;
    double d2s = fmax(d2n, 1e-8);
    return sqrt(d2s) - s->radius * sqrt(inv_scale_sq);
}

/* backends/cuda/src/sad_common.cuh:113-125 */
static inline int cand_index_for_pixel(int x, int y, int w, int h, int cw, int ch) {
    int sw = w > 0 ? w : 1, sh = h > 0 ? h : 1;
    int cx = clampi((x * cw) / sw, 0, cw - 1);
    int cy = clampi((y * ch) / sh, 0, ch - 1);
    return cy * cw + cx;
}

static inline void load_cands(const uint32_t* c0, const uint32_t* c1, int ci, uint32_t ids[K]) {
    for (int i = 0; i < 4; i++) { ids[i] = c0[ci * 4 + i]; ids[4 + i] = c1[ci * 4 + i]; }
}

/* ------------------------------------------------------------------------ */
/* render and adjoint                                                        */
/* ------------------------------------------------------------------------ */

/* backends/cuda/src/render.cu:5-92 (renderVoronoiKernel) */
void orc_render(const uint32_t* cand0, const uint32_t* cand1, const orc_site* sites,
                uint32_t n, int w, int h, int cw, int ch, float inv_s2, float* out) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            int p = y * w + x;
            float ux = (float)x, uy = (float)y;
            uint32_t ids[K];
            load_cands(cand0, cand1, cand_index_for_pixel(x, y, w, h, cw, ch), ids);
            float logits[K], mx = -INFINITY;
            for (int i = 0; i < K; i++) {
                uint32_t id = ids[i];
                if (id >= n || sites[id].px < 0.0f) { logits[i] = -INFINITY; continue; }
                float tau = expf(sites[id].log_tau);
                logits[i] = -tau * orc_dmix2(&sites[id], ux, uy, inv_s2);
                mx = fmaxf(mx, logits[i]);
            }
            if (isinf(mx) && mx < 0.0f) {
                out[3 * p] = out[3 * p + 1] = out[3 * p + 2] = 0.0f;
                continue;
            }
            float wts[K], sum = 0.0f;
            for (int i = 0; i < K; i++) { wts[i] = expf(logits[i] - mx); sum += wts[i]; }
            float inv = 1.0f / fmaxf(sum, 1e-8f);
            float r = 0.0f, g = 0.0f, b = 0.0f;
            for (int i = 0; i < K; i++) {
                float wi = wts[i] * inv;
                uint32_t id = ids[i];
                if (!isnan(wi) && !isinf(wi) && id < n && sites[id].px >= 0.0f) {
                    r += wi * sites[id].r; g += wi * sites[id].g; b += wi * sites[id].b;
                }
            }
            out[3 * p] = r; out[3 * p + 1] = g; out[3 * p + 2] = b;
        }
    }
}

/* Same forward in double, candidate field at full resolution (FP64 gradcheck). */
void orc_render_d(const uint32_t* cand0, const uint32_t* cand1, const orc_site_d* sites,
                  uint32_t n, int w, int h, double inv_s2, double* out) {
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            int p = y * w + x;
            uint32_t ids[K];
            load_cands(cand0, cand1, p, ids);
            double logits[K], mx = -INFINITY;
            for (int i = 0; i < K; i++) {
                uint32_t id = ids[i];
                if (id >= n || sites[id].px < 0.0) { logits[i] = -INFINITY; continue; }
                logits[i] = -exp(sites[id].log_tau) * orc_dmix2_d(&sites[id], x, y, inv_s2);
                mx = fmax(mx, logits[i]);
            }
            if (isinf(mx) && mx < 0.0) { out[3 * p] = out[3 * p + 1] = out[3 * p + 2] = 0.0; continue; }
            double wts[K], sum = 0.0;
            for (int i = 0; i < K; i++) { wts[i] = exp(logits[i] - mx); sum += wts[i]; }
            double inv = 1.0 / fmax(sum, 1e-8);
            double r = 0, g = 0, b = 0;
            for (int i = 0; i < K; i++) {
                double wi = wts[i] * inv;
                uint32_t id = ids[i];
                if (id < n && sites[id].px >= 0.0) { r += wi * sites[id].r; g += wi * sites[id].g; b += wi * sites[id].b; }
            }
            out[3 * p] = r; out[3 * p + 1] = g; out[3 * p + 2] = b;
        }
    }
}

/* backends/pytorch/torch_ext/cuda/sad_bindings.cu:41-98 (compute_candidate_weights_raw) */
static int weights_raw(const uint32_t ids[K], const orc_site* sites, uint32_t n, float ux, float uy,
                       float inv_s2, float wts[K], float pred[3]) {
    float logits[K], mx = -INFINITY;
    int any = 0;
    for (int i = 0; i < K; i++) {
        uint32_t id = ids[i];
        if (id >= n || sites[id].px < 0.0f) { logits[i] = -INFINITY; continue; }
        float tau = expf(sites[id].log_tau);
        logits[i] = -tau * orc_dmix2(&sites[id], ux, uy, inv_s2);
        mx = fmaxf(mx, logits[i]);
        any = 1;
    }
    if (!any || isinf(mx)) return 0;
    float sum = 0.0f;
    for (int i = 0; i < K; i++) { wts[i] = expf(logits[i] - mx); sum += wts[i]; }
    float inv = 1.0f / fmaxf(sum, 1e-8f);
    pred[0] = pred[1] = pred[2] = 0.0f;
    for (int i = 0; i < K; i++) {
        wts[i] *= inv;
        uint32_t id = ids[i];
        if (id < n && sites[id].px >= 0.0f) {
            pred[0] += wts[i] * sites[id].r; pred[1] += wts[i] * sites[id].g; pred[2] += wts[i] * sites[id].b;
        }
    }
    return 1;
}

/* Per-candidate parameter gradients given dL/dpred, shared by the autograd
 * adjoint (sad_bindings.cu:135-193, l2 = 1/l1) and the fused training kernel
 * (gradients.cu:352-420, l2 = 1/max(l1,1e-8)). Output order = site layout. */
static void site_param_grads(const orc_site* s, float ux, float uy, float inv_s2, float w,
                             const float dLdp[3], const float pred[3], int clamp_l1, float g[10]) {
    float dldc0 = w * dLdp[0], dldc1 = w * dLdp[1], dldc2 = w * dLdp[2];
    float dlogit = dLdp[0] * (w * (s->r - pred[0])) + dLdp[1] * (w * (s->g - pred[1])) +
                   dLdp[2] * (w * (s->b - pred[2]));
    float tau = expf(s->log_tau);
    float dx = ux - s->px, dy = uy - s->py;
    float diff2 = dx * dx + dy * dy;
    float proj = s->dx * dx + s->dy * dy;
    float proj2 = proj * proj;
    float perp2 = fmaxf(diff2 - proj2, 0.0f);
    float l1 = expf(s->log_aniso);
    float l2 = clamp_l1 ? 1.0f / fmaxf(l1, 1e-8f) : 1.0f / l1;
    float d2n = (l1 * proj2 + l2 * perp2) * inv_s2;
    float d2s = fmaxf(d2n, 1e-8f);
    float isq = 1.0f / sqrtf(d2s);
    float inv_scale = sqrtf(inv_s2);
    float dmix2 = sqrtf(d2s) - s->radius * inv_scale;
    float gdx = l2 * dx + (l1 - l2) * s->dx * proj;
    float gdy = l2 * dy + (l1 - l2) * s->dy * proj;
    float kpos = tau * inv_s2 * isq;
    g[0] = dlogit * kpos * gdx;
    g[1] = dlogit * kpos * gdy;
    g[2] = dlogit * (-dmix2) * tau;
    g[3] = dlogit * tau * inv_scale;
    g[4] = dldc0; g[5] = dldc1; g[6] = dldc2;
    float dla = (l1 * proj2 - l2 * perp2) * inv_s2;
    float kdir = 2.0f * (l1 - l2) * proj * inv_s2;
    float kang = dlogit * (-tau) * (0.5f * isq);
    g[7] = kang * (kdir * dx);
    g[8] = kang * (kdir * dy);
    g[9] = kang * dla;
}

/* backends/pytorch/torch_ext/cuda/sad_bindings.cu:100-207 (render_sad_backward_kernel) */
void orc_render_backward(const uint32_t* cand0, const uint32_t* cand1, const orc_site* sites,
                         uint32_t n, int w, int h, int cw, int ch, float inv_s2,
                         const float* grad_out, double* grad_sites, double* abs_sites) {
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            int p = y * w + x;
            float ux = (float)x, uy = (float)y;
            uint32_t ids[K];
            load_cands(cand0, cand1, cand_index_for_pixel(x, y, w, h, cw, ch), ids);
            float wts[K], pred[3];
            if (!weights_raw(ids, sites, n, ux, uy, inv_s2, wts, pred)) continue;
            float dLdp[3] = {grad_out[3 * p], grad_out[3 * p + 1], grad_out[3 * p + 2]};
            for (int i = 0; i < K; i++) {
                uint32_t id = ids[i];
                if (id >= n || sites[id].px < 0.0f) continue;
                float g[10];
                site_param_grads(&sites[id], ux, uy, inv_s2, wts[i], dLdp, pred, 0, g);
                for (int c = 0; c < 10; c++) {
                    grad_sites[(size_t)id * 10 + c] += g[c];
                    if (abs_sites) abs_sites[(size_t)id * 10 + c] += fabs((double)g[c]);
                }
            }
        }
    }
}

/* FP64 version of the adjoint (candidate field at full resolution). */
void orc_render_backward_d(const uint32_t* cand0, const uint32_t* cand1, const orc_site_d* sites,
                           uint32_t n, int w, int h, double inv_s2, const double* grad_out,
                           double* grad_sites) {
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            int p = y * w + x;
            double ux = x, uy = y;
            uint32_t ids[K];
            load_cands(cand0, cand1, p, ids);
            double logits[K], mx = -INFINITY;
            int any = 0;
            for (int i = 0; i < K; i++) {
                uint32_t id = ids[i];
                if (id >= n || sites[id].px < 0.0) { logits[i] = -INFINITY; continue; }
                logits[i] = -exp(sites[id].log_tau) * orc_dmix2_d(&sites[id], ux, uy, inv_s2);
                mx = fmax(mx, logits[i]);
                any = 1;
            }
            if (!any || isinf(mx)) continue;
            double wts[K], sum = 0.0, pred[3] = {0, 0, 0};
            for (int i = 0; i < K; i++) { wts[i] = exp(logits[i] - mx); sum += wts[i]; }
            double inv = 1.0 / fmax(sum, 1e-8);
            for (int i = 0; i < K; i++) {
                wts[i] *= inv;
                uint32_t id = ids[i];
                if (id < n && sites[id].px >= 0.0) { pred[0] += wts[i] * sites[id].r; pred[1] += wts[i] * sites[id].g; pred[2] += wts[i] * sites[id].b; }
            }
            double d[3] = {grad_out[3 * p], grad_out[3 * p + 1], grad_out[3 * p + 2]};
            for (int i = 0; i < K; i++) {
                uint32_t id = ids[i];
                if (id >= n || sites[id].px < 0.0) continue;
                const orc_site_d* s = &sites[id];
                double wv = wts[i];
                double dlogit = d[0] * wv * (s->r - pred[0]) + d[1] * wv * (s->g - pred[1]) + d[2] * wv * (s->b - pred[2]);
                double tau = exp(s->log_tau);
                double dx = ux - s->px, dy = uy - s->py;
                double diff2 = dx * dx + dy * dy, proj = s->dx * dx + s->dy * dy;
                double proj2 = proj * proj, perp2 = fmax(diff2 - proj2, 0.0);
                double l1 = exp(s->log_aniso), l2 = 1.0 / l1;
                double d2s = fmax((l1 * proj2 + l2 * perp2) * inv_s2, 1e-8);
                double isq = 1.0 / sqrt(d2s), isc = sqrt(inv_s2);
                double dmix2 = sqrt(d2s) - s->radius * isc;
                double* g = grad_sites + (size_t)id * 10;
                g[0] += dlogit * tau * inv_s2 * isq * (l2 * dx + (l1 - l2) * s->dx * proj);
                g[1] += dlogit * tau * inv_s2 * isq * (l2 * dy + (l1 - l2) * s->dy * proj);
                g[2] += dlogit * (-dmix2) * tau;
                g[3] += dlogit * tau * isc;
                g[4] += wv * d[0]; g[5] += wv * d[1]; g[6] += wv * d[2];
                double kang = dlogit * (-tau) * 0.5 * isq;
                g[7] += kang * 2.0 * (l1 - l2) * proj * inv_s2 * dx;
                g[8] += kang * 2.0 * (l1 - l2) * proj * inv_s2 * dy;
                g[9] += kang * (l1 * proj2 - l2 * perp2) * inv_s2;
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* candidate construction                                                    */
/* ------------------------------------------------------------------------ */

/* backends/cuda/src/render.cu:95-136.  site_count == 0 in random mode is a
 * division by zero in the reference; here every slot is left empty. */
void orc_init_candidates(uint32_t* cand0, uint32_t* cand1, uint32_t n, uint32_t seed,
                         int per_pixel, int w, int h) {
    static const int nb[7][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}, {-1, -1}, {1, -1}, {-1, 1}};
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            int p = y * w + x;
            uint32_t idx[K];
            if (per_pixel && n == (uint32_t)(w * h)) {
                idx[0] = (uint32_t)p;
                for (int i = 0; i < 7; i++) {
                    int nx = clampi(x + nb[i][0], 0, w - 1), ny = clampi(y + nb[i][1], 0, h - 1);
                    idx[i + 1] = (uint32_t)(ny * w + nx);
                }
            } else if (n == 0) {
                for (int i = 0; i < K; i++) idx[i] = EMPTY;
            } else {
                uint32_t st = seed ^ ((uint32_t)x * 1973u) ^ ((uint32_t)y * 9277u);
                for (int i = 0; i < K; i++) { st = orc_xorshift32(st + (uint32_t)i); idx[i] = st % n; }
            }
            for (int i = 0; i < 4; i++) { cand0[p * 4 + i] = idx[i]; cand1[p * 4 + i] = idx[4 + i]; }
        }
    }
}

/* backends/cuda/src/render.cu:139-154 */
void orc_clear_candidates(uint32_t* cand0, uint32_t* cand1, int w, int h) {
    for (size_t i = 0; i < (size_t)w * h * 4; i++) { cand0[i] = EMPTY; cand1[i] = EMPTY; }
}

/* backends/cuda/src/candidate_pack.cu:3-28 */
void orc_pack_candidate_sites(const orc_site* sites, uint16_t* packed, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        const orc_site* s = &sites[i];
        uint16_t* o = packed + (size_t)i * 8;
        if (s->px < 0.0f) {
            uint16_t neg = orc_f32_to_f16(-1.0f), z = orc_f32_to_f16(0.0f);
            o[0] = neg; o[1] = neg;
            for (int k = 2; k < 8; k++) o[k] = z;
        } else {
            o[0] = orc_f32_to_f16(s->px); o[1] = orc_f32_to_f16(s->py);
            o[2] = orc_f32_to_f16(s->log_tau); o[3] = orc_f32_to_f16(s->radius);
            o[4] = orc_f32_to_f16(s->dx); o[5] = orc_f32_to_f16(s->dy);
            o[6] = orc_f32_to_f16(s->log_aniso); o[7] = orc_f32_to_f16(0.0f);
        }
    }
}

/* backends/cuda/src/jfa.cu:66-92.  The reference's seed is a racy
 * last-writer-wins store when several sites fall on one pixel; the oracle (and
 * the CUDA path) resolve the collision deterministically: the lowest site id. */
void orc_jfa_seed(uint32_t* cand0, const orc_site* sites, uint32_t n, int w, int h, int ds) {
    float inv = 1.0f / fmaxf((float)ds, 1.0f);
    for (uint32_t i = n; i-- > 0;) {
        const orc_site* s = &sites[i];
        if (s->px < 0.0f) continue;
        int x = clampi((int)(s->px * inv), 0, w - 1);
        int y = clampi((int)(s->py * inv), 0, h - 1);
        cand0[(y * w + x) * 4] = i;
    }
}

/* Insert (d, id) into an ascending list of `len`: the first slot j with d < best[j]
 * takes it and the tail shifts down (jfa.cu:14-63 for len 4, jfa.cu:176-248 for 8). */
static inline void sorted_insert(uint32_t* bi, float* bd, int len, uint32_t id, float d) {
    int j = 0;
    while (j < len && !(d < bd[j])) j++;
    if (j == len) return;
    for (int k = len - 1; k > j; k--) { bd[k] = bd[k - 1]; bi[k] = bi[k - 1]; }
    bd[j] = d; bi[j] = id;
}

/* backends/cuda/src/jfa.cu:14-63 (insertClosest4) */
static void insert4(uint32_t bi[4], float bd[4], uint32_t id, float ux, float uy,
                    const orc_site* sites, uint32_t n, float inv_s2) {
    if (id >= n) return;
    for (int i = 0; i < 4; i++) if (bi[i] == id) return;
    if (sites[id].px < 0.0f) return;
    float dm = orc_dmix2(&sites[id], ux, uy, inv_s2);
    float tau = fmaxf(expf(sites[id].log_tau), 1e-4f);
    sorted_insert(bi, bd, 4, id, tau * dm);
}

/* backends/cuda/src/jfa.cu:95-144 (jfaFloodKernel) */
void orc_jfa_flood(const uint32_t* in0, uint32_t* out0, const orc_site* sites, uint32_t n,
                   uint32_t step, float inv_s2, int w, int h, int ds, int tw, int th) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            float ux = fminf((float)x * (float)ds, (float)(tw - 1));
            float uy = fminf((float)y * (float)ds, (float)(th - 1));
            uint32_t bi[4] = {EMPTY, EMPTY, EMPTY, EMPTY};
            float bd[4] = {INFINITY, INFINITY, INFINITY, INFINITY};
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    int sx = clampi(x + dx * (int)step, 0, w - 1), sy = clampi(y + dy * (int)step, 0, h - 1);
                    const uint32_t* c = in0 + (size_t)(sy * w + sx) * 4;
                    for (int k = 0; k < 4; k++) insert4(bi, bd, c[k], ux, uy, sites, n, inv_s2);
                }
            for (int k = 0; k < 4; k++) out0[(size_t)(y * w + x) * 4 + k] = bi[k];
        }
    }
}

/* backends/cuda/src/jfa.cu:150-174 (candidatePackedDistance) */
float orc_packed_distance(const uint16_t* ps, float ux, float uy, float inv_s2) {
    orc_site s;
    s.px = orc_f16_to_f32(ps[0]);
    s.py = orc_f16_to_f32(ps[1]);
    if (s.px < 0.0f) return INFINITY;
    s.log_tau = orc_f16_to_f32(ps[2]);
    s.radius = orc_f16_to_f32(ps[3]);
    s.dx = orc_f16_to_f32(ps[4]);
    s.dy = orc_f16_to_f32(ps[5]);
    s.log_aniso = orc_f16_to_f32(ps[6]);
    s.r = s.g = s.b = 0.0f;
    float dm = orc_dmix2(&s, ux, uy, inv_s2);
    float tau = fmaxf(expf(s.log_tau), 1e-4f);
    return tau * dm;
}

/* backends/cuda/src/jfa.cu:176-248 (insertClosest8Packed) */
static void insert8(uint32_t bi[8], float bd[8], uint32_t id, float ux, float uy,
                    const uint16_t* packed, uint32_t n, float inv_s2) {
    if (id >= n) return;
    for (int i = 0; i < 8; i++) if (bi[i] == id) return;
    float d = orc_packed_distance(packed + (size_t)id * 8, ux, uy, inv_s2);
    sorted_insert(bi, bd, 8, id, d);
}

/* backends/cuda/src/jfa.cu:271-386 (updateCandidatesKernel) */
void orc_vpt_pass(const uint32_t* in0, const uint32_t* in1, uint32_t* out0, uint32_t* out1,
                  const uint16_t* packed, uint32_t n, uint32_t step, float inv_s2,
                  uint32_t step_high, float radius_scale, uint32_t radius_probes, uint32_t inject,
                  const uint32_t* horder, const uint32_t* hpos, uint32_t hprobes, uint32_t hwin,
                  int ds, int tw, int th, int w, int h) {
    uint32_t step_index = step & 0xffffu;
    uint32_t jump = step >> 16;
    if (jump == 0u) jump = 1u;
    uint32_t full_step = (step_high << 16) | step_index;
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            int p = y * w + x;
            float ux = fminf((float)x * (float)ds, (float)(tw - 1));
            float uy = fminf((float)y * (float)ds, (float)(th - 1));
            uint32_t bi[8];
            float bd[8];
            for (int i = 0; i < 8; i++) { bi[i] = EMPTY; bd[i] = INFINITY; }
            for (int k = 0; k < 4; k++) insert8(bi, bd, in0[(size_t)p * 4 + k], ux, uy, packed, n, inv_s2);
            for (int k = 0; k < 4; k++) insert8(bi, bd, in1[(size_t)p * 4 + k], ux, uy, packed, n, inv_s2);
            static const int off[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};
            for (int i = 0; i < 4; i++) {
                int nx = clampi(x + off[i][0] * (int)jump, 0, w - 1);
                int ny = clampi(y + off[i][1] * (int)jump, 0, h - 1);
                size_t q = (size_t)(ny * w + nx) * 4;
                for (int k = 0; k < 4; k++) insert8(bi, bd, in0[q + k], ux, uy, packed, n, inv_s2);
                for (int k = 0; k < 4; k++) insert8(bi, bd, in1[q + k], ux, uy, packed, n, inv_s2);
            }
            float rad = radius_scale * ((float)w / 1024.0f);
            uint32_t st = ((uint32_t)x * 73856093u) ^ ((uint32_t)y * 19349663u) ^ ((step_index + jump) * 83492791u);
            for (uint32_t r = 0; r < radius_probes; r++) {
                float a = orc_rand01(&st) * 6.2831853f;
                int ddx = (int)(cosf(a) * rad), ddy = (int)(sinf(a) * rad);
                int px = clampi(x + ddx, 0, w - 1), py = clampi(y + ddy, 0, h - 1);
                if (px == x && py == y) continue;
                size_t q = (size_t)(py * w + px) * 4;
                for (int k = 0; k < 4; k++) insert8(bi, bd, in0[q + k], ux, uy, packed, n, inv_s2);
                for (int k = 0; k < 4; k++) insert8(bi, bd, in1[q + k], ux, uy, packed, n, inv_s2);
            }
            if (hprobes > 0 && hwin > 0) {
                uint32_t best = bi[0];
                if (best < n) {
                    uint32_t pos = hpos[best];
                    uint32_t span = hwin * 2u + 1u;
                    uint32_t hs = ((uint32_t)x * 2654435761u) ^ ((uint32_t)y * 1597334677u) ^ (full_step * 374761393u);
                    for (uint32_t i = 0; i < hprobes; i++) {
                        hs = orc_xorshift32(hs + i);
                        int o = (int)(hs % span) - (int)hwin;
                        int idx = clampi((int)pos + o, 0, (int)(n - 1));
                        insert8(bi, bd, horder[idx], ux, uy, packed, n, inv_s2);
                    }
                }
            }
            uint32_t is = ((uint32_t)x * 1664525u) ^ ((uint32_t)y * 1013904223u) ^ (full_step * 374761393u);
            for (uint32_t i = 0; i < inject; i++) {
                is = orc_xorshift32(is + i);
                insert8(bi, bd, is % n, ux, uy, packed, n, inv_s2);
            }
            for (int k = 0; k < 4; k++) { out0[(size_t)p * 4 + k] = bi[k]; out1[(size_t)p * 4 + k] = bi[4 + k]; }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* fused training gradient (backends/cuda/src/gradients.cu:103-486)          */
/* ------------------------------------------------------------------------ */

/* backends/cuda/src/gradients.cu:4-42 (ssim_window_stats with clamped taps) */
static void ssim_stats(const float* ren, const float* tgt, int x, int y, int w, int h, float st[5]) {
    float mx = 0, my = 0, ex2 = 0, ey2 = 0, exy = 0;
    for (int dy = -1; dy <= 1; dy++) {
        int yy = clampi(y + dy, 0, h - 1);
        for (int dx = -1; dx <= 1; dx++) {
            int xx = clampi(x + dx, 0, w - 1);
            int i = yy * w + xx;
            float xv = ren[3 * i] * 0.299f + ren[3 * i + 1] * 0.587f + ren[3 * i + 2] * 0.114f;
            float yv = tgt[3 * i] * 0.299f + tgt[3 * i + 1] * 0.587f + tgt[3 * i + 2] * 0.114f;
            mx += xv; my += yv; ex2 += xv * xv; ey2 += yv * yv; exy += xv * yv;
        }
    }
    const float invn = 0.111111111f;
    st[0] = mx * invn; st[1] = my * invn; st[2] = ex2 * invn; st[3] = ey2 * invn; st[4] = exy * invn;
}

/* Per-pixel contributions of the fused kernel.  Returns the number of
 * candidate entries written to ids/g (one per valid slot, duplicates kept) and
 * the unique-site removal deltas in rid/rdelta (count in *nrem). */
static int pixel_grad_terms(const uint32_t* cand0, const uint32_t* cand1, const float* target,
                            const float* rendered, const orc_site* sites, uint32_t n, int x, int y,
                            int w, int h, int cw, int ch, float inv_s2, float ssim_w, int want_removal,
                            uint32_t ids_out[K], float g_out[K][10], uint32_t rid[K], float rdelta[K],
                            int* nrem) {
    int p = y * w + x;
    float ux = (float)x, uy = (float)y;
    uint32_t ids[K];
    load_cands(cand0, cand1, cand_index_for_pixel(x, y, w, h, cw, ch), ids);
    float logits[K], mx = -INFINITY;
    *nrem = 0;
    for (int i = 0; i < K; i++) {
        uint32_t id = ids[i];
        if (id >= n || sites[id].px < 0.0f) { logits[i] = -INFINITY; continue; }
        float tau = expf(sites[id].log_tau);
        logits[i] = -tau * orc_dmix2(&sites[id], ux, uy, inv_s2);
        mx = fmaxf(mx, logits[i]);
    }
    if (!(!isinf(mx) || mx > 0.0f)) return 0;
    float wts[K], sum = 0.0f;
    for (int i = 0; i < K; i++) { wts[i] = expf(logits[i] - mx); sum += wts[i]; }
    float inv = 1.0f / fmaxf(sum, 1e-8f);
    float pred[3] = {0, 0, 0};
    for (int i = 0; i < K; i++) {
        wts[i] *= inv;
        uint32_t id = ids[i];
        if (id < n && sites[id].px >= 0.0f) { pred[0] += wts[i] * sites[id].r; pred[1] += wts[i] * sites[id].g; pred[2] += wts[i] * sites[id].b; }
    }
    const float* t = target + 3 * p;
    float dLdp[3] = {2.0f * (pred[0] - t[0]), 2.0f * (pred[1] - t[1]), 2.0f * (pred[2] - t[2])};
    if (ssim_w > 0.0f) {
        float st[5];
        ssim_stats(rendered, target, x, y, w, h, st);
        float mux = st[0], muy = st[1];
        float sx2 = fmaxf(st[2] - mux * mux, 0.0f), sy2 = fmaxf(st[3] - muy * muy, 0.0f);
        float sxy = st[4] - mux * muy;
        float A = 2.0f * mux * muy + 0.0001f, B = 2.0f * sxy + 0.0009f;
        float C = mux * mux + muy * muy + 0.0001f, D = sx2 + sy2 + 0.0009f;
        float den = fmaxf(C * D, 1e-8f), num = A * B;
        const float* r = rendered + 3 * p;
        float xk = r[0] * 0.299f + r[1] * 0.587f + r[2] * 0.114f;
        float yk = t[0] * 0.299f + t[1] * 0.587f + t[2] * 0.114f;
        const float invn = 0.111111111f;
        float dA = 2.0f * muy * invn, dB = 2.0f * (invn * (yk - muy));
        float dC = 2.0f * mux * invn, dD = (2.0f * invn) * (xk - mux);
        float dS = (dA * B + A * dB) / den - num * (dC * D + C * dD) / (den * den);
        dLdp[0] += (-ssim_w * dS) * 0.299f;
        dLdp[1] += (-ssim_w * dS) * 0.587f;
        dLdp[2] += (-ssim_w * dS) * 0.114f;
    }
    if (want_removal) {
        uint32_t us[K];
        float uw[K];
        int nu = 0;
        for (int i = 0; i < K; i++) {
            uint32_t id = ids[i];
            if (id >= n || sites[id].px < 0.0f) continue;
            int found = 0;
            for (int j = 0; j < nu; j++) if (us[j] == id) { uw[j] += wts[i]; found = 1; break; }
            if (!found) { us[nu] = id; uw[nu] = wts[i]; nu++; }
        }
        for (int i = 0; i < nu; i++) {
            float wt = uw[i];
            if (!(wt > 0.0f)) continue;
            const orc_site* s = &sites[us[i]];
            float keep = 1.0f - wt, delta;
            if (keep < 1e-4f) {
                delta = 1.0e6f;
            } else {
                float pk0 = (pred[0] - wt * s->r) / keep, pk1 = (pred[1] - wt * s->g) / keep, pk2 = (pred[2] - wt * s->b) / keep;
                float d0 = pred[0] - t[0], d1 = pred[1] - t[1], d2 = pred[2] - t[2];
                float k0 = pk0 - t[0], k1 = pk1 - t[1], k2 = pk2 - t[2];
                delta = (k0 * k0 + k1 * k1 + k2 * k2) - (d0 * d0 + d1 * d1 + d2 * d2);
            }
            rid[*nrem] = us[i];
            rdelta[*nrem] = delta;
            (*nrem)++;
        }
    }
    int cnt = 0;
    for (int i = 0; i < K; i++) {
        uint32_t id = ids[i];
        if (id >= n || sites[id].px < 0.0f) continue;
        site_param_grads(&sites[id], ux, uy, inv_s2, wts[i], dLdp, pred, 1, g_out[cnt]);
        ids_out[cnt++] = id;
    }
    return cnt;
}

int orc_pixel_terms(const uint32_t* cand0, const uint32_t* cand1, const float* target,
                    const orc_site* sites, uint32_t n, int x, int y, int w, int h, float inv_s2,
                    int want_removal, uint32_t* ids, float (*g)[10], uint32_t* rid, float* rdelta,
                    int* nrem) {
    return pixel_grad_terms(cand0, cand1, target, NULL, sites, n, x, y, w, h, w, h, inv_s2, 0.0f,
                            want_removal, ids, g, rid, rdelta, nrem);
}

void orc_compute_gradients(const uint32_t* cand0, const uint32_t* cand1, const float* target,
                           const float* rendered, const float* mask, const orc_site* sites,
                           uint32_t n, int w, int h, int cw, int ch, float inv_s2, float ssim_w,
                           double* grads, double* abs_grads, double* removal) {
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            if (mask && !(mask[y * w + x] > 0.0f)) continue;
            uint32_t ids[K], rid[K];
            float g[K][10], rd[K];
            int nrem;
            int cnt = pixel_grad_terms(cand0, cand1, target, rendered, sites, n, x, y, w, h, cw, ch,
                                       inv_s2, ssim_w, removal != NULL, ids, g, rid, rd, &nrem);
            for (int i = 0; i < cnt; i++)
                for (int c = 0; c < 10; c++) {
                    grads[(size_t)c * n + ids[i]] += g[i][c];
                    if (abs_grads) abs_grads[(size_t)c * n + ids[i]] += fabs((double)g[i][c]);
                }
            if (removal)
                for (int i = 0; i < nrem; i++) removal[rid[i]] += rd[i];
        }
    }
}

/* backends/cuda/src/tau_diffusion.cu:27-89 */
void orc_tau_diffuse(const uint32_t* cand0, const uint32_t* cand1, const orc_site* sites,
                     const float* raw, const float* gin, float* gout, uint32_t n, float lambda,
                     int w, int h, int ds) {
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)n; ii++) {
        uint32_t i = (uint32_t)ii;
        if (lambda <= 0.0f || sites[i].px < 0.0f) { gout[i] = gin[i]; continue; }
        float inv = 1.0f / fmaxf((float)ds, 1.0f);
        int px = clampi((int)(sites[i].px * inv + 0.5f), 0, w - 1);
        int py = clampi((int)(sites[i].py * inv + 0.5f), 0, h - 1);
        uint32_t ids[K];
        load_cands(cand0, cand1, py * w + px, ids);
        float sum = 0.0f;
        uint32_t cnt = 0;
        for (int k = 0; k < K; k++) {
            uint32_t m = ids[k];
            if (m >= n || m == i) continue;
            int seen = 0;
            for (int j = 0; j < k; j++) if (ids[j] == m) { seen = 1; break; }
            if (seen || sites[m].px < 0.0f) continue;
            sum += gin[m];
            cnt++;
        }
        float diag = 1.0f + lambda * (float)cnt;
        gout[i] = (raw[i] + lambda * sum) / diag;
    }
}

/* backends/cuda/src/adam.cu:5-180 (adamUpdateKernel) over the 20-float state */
void orc_adam_update(orc_site* sites, float* adam, const float* grads, uint32_t n, float lr_pos,
                     float lr_tau, float lr_radius, float lr_color, float lr_dir, float lr_aniso,
                     float b1, float b2, float eps, uint32_t t, int w, int h) {
    float norm = 1.0f / (float)(w * h);
    float tt = (float)t;
    float c1 = 1.0f / (1.0f - powf(b1, tt));
    float c2 = 1.0f / (1.0f - powf(b2, tt));
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)n; ii++) {
        uint32_t i = (uint32_t)ii;
        orc_site* s = &sites[i];
        float* a = adam + (size_t)i * 20;
        float g[10];
        for (int c = 0; c < 10; c++) g[c] = grads[(size_t)c * n + i] * norm;
        if (s->px < 0.0f) continue;
        /* position: isotropic Adam */
        a[0] = b1 * a[0] + (1.0f - b1) * g[0];
        a[1] = b1 * a[1] + (1.0f - b1) * g[1];
        a[2] = b2 * a[2] + (1.0f - b2) * (g[0] * g[0] + g[1] * g[1]);
        {
            float mh0 = a[0] * c1, mh1 = a[1] * c1, vh = a[2] * c2;
            float idn = 1.0f / (sqrtf(vh) + eps);
            s->px -= lr_pos * mh0 * idn;
            s->py -= lr_pos * mh1 * idn;
            s->px = clampf(s->px, 0.0f, (float)(w - 1));
            s->py = clampf(s->py, 0.0f, (float)(h - 1));
        }
        /* log_tau */
        a[3] = b1 * a[3] + (1.0f - b1) * g[2];
        a[4] = b2 * a[4] + (1.0f - b2) * (g[2] * g[2]);
        s->log_tau -= lr_tau * (a[3] * c1) / (sqrtf(a[4] * c2) + eps);
        /* radius */
        a[5] = b1 * a[5] + (1.0f - b1) * g[3];
        a[6] = b2 * a[6] + (1.0f - b2) * (g[3] * g[3]);
        s->radius -= lr_radius * (a[5] * c1) / (sqrtf(a[6] * c2) + eps);
        s->radius = clampf(s->radius, 1.0f, 512.0f);
        /* colour, per channel */
        {
            float* col[3] = {&s->r, &s->g, &s->b};
            for (int c = 0; c < 3; c++) {
                a[7 + c] = b1 * a[7 + c] + (1.0f - b1) * g[4 + c];
                a[10 + c] = b2 * a[10 + c] + (1.0f - b2) * (g[4 + c] * g[4 + c]);
            }
            for (int c = 0; c < 3; c++) {
                float step = lr_color * (a[7 + c] * c1) / (sqrtf(a[10 + c] * c2) + eps);
                *col[c] = clampf(*col[c] - step, 0.0f, 1.0f);
            }
        }
        /* direction: tangent-space isotropic Adam, renormalised */
        {
            float dx = s->dx, dy = s->dy;
            float gd = g[7] * dx + g[8] * dy;
            float gtx = g[7] - dx * gd, gty = g[8] - dy * gd;
            a[13] = b1 * a[13] + (1.0f - b1) * gtx;
            a[14] = b1 * a[14] + (1.0f - b1) * gty;
            a[15] = b2 * a[15] + (1.0f - b2) * (gtx * gtx + gty * gty);
            float idn = 1.0f / (sqrtf(a[15] * c2) + eps);
            float nx = dx - lr_dir * (a[13] * c1) * idn, ny = dy - lr_dir * (a[14] * c1) * idn;
            float l2 = nx * nx + ny * ny;
            if (l2 < 1e-12f) { nx = 1.0f; ny = 0.0f; }
            else { float il = 1.0f / sqrtf(l2); nx *= il; ny *= il; }
            s->dx = nx; s->dy = ny;
        }
        /* log_aniso */
        a[16] = b1 * a[16] + (1.0f - b1) * g[9];
        a[17] = b2 * a[17] + (1.0f - b2) * (g[9] * g[9]);
        s->log_aniso -= lr_aniso * (a[16] * c1) / (sqrtf(a[17] * c2) + eps);
        s->log_aniso = clampf(s->log_aniso, -4.0f, 4.0f);
    }
}

/* ------------------------------------------------------------------------ */
/* densify / prune / sort                                                    */
/* ------------------------------------------------------------------------ */

/* backends/cuda/src/densify_prune.cu:223-254 */
void orc_densify_score_pairs(const orc_site* sites, const float* mass, const float* energy,
                             uint32_t* pairs, uint32_t n, float min_mass, float alpha, uint32_t pc) {
    for (uint32_t i = 0; i < pc; i++) {
        uint32_t k = EMPTY, v = EMPTY;
        if (i < n) {
            float m = mass[i], e = energy[i];
            if (sites[i].px >= 0.0f && m > min_mass && isfinite(e)) {
                float den = powf(fmaxf(m, 1e-8f), alpha);
                float score = fmaxf(e, 0.0f) / den;
                k = 0xffffffffu - f2u(score);
                v = i;
            }
        }
        pairs[2 * i] = k; pairs[2 * i + 1] = v;
    }
}

/* backends/cuda/src/densify_prune.cu:257-281 */
void orc_prune_score_pairs(const orc_site* sites, const float* removal, uint32_t* pairs,
                           uint32_t n, float delta_norm, uint32_t pc) {
    for (uint32_t i = 0; i < pc; i++) {
        uint32_t k = EMPTY, v = EMPTY;
        if (i < n) {
            float d = removal[i] * delta_norm;
            if (sites[i].px >= 0.0f && isfinite(d)) { k = f2u(fmaxf(d, 0.0f)); v = i; }
        }
        pairs[2 * i] = k; pairs[2 * i + 1] = v;
    }
}

/* backends/cuda/src/radix_sort.cu:279-336: LSD, 8-bit digits, 2 passes when
 * max_key_exclusive <= 65536 else 4; each pass a stable counting sort. */
void orc_radix_sort_pairs(uint32_t* pairs, uint32_t count, uint32_t max_key_exclusive) {
    int passes = max_key_exclusive <= 65536u ? 2 : 4;
    uint32_t* tmp = (uint32_t*)malloc((size_t)count * 8 + 8);
    uint32_t* src = pairs;
    uint32_t* dst = tmp;
    for (int pass = 0; pass < passes; pass++) {
        uint32_t shift = (uint32_t)pass * 8u;
        size_t cnt[257];
        memset(cnt, 0, sizeof(cnt));
        for (uint32_t i = 0; i < count; i++) cnt[((src[2 * i] >> shift) & 0xffu) + 1]++;
        for (int b = 0; b < 256; b++) cnt[b + 1] += cnt[b];
        for (uint32_t i = 0; i < count; i++) {
            size_t d = cnt[(src[2 * i] >> shift) & 0xffu]++;
            dst[2 * d] = src[2 * i]; dst[2 * d + 1] = src[2 * i + 1];
        }
        uint32_t* t = src; src = dst; dst = t;
    }
    if (src != pairs) memcpy(pairs, src, (size_t)count * 8);
    free(tmp);
}

/* backends/cuda/src/densify_prune.cu:284-292 */
void orc_write_split_indices(const uint32_t* pairs, uint32_t* indices, uint32_t k) {
    for (uint32_t i = 0; i < k; i++) indices[i] = pairs[2 * i + 1];
}

/* backends/cuda/src/densify_prune.cu:295-307 */
void orc_prune_sites(orc_site* sites, const uint32_t* indices, uint32_t count) {
    for (uint32_t i = 0; i < count; i++) {
        uint32_t id = indices[i];
        if (id == EMPTY) continue;
        sites[id].px = -1.0f; sites[id].py = -1.0f;
    }
}

static float lum_at(const float* t, int w, int h, int x, int y) {
    x = clampi(x, 0, w - 1); y = clampi(y, 0, h - 1);
    const float* p = t + 3 * (y * w + x);
    return 0.299f * p[0] + 0.587f * p[1] + 0.114f * p[2];
}

/* backends/cuda/src/densify_prune.cu:86-220 (splitSitesKernel) */
void orc_split_sites(orc_site* sites, float* adam, const uint32_t* split_idx, uint32_t num,
                     const float* mass, const float* ew_, const float* ewx, const float* ewy,
                     const float* ewxx, const float* ewxy, const float* ewyy, uint32_t cur,
                     const float* target, int w, int h) {
    for (uint32_t gid = 0; gid < num; gid++) {
        uint32_t pi = split_idx[gid];
        orc_site par = sites[pi];
        if (par.px < 0.0f) continue;
        float ew = ew_[pi];
        float ax = par.dx, ay = par.dy, cx = par.px, cy = par.py;
        float la = par.log_aniso * 0.8f;
        if (ew > 1e-3f) {
            float mx = ewx[pi] / ew, my = ewy[pi] / ew;
            cx = 0.4f * par.px + 0.6f * mx;
            cy = 0.4f * par.py + 0.6f * my;
            float exx = ewxx[pi] / ew - mx * mx, exy = ewxy[pi] / ew - mx * my, eyy = ewyy[pi] / ew - my * my;
            exx = fmaxf(exx, 1e-4f); eyy = fmaxf(eyy, 1e-4f);
            float th = 0.5f * atan2f(2.0f * exy, exx - eyy);
            ax = cosf(th); ay = sinf(th);
            float tr = exx + eyy;
            float disc = sqrtf(fmaxf(0.0f, 0.25f * (exx - eyy) * (exx - eyy) + exy * exy));
            float lam1 = fmaxf(1e-4f, 0.5f * tr + disc), lam2 = fmaxf(1e-4f, 0.5f * tr - disc);
            la = clampf(-0.5f * logf(lam1 / lam2), -2.0f, 2.0f);
        } else {
            int ix = clampi((int)par.px, 0, w - 1), iy = clampi((int)par.py, 0, h - 1);
            float TL = lum_at(target, w, h, ix - 1, iy - 1), T = lum_at(target, w, h, ix, iy - 1), TR = lum_at(target, w, h, ix + 1, iy - 1);
            float L = lum_at(target, w, h, ix - 1, iy), R = lum_at(target, w, h, ix + 1, iy);
            float BL = lum_at(target, w, h, ix - 1, iy + 1), B = lum_at(target, w, h, ix, iy + 1), BR = lum_at(target, w, h, ix + 1, iy + 1);
            float gx = (-TL + TR - 2.0f * L + 2.0f * R - BL + BR) / 4.0f;
            float gy = (-TL - 2.0f * T - TR + BL + 2.0f * B + BR) / 4.0f;
            if (gx * gx + gy * gy > 1e-8f) {
                float len = sqrtf(gx * gx + gy * gy);
                if (len > 1e-8f) { ax = gx / len; ay = gy / len; } else { ax = 1.0f; ay = 0.0f; }
            }
        }
        float m = fmaxf(mass[pi], 1.0f);
        float od = clampf(sqrtf(m) * 0.5f, 1.5f, 48.0f);
        float ox = ax * od, oy = ay * od;
        float pax = clampf(cx + ox, 0.0f, (float)(w - 1)), pay = clampf(cy + oy, 0.0f, (float)(h - 1));
        float pbx = clampf(cx - ox, 0.0f, (float)(w - 1)), pby = clampf(cy - oy, 0.0f, (float)(h - 1));
        const float* ca = target + 3 * ((int)pay * w + (int)pax);
        const float* cb = target + 3 * ((int)pby * w + (int)pbx);
        uint32_t ci = cur + gid;
        if (ci == pi) continue;
        orc_site c0 = par, c1 = par;
        c0.px = pax; c0.py = pay; c1.px = pbx; c1.py = pby;
        c0.r = ca[0]; c0.g = ca[1]; c0.b = ca[2];
        c1.r = cb[0]; c1.g = cb[1]; c1.b = cb[2];
        c0.log_tau = par.log_tau - 0.25f; c1.log_tau = par.log_tau - 0.25f;
        c0.radius = par.radius * 0.85f; c1.radius = par.radius * 0.85f;
        c0.dx = ax; c0.dy = ay; c1.dx = ax; c1.dy = ay;
        c0.log_aniso = la; c1.log_aniso = la;
        sites[pi] = c0;
        sites[ci] = c1;
        memset(adam + (size_t)pi * 20, 0, 80);
        memset(adam + (size_t)ci * 20, 0, 80);
    }
}

/* Luminance / Sobel magnitude of the init proposals with explicit fused
 * multiply-adds (the CUDA path evaluates the same sequence of single roundings). */
static float init_lum(const float* t, int w, int h, int x, int y) {
    x = clampi(x, 0, w - 1); y = clampi(y, 0, h - 1);
    const float* p = t + 3 * (y * w + x);
    return fmaf(0.114f, p[2], fmaf(0.299f, p[0], 0.587f * p[1]));
}

/* backends/cuda/src/densify_prune.cu:5-83 with the shared seed counter handed
 * out in site order (the reference's atomicAdd order is unspecified; this is the
 * serialised order, which the CUDA path reproduces exactly). */
void orc_init_gradient_weighted(orc_site* sites, uint32_t n, const float* target, const float* mask,
                                float thr, uint32_t max_attempts, float init_log_tau,
                                float init_radius, int w, int h) {
    const float gr = 1.32471795724474602596f;
    const float a1 = 1.0f / gr;
    const float a2 = 1.0f / (gr * gr);
    uint32_t seed = 0;
    if (max_attempts == 0) max_attempts = 1;
    for (uint32_t gid = 0; gid < n; gid++) {
        float apx = -1.0f, apy = -1.0f, cr = 0.5f, cg = 0.5f, cb = 0.5f, ag = 0.0f;
        for (uint32_t at = 0; at < max_attempts; at++) {
            uint32_t s = seed++;
            float u = fmodf(fmaf((float)s, a1, 0.5f), 1.0f);
            float v = fmodf(fmaf((float)s, a2, 0.5f), 1.0f);
            float px = u * (float)(w - 1), py = v * (float)(h - 1);
            int ix = (int)px, iy = (int)py;
            float mv = mask ? mask[iy * w + ix] : 1.0f;
            if (mv <= 0.0f) continue;
            float TL = init_lum(target, w, h, ix - 1, iy - 1), T = init_lum(target, w, h, ix, iy - 1), TR = init_lum(target, w, h, ix + 1, iy - 1);
            float L = init_lum(target, w, h, ix - 1, iy), R = init_lum(target, w, h, ix + 1, iy);
            float BL = init_lum(target, w, h, ix - 1, iy + 1), B = init_lum(target, w, h, ix, iy + 1), BR = init_lum(target, w, h, ix + 1, iy + 1);
            float gx = (-TL + TR - 2.0f * L + 2.0f * R - BL + BR) * 0.25f;
            float gy = (-TL - 2.0f * T - TR + BL + 2.0f * B + BR) * 0.25f;
            float g = sqrtf(fmaf(gx, gx, gy * gy)) * mv;
            if (g > thr) {
                apx = px; apy = py;
                const float* c = target + 3 * (iy * w + ix);
                cr = c[0]; cg = c[1]; cb = c[2];
                ag = g;
                break;
            }
        }
        orc_site* o = &sites[gid];
        o->px = apx; o->py = apy;
        o->log_tau = fmaf(powf(ag, 0.25f), 2.0f, init_log_tau);
        o->radius = init_radius;
        o->r = cr; o->g = cg; o->b = cb;
        o->dx = 1.0f; o->dy = 0.0f;
        o->log_aniso = 0.0f;
    }
}

/* backends/cuda/src/utils.cu:106-231 (computeSiteStatsSimpleKernel);
 * stats8 = 8 arrays of N: mass, energy, err_w, err_wx, err_wy, err_wxx, err_wxy, err_wyy */
void orc_site_stats(const uint32_t* cand0, const uint32_t* cand1, const float* target,
                    const float* mask, const orc_site* sites, uint32_t n, int w, int h, int cw,
                    int ch, float inv_s2, double* st) {
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            int p = y * w + x;
            if (mask && !(mask[p] > 0.0f)) continue;
            float ux = (float)x, uy = (float)y;
            uint32_t ids[K];
            load_cands(cand0, cand1, cand_index_for_pixel(x, y, w, h, cw, ch), ids);
            float logits[K], mx = -INFINITY;
            for (int i = 0; i < K; i++) {
                uint32_t id = ids[i];
                if (id >= n || sites[id].px < 0.0f) { logits[i] = -INFINITY; continue; }
                logits[i] = -expf(sites[id].log_tau) * orc_dmix2(&sites[id], ux, uy, inv_s2);
                mx = fmaxf(mx, logits[i]);
            }
            if (isinf(mx) && mx < 0.0f) continue;
            float wts[K], sum = 0.0f;
            for (int i = 0; i < K; i++) { wts[i] = expf(logits[i] - mx); sum += wts[i]; }
            float inv = 1.0f / fmaxf(sum, 1e-8f);
            float pr[3] = {0, 0, 0};
            for (int i = 0; i < K; i++) {
                wts[i] *= inv;
                uint32_t id = ids[i];
                if (id < n && sites[id].px >= 0.0f) { pr[0] += wts[i] * sites[id].r; pr[1] += wts[i] * sites[id].g; pr[2] += wts[i] * sites[id].b; }
            }
            const float* t = target + 3 * p;
            float d0 = pr[0] - t[0], d1 = pr[1] - t[1], d2 = pr[2] - t[2];
            float err = d0 * d0 + d1 * d1 + d2 * d2;
            int seen[K] = {0};
            for (int i = 0; i < K; i++) {
                uint32_t id = ids[i];
                if (id >= n || sites[id].px < 0.0f || seen[i]) continue;
                int dup = 0;
                for (int j = 0; j < i; j++) if (ids[j] == id) { dup = 1; seen[j] = 1; break; }
                if (dup) continue;
                float wt = 0.0f;
                for (int j = i; j < K; j++) if (ids[j] == id) { wt += wts[j]; seen[j] = 1; }
                if (wt > 0.0f) {
                    float we = wt * fminf(err, 1.0f);
                    st[0 * (size_t)n + id] += wt;
                    st[1 * (size_t)n + id] += wt * err;
                    st[2 * (size_t)n + id] += we;
                    st[3 * (size_t)n + id] += we * ux;
                    st[4 * (size_t)n + id] += we * uy;
                    st[5 * (size_t)n + id] += we * ux * ux;
                    st[6 * (size_t)n + id] += we * ux * uy;
                    st[7 * (size_t)n + id] += we * uy * uy;
                }
            }
        }
    }
}

/* backends/cuda/src/sad_cuda.cu:1547-1570 */
void orc_hilbert_pairs(const orc_site* sites, uint32_t* pairs, uint32_t n, uint32_t padded,
                       int w, int h, int bits) {
    for (uint32_t i = 0; i < padded; i++) {
        if (i < n) {
            int px = (int)sites[i].px, py = (int)sites[i].py;
            px = px < 0 ? 0 : (px >= w ? w - 1 : px);
            py = py < 0 ? 0 : (py >= h ? h - 1 : py);
            pairs[2 * i] = orc_hilbert_index((uint32_t)px, (uint32_t)py, bits);
            pairs[2 * i + 1] = i;
        } else {
            pairs[2 * i] = 0xffffffffu; pairs[2 * i + 1] = 0u;
        }
    }
}

/* backends/cuda/src/sad_cuda.cu:1572-1584 */
void orc_write_hilbert_order(const uint32_t* pairs, uint32_t* order, uint32_t* pos, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) { uint32_t s = pairs[2 * i + 1]; order[i] = s; pos[s] = i; }
}

/* backends/cuda/src/utils.cu:5-26 plus the host formula sad_cuda.cu:2438-2441 */
double orc_psnr(const float* ren, const float* tgt, const float* mask, int w, int h) {
    double s = 0.0, msum = 0.0;
    for (int i = 0; i < w * h; i++) {
        float m = mask ? mask[i] : 1.0f;
        msum += m;
        if (m <= 0.0f) continue;
        float d0 = ren[3 * i] - tgt[3 * i], d1 = ren[3 * i + 1] - tgt[3 * i + 1], d2 = ren[3 * i + 2] - tgt[3 * i + 2];
        s += d0 * d0 + d1 * d1 + d2 * d2;
    }
    double mse = s / (fmax(1.0, msum) * 3.0);
    return mse > 0.0 ? 20.0 * log10(1.0 / sqrt(mse)) : 100.0;
}

/* backends/cuda/src/utils.cu:29-87 (sum over masked pixels) */
double orc_ssim_sum(const float* ren, const float* tgt, const float* mask, int w, int h) {
    double acc = 0.0;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            if (mask && mask[y * w + x] <= 0.0f) continue;
            float st[5];
            ssim_stats(ren, tgt, x, y, w, h, st);
            float mux = st[0], muy = st[1];
            float sx2 = fmaxf(st[2] - mux * mux, 0.0f), sy2 = fmaxf(st[3] - muy * muy, 0.0f);
            float sxy = st[4] - mux * muy;
            float A = 2.0f * mux * muy + 0.0001f, B = 2.0f * sxy + 0.0009f;
            float C = mux * mux + muy * muy + 0.0001f, D = sx2 + sy2 + 0.0009f;
            acc += (A * B) / fmaxf(C * D, 1e-8f);
        }
    return acc;
}

/* backends/cuda/src/utils.cu:90-101 */
uint32_t orc_count_active(const orc_site* sites, uint32_t n) {
    uint32_t c = 0;
    for (uint32_t i = 0; i < n; i++) c += sites[i].px >= 0.0f;
    return c;
}

/* ------------------------------------------------------------------------ */
/* host schedule                                                              */
/* ------------------------------------------------------------------------ */

/* backends/cuda/src/sad_cuda.cu:904-960 */
int orc_simulate_final_sites(int init_sites, int max_sites, int iters, int densify_enabled,
                             int ds, int de, int df, float dp, int pdd, int ps, int pe, int pf,
                             float pp, int max_split) {
    int actual = init_sites, active = init_sites;
    int maxc = max_sites > init_sites ? max_sites : init_sites;
    int eps = ps;
    if (densify_enabled && !pdd && ps < de) eps = de;
    if (iters <= 0) return active;
    for (int it = 0; it < iters; it++) {
        if (densify_enabled && dp > 0.0f && it >= ds && it <= de && it % (df > 1 ? df : 1) == 0 && actual < maxc) {
            int desired = (int)(active * dp);
            int avail = maxc - actual;
            int k = desired < avail ? desired : avail;
            if (max_split < k) k = max_split;
            if (k > 0) { actual += k; active += k; }
        }
        if (pp > 0.0f && it >= eps && it < pe && it % (pf > 1 ? pf : 1) == 0) {
            int desired = (int)(active * pp);
            int k = desired < max_split ? desired : max_split;
            if (k > 0) { active = active - k; if (active < 0) active = 0; }
        }
    }
    return active;
}

/* backends/cuda/src/sad_cuda.cu:962-1066 (solveTargetBpp) */
void orc_solve_target_bpp(float bpp, int w, int h, int init_sites, int max_sites, int iters,
                          int de_, int ds, int de, int df, float bd, int pdd, int ps, int pe, int pf,
                          float bp, int max_split, float* out) {
    const float bits = 16.0f * 8.0f;
    int target = (int)roundf(bpp * (float)(w * h) / bits);
    if (target < 1) target = 1;
    float max_base = bd > bp ? bd : bp;
    if (max_base <= 0.0f) {
        int fs = orc_simulate_final_sites(init_sites, max_sites, iters, de_, ds, de, df, 0.0f, pdd, ps, pe, pf, 0.0f, max_split);
        out[0] = 0.0f; out[1] = 0.0f; out[2] = (float)fs; out[3] = (float)fs * bits / (float)(w * h);
        return;
    }
    const float max_pct = 0.95f;
    float smax = max_pct / max_base;
    if (smax > 50.0f) smax = 50.0f;
#define EVAL(scale, res)                                                                         \
    do {                                                                                         \
        float d_ = de_ ? fminf(max_pct, bd * (scale)) : 0.0f;                                    \
        float p_ = fminf(max_pct, bp * (scale));                                                 \
        res = orc_simulate_final_sites(init_sites, max_sites, iters, de_, ds, de, df, d_, pdd, ps, \
                                       pe, pf, p_, max_split);                                   \
    } while (0)
    float best_scale = 0.0f;
    int best_sites;
    EVAL(0.0f, best_sites);
    int best_err = abs(best_sites - target);
    const int samples = 80;
    for (int i = 0; i <= samples; i++) {
        float s = smax * (float)i / (float)samples;
        int st;
        EVAL(s, st);
        int err = abs(st - target);
        if (err < best_err) { best_err = err; best_scale = s; best_sites = st; }
    }
    float step = smax / (float)samples;
    for (int i = 0; i < 20; i++) {
        int improved = 0;
        float s0 = best_scale - step, s1 = best_scale + step;
        if (s0 >= 0.0f) {
            int st; EVAL(s0, st);
            int err = abs(st - target);
            if (err < best_err) { best_err = err; best_scale = s0; best_sites = st; improved = 1; }
        }
        if (s1 <= smax) {
            int st; EVAL(s1, st);
            int err = abs(st - target);
            if (err < best_err) { best_err = err; best_scale = s1; best_sites = st; improved = 1; }
        }
        if (!improved) step *= 0.5f;
    }
#undef EVAL
    out[0] = de_ ? fminf(max_pct, bd * best_scale) : 0.0f;
    out[1] = fminf(max_pct, bp * best_scale);
    out[2] = (float)best_sites;
    out[3] = (float)best_sites * bits / (float)(w * h);
}

/* ------------------------------------------------------------------------ */
/* 16-byte quantised inference sites                                         */
/* makePackedInferenceSites, backends/metal/sources/utils/packed_inference.swift:20-199;  */
/* decodePackedSite, backends/metal/shaders/sad_common.metal:71-120.                      */
/* Plain float arithmetic, one rounding per operation (built with -ffp-contract=off).     */
/* ------------------------------------------------------------------------ */

static uint32_t pk_unorm(float v, float minv, float scale, float levels) {
    if (scale <= 0.0f) return 0u;
    float n = fminf(fmaxf((v - minv) / scale, 0.0f), 1.0f);
    return (uint32_t)(n * levels + 0.5f);
}

static uint32_t pk_unorm_max(float v, float maxv, float levels) {
    if (maxv <= 0.0f) return 0u;
    float n = fminf(fmaxf(v / maxv, 0.0f), 1.0f);
    return (uint32_t)(n * levels + 0.5f);
}

static uint32_t pk_angle(float dx, float dy) {
    float len2 = dx * dx + dy * dy;
    float ux = 1.0f, uy = 0.0f;
    if (!(len2 < 1.0e-8f)) {
        float inv = 1.0f / sqrtf(len2);
        ux = dx * inv;
        uy = dy * inv;
    }
    const float pi = 3.14159265358979f;
    float angle = atan2f(uy, ux);
    float n = fminf(fmaxf((angle + pi) / (pi * 2.0f), 0.0f), 1.0f);
    return (uint32_t)(n * 65535.0f + 0.5f);
}

void orc_pack_inference_sites(const orc_site* sites, uint32_t n, int width, int height,
                              uint32_t* packed, float* quant) {
    float mn[5], mx[5];
    for (int f = 0; f < 5; f++) { mn[f] = INFINITY; mx[f] = -INFINITY; }
    for (uint32_t i = 0; i < n; i++) {
        const orc_site* s = &sites[i];
        if (!(s->px >= 0.0f && s->py >= 0.0f)) continue;
        float v[5] = {s->log_tau, s->radius, s->r, s->g, s->b};
        for (int f = 0; f < 5; f++) {
            if (!isfinite(v[f])) continue;
            if (v[f] < mn[f]) mn[f] = v[f];
            if (v[f] > mx[f]) mx[f] = v[f];
        }
    }
    for (int f = 0; f < 5; f++) {
        if (!isfinite(mn[f]) || !isfinite(mx[f])) { mn[f] = 0.0f; mx[f] = 0.0f; }
        quant[2 * f] = mn[f];
        quant[2 * f + 1] = fmaxf(mx[f] - mn[f], 1.0e-6f);
    }
    float max_x = (float)(width > 1 ? width - 1 : 0), max_y = (float)(height > 1 ? height - 1 : 0);
    for (uint32_t i = 0; i < n; i++) {
        const orc_site* s = &sites[i];
        int active = s->px >= 0.0f && s->py >= 0.0f;
        float x = fminf(fmaxf(s->px, 0.0f), max_x), y = fminf(fmaxf(s->py, 0.0f), max_y);
        uint32_t w0 = pk_unorm_max(x, max_x, 32767.0f) | (pk_unorm_max(y, max_y, 32767.0f) << 15);
        w0 = (w0 & 0x3fffffffu) | ((active ? 0u : 1u) << 30);
        uint32_t w1 = pk_unorm(s->r, quant[4], quant[5], 2047.0f) | (pk_unorm(s->g, quant[6], quant[7], 2047.0f) << 11) |
                      (pk_unorm(s->b, quant[8], quant[9], 1023.0f) << 22);
        float lt = isfinite(s->log_tau) ? s->log_tau : quant[0];
        float rd = isfinite(s->radius) ? s->radius : quant[2];
        uint32_t w2 = pk_unorm(lt, quant[0], quant[1], 65535.0f) | (pk_unorm(rd, quant[2], quant[3], 65535.0f) << 16);
        float la = isfinite(s->log_aniso) ? s->log_aniso : 0.0f;
        uint32_t w3 = (pk_angle(s->dx, s->dy) & 0xffffu) | ((uint32_t)orc_f32_to_f16(la) << 16);
        packed[4 * i + 0] = w0;
        packed[4 * i + 1] = w1;
        packed[4 * i + 2] = w2;
        packed[4 * i + 3] = w3;
    }
}

static float pk_unpack(uint32_t v, float inv_levels, float minv, float scale) {
    return minv + ((float)v * inv_levels) * fmaxf(scale, 0.0f);
}

void orc_unpack_inference_sites(const uint32_t* packed, const float* quant, uint32_t n, int width, int height,
                                orc_site* sites) {
    const float inv16 = 1.0f / 65535.0f, inv15 = 1.0f / 32767.0f, inv11 = 1.0f / 2047.0f, inv10 = 1.0f / 1023.0f;
    const float pi = 3.14159265f, two_pi = 6.2831853f;
    float dim_x = (float)(width - 1), dim_y = (float)(height - 1);
    for (uint32_t i = 0; i < n; i++) {
        const uint32_t* w = packed + 4 * i;
        orc_site* s = &sites[i];
        s->px = ((float)(w[0] & 0x7fffu) * inv15) * fmaxf(dim_x, 0.0f);
        s->py = ((float)((w[0] >> 15) & 0x7fffu) * inv15) * fmaxf(dim_y, 0.0f);
        s->r = pk_unpack(w[1] & 0x7ffu, inv11, quant[4], quant[5]);
        s->g = pk_unpack((w[1] >> 11) & 0x7ffu, inv11, quant[6], quant[7]);
        s->b = pk_unpack((w[1] >> 22) & 0x3ffu, inv10, quant[8], quant[9]);
        s->log_tau = pk_unpack(w[2] & 0xffffu, inv16, quant[0], quant[1]);
        s->radius = pk_unpack(w[2] >> 16, inv16, quant[2], quant[3]);
        float angle = ((float)(w[3] & 0xffffu) * inv16) * two_pi - pi;
        s->dx = cosf(angle);
        s->dy = sinf(angle);
        s->log_aniso = orc_f16_to_f32((uint16_t)(w[3] >> 16));
        if ((w[0] >> 30) & 1u) s->px = s->py = -1.0f;
    }
}
