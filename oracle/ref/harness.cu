// harness.cu -- runs single kernels of the reference's CUDA backend on raw input files, so
// the reference's own outputs can be recorded as golden fixtures.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/ref/build.sh against the staged reference
// sources (its launch* entry points, declared below as the reference declares them in
// backends/cuda/src/sad_cuda.cu:1185-1437, and its record types from sad_common.cuh).
//
//   ref_harness <command> <dir> [scalars...]
// reads <dir>/<name>.bin (raw little-endian arrays), runs the kernel, writes outputs to
// <dir>/<name>.bin.  The adam state is converted between the 20-float packed layout of the
// fixtures and the reference's 88-byte AdamState struct.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sad_common.cuh"

extern "C" {
void launchRenderVoronoi(const uint32_t*, const uint32_t*, float3*, const Site*, float, uint32_t, int,
                         int, int, int, cudaStream_t);
void launchInitCandidates(uint32_t*, uint32_t*, uint32_t, uint32_t, bool, int, int, cudaStream_t);
void launchPackCandidateSites(const Site*, PackedCandidateSite*, uint32_t, cudaStream_t);
void launchJFASeed(uint32_t*, const Site*, uint32_t, int, int, int, cudaStream_t);
void launchJFAFlood(const uint32_t*, uint32_t*, const Site*, uint32_t, uint32_t, float, int, int, int,
                    int, int, cudaStream_t);
void launchUpdateCandidates(const uint32_t*, const uint32_t*, uint32_t*, uint32_t*,
                            const PackedCandidateSite*, uint32_t, uint32_t, float, uint32_t, float,
                            uint32_t, uint32_t, const uint32_t*, const uint32_t*, uint32_t, uint32_t,
                            int, int, int, int, int, cudaStream_t);
void launchComputeGradientsTiled(const uint32_t*, const uint32_t*, const float3*, const float3*,
                                 const float*, float*, float*, float*, float*, float*, float*, float*,
                                 float*, float*, float*, const Site*, float, uint32_t, float*,
                                 uint32_t, float, int, int, int, int, cudaStream_t);
void launchTauDiffuse(const uint32_t*, const uint32_t*, const Site*, const float*, const float*,
                      float*, uint32_t, float, int, int, int, cudaStream_t);
void launchAdamUpdate(Site*, AdamState*, const float*, const float*, const float*, const float*,
                      const float*, const float*, const float*, const float*, const float*,
                      const float*, float, float, float, float, float, float, float, float, float,
                      uint32_t, uint32_t, int, int, cudaStream_t);
void launchComputeDensifyScorePairs(const Site*, const float*, const float*, uint2*, uint32_t, float,
                                    float, uint32_t, cudaStream_t);
void launchComputePruneScorePairs(const Site*, const float*, uint2*, uint32_t, float, uint32_t,
                                  cudaStream_t);
void launchRadixSortUInt2(uint2*, uint2*, uint32_t*, uint32_t*, uint32_t, uint32_t, cudaStream_t);
void launchPruneSitesByIndex(Site*, const uint32_t*, uint32_t, cudaStream_t);
void launchSplitSites(Site*, AdamState*, const uint32_t*, uint32_t, const float*, const float*,
                      const float*, const float*, const float*, const float*, const float*, uint32_t,
                      const float3*, int, int, cudaStream_t);
void launchComputeSiteStatsSimple(const uint32_t*, const uint32_t*, const float3*, const float*,
                                  const Site*, float, uint32_t, float*, float*, float*, float*,
                                  float*, float*, float*, float*, int, int, int, int, cudaStream_t);
}

#define CK(x)                                                                             \
    do {                                                                                  \
        cudaError_t e_ = (x);                                                             \
        if (e_ != cudaSuccess) {                                                          \
            fprintf(stderr, "%s:%d %s: %s\n", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
            exit(2);                                                                      \
        }                                                                                 \
    } while (0)

static std::string g_dir;

static std::vector<char> read_file(const std::string& name) {
    std::string p = g_dir + "/" + name + ".bin";
    FILE* f = fopen(p.c_str(), "rb");
    if (!f) {
        fprintf(stderr, "missing %s\n", p.c_str());
        exit(3);
    }
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    std::vector<char> b(n);
    if (n && fread(b.data(), 1, n, f) != static_cast<size_t>(n)) exit(3);
    fclose(f);
    return b;
}

static void write_file(const std::string& name, const void* p, size_t n) {
    std::string path = g_dir + "/" + name + ".bin";
    FILE* f = fopen(path.c_str(), "wb");
    fwrite(p, 1, n, f);
    fclose(f);
}

template <class T>
static T* dev_in(const std::string& name, size_t* count = nullptr, size_t min_bytes = 0) {
    std::vector<char> b = read_file(name);
    void* d = nullptr;
    size_t bytes = std::max(b.size(), min_bytes);
    CK(cudaMalloc(&d, bytes ? bytes : 16));
    CK(cudaMemset(d, 0, bytes ? bytes : 16));
    if (!b.empty()) CK(cudaMemcpy(d, b.data(), b.size(), cudaMemcpyHostToDevice));
    if (count) *count = b.size() / sizeof(T);
    return static_cast<T*>(d);
}

template <class T>
static T* dev_zero(size_t count) {
    void* d = nullptr;
    CK(cudaMalloc(&d, count * sizeof(T) + 16));
    CK(cudaMemset(d, 0, count * sizeof(T) + 16));
    return static_cast<T*>(d);
}

template <class T>
static void dev_out(const std::string& name, const T* d, size_t count) {
    std::vector<T> h(count);
    CK(cudaDeviceSynchronize());
    CK(cudaMemcpy(h.data(), d, count * sizeof(T), cudaMemcpyDeviceToHost));
    write_file(name, h.data(), count * sizeof(T));
}

static AdamState* adam_in(const std::string& name, size_t n) {
    std::vector<char> b = read_file(name);
    const float* a = reinterpret_cast<const float*>(b.data());
    std::vector<AdamState> s(n);
    for (size_t i = 0; i < n; ++i) {
        const float* v = a + i * 20;
        AdamState& q = s[i];
        q.m_pos = make_float2(v[0], v[1]);
        q.v_pos = v[2]; q.m_log_tau = v[3]; q.v_log_tau = v[4]; q.m_radius = v[5]; q.v_radius = v[6];
        q.m_color = make_float3(v[7], v[8], v[9]);
        q.v_color = make_float3(v[10], v[11], v[12]);
        q.m_dir = make_float2(v[13], v[14]);
        q.v_dir = v[15]; q.m_log_aniso = v[16]; q.v_log_aniso = v[17];
        q._pad = make_float2(v[18], v[19]);
    }
    AdamState* d = nullptr;
    CK(cudaMalloc(&d, n * sizeof(AdamState) + 16));
    CK(cudaMemcpy(d, s.data(), n * sizeof(AdamState), cudaMemcpyHostToDevice));
    return d;
}

static void adam_out(const std::string& name, const AdamState* d, size_t n) {
    std::vector<AdamState> s(n);
    CK(cudaDeviceSynchronize());
    CK(cudaMemcpy(s.data(), d, n * sizeof(AdamState), cudaMemcpyDeviceToHost));
    std::vector<float> a(n * 20);
    for (size_t i = 0; i < n; ++i) {
        const AdamState& q = s[i];
        float v[20] = {q.m_pos.x, q.m_pos.y, q.v_pos, q.m_log_tau, q.v_log_tau, q.m_radius,
                       q.v_radius, q.m_color.x, q.m_color.y, q.m_color.z, q.v_color.x, q.v_color.y,
                       q.v_color.z, q.m_dir.x, q.m_dir.y, q.v_dir, q.m_log_aniso, q.v_log_aniso,
                       q._pad.x, q._pad.y};
        memcpy(&a[i * 20], v, sizeof(v));
    }
    write_file(name, a.data(), a.size() * 4);
}

int main(int argc, char** argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: ref_harness <command> <dir> [scalars]\n");
        return 1;
    }
    std::string cmd = argv[1];
    g_dir = argv[2];
    auto I = [&](int k) { return static_cast<uint32_t>(strtoul(argv[3 + k], nullptr, 10)); };
    auto N = [&](int k) { return static_cast<int>(strtol(argv[3 + k], nullptr, 10)); };
    auto F = [&](int k) { return strtof(argv[3 + k], nullptr); };
    cudaStream_t st = 0;
    if (cmd == "render") {  // n w h cw ch inv_s2
        uint32_t n = I(0);
        int w = N(1), h = N(2), cw = N(3), ch = N(4);
        auto c0 = dev_in<uint32_t>("cand0"), c1 = dev_in<uint32_t>("cand1");
        auto s = dev_in<Site>("sites");
        auto out = dev_zero<float>(static_cast<size_t>(w) * h * 3);
        launchRenderVoronoi(c0, c1, reinterpret_cast<float3*>(out), s, F(5), n, w, h, cw, ch, st);
        dev_out("out", out, static_cast<size_t>(w) * h * 3);
    } else if (cmd == "init_cand") {  // n seed per_pixel w h
        int w = N(3), h = N(4);
        auto c0 = dev_zero<uint32_t>(static_cast<size_t>(w) * h * 4);
        auto c1 = dev_zero<uint32_t>(static_cast<size_t>(w) * h * 4);
        launchInitCandidates(c0, c1, I(0), I(1), N(2) != 0, w, h, st);
        dev_out("c0", c0, static_cast<size_t>(w) * h * 4);
        dev_out("c1", c1, static_cast<size_t>(w) * h * 4);
    } else if (cmd == "pack") {  // n
        uint32_t n = I(0);
        auto s = dev_in<Site>("sites");
        auto p = dev_zero<PackedCandidateSite>(n);
        launchPackCandidateSites(s, p, n, st);
        dev_out("packed", reinterpret_cast<uint16_t*>(p), static_cast<size_t>(n) * 8);
    } else if (cmd == "jfa_seed") {  // n w h ds
        size_t cnt;
        auto c0 = dev_in<uint32_t>("cand0", &cnt);
        auto s = dev_in<Site>("sites");
        launchJFASeed(c0, s, I(0), N(1), N(2), N(3), st);
        dev_out("out", c0, cnt);
    } else if (cmd == "jfa_flood") {  // n step inv w h ds tw th
        size_t cnt;
        auto in = dev_in<uint32_t>("cand0", &cnt);
        auto s = dev_in<Site>("sites");
        auto out = dev_zero<uint32_t>(cnt);
        launchJFAFlood(in, out, s, I(0), I(1), F(2), N(3), N(4), N(5), N(6), N(7), st);
        dev_out("out", out, cnt);
    } else if (cmd == "vpt") {
        // n step inv step_high radius_scale radius_probes inject hprobes hwin ds tw th w h
        size_t cnt;
        auto c0 = dev_in<uint32_t>("cand0", &cnt);
        auto c1 = dev_in<uint32_t>("cand1");
        auto p = dev_in<PackedCandidateSite>("packed");
        uint32_t hp = I(7), hw = I(8);
        const uint32_t* ho = nullptr;
        const uint32_t* hpos = nullptr;
        if (hp > 0 && hw > 0) {
            ho = dev_in<uint32_t>("horder");
            hpos = dev_in<uint32_t>("hpos");
        }
        auto o0 = dev_zero<uint32_t>(cnt), o1 = dev_zero<uint32_t>(cnt);
        launchUpdateCandidates(c0, c1, o0, o1, p, I(0), I(1), F(2), I(3), F(4), I(5), I(6), ho, hpos,
                               hp, hw, N(9), N(10), N(11), N(12), N(13), st);
        dev_out("out0", o0, cnt);
        dev_out("out1", o1, cnt);
    } else if (cmd == "grads") {  // n inv removal ssim w h cw ch
        uint32_t n = I(0);
        int w = N(4), h = N(5);
        auto c0 = dev_in<uint32_t>("cand0"), c1 = dev_in<uint32_t>("cand1");
        auto tg = dev_in<float3>("target"), rd = dev_in<float3>("rendered");
        auto mk = dev_in<float>("mask");
        auto s = dev_in<Site>("sites");
        float* g[10];
        for (auto& p : g) p = dev_zero<float>(n);
        auto rem = dev_zero<float>(n);
        launchComputeGradientsTiled(c0, c1, tg, rd, mk, g[0], g[1], g[2], g[3], g[4], g[5], g[6], g[7],
                                    g[8], g[9], s, F(1), n, rem, I(2), F(3), w, h, N(6), N(7), st);
        for (int k = 0; k < 10; ++k) dev_out("g" + std::to_string(k), g[k], n);
        dev_out("removal", rem, n);
    } else if (cmd == "tau") {  // n lambda w h ds
        uint32_t n = I(0);
        auto c0 = dev_in<uint32_t>("cand0"), c1 = dev_in<uint32_t>("cand1");
        auto s = dev_in<Site>("sites");
        auto raw = dev_in<float>("raw"), gin = dev_in<float>("gin");
        auto out = dev_zero<float>(n);
        launchTauDiffuse(c0, c1, s, raw, gin, out, n, F(1), N(2), N(3), N(4), st);
        dev_out("out", out, n);
    } else if (cmd == "adam") {  // n lr*6 b1 b2 eps t w h
        uint32_t n = I(0);
        auto s = dev_in<Site>("sites");
        auto a = adam_in("adam", n);
        const float* g[10];
        for (int k = 0; k < 10; ++k) g[k] = dev_in<float>("g" + std::to_string(k));
        launchAdamUpdate(s, a, g[0], g[1], g[2], g[3], g[4], g[5], g[6], g[7], g[8], g[9], F(1), F(2),
                         F(3), F(4), F(5), F(6), F(7), F(8), F(9), I(10), n, N(11), N(12), st);
        dev_out("sites_out", reinterpret_cast<float*>(s), static_cast<size_t>(n) * 10);
        adam_out("adam_out", a, n);
    } else if (cmd == "sort") {  // count maxkey
        uint32_t count = I(0);
        auto d = dev_in<uint2>("pairs");
        auto scratch = dev_zero<uint2>(count);
        uint32_t grid = (count + 1023) / 1024;
        auto hist = dev_zero<uint32_t>(static_cast<size_t>(grid) * 256);
        auto sums = dev_zero<uint32_t>((grid * 256 + 255) / 256);
        launchRadixSortUInt2(d, scratch, hist, sums, count, I(1), st);
        dev_out("out", reinterpret_cast<uint32_t*>(d), static_cast<size_t>(count) * 2);
    } else if (cmd == "prune_pairs") {  // n norm pc
        uint32_t pc = I(2);
        auto s = dev_in<Site>("sites");
        auto r = dev_in<float>("removal");
        auto p = dev_zero<uint2>(pc);
        launchComputePruneScorePairs(s, r, p, I(0), F(1), pc, st);
        dev_out("pairs", reinterpret_cast<uint32_t*>(p), static_cast<size_t>(pc) * 2);
    } else if (cmd == "densify_pairs") {  // n min_mass alpha pc
        uint32_t pc = I(3);
        auto s = dev_in<Site>("sites");
        auto m = dev_in<float>("mass"), e = dev_in<float>("energy");
        auto p = dev_zero<uint2>(pc);
        launchComputeDensifyScorePairs(s, m, e, p, I(0), F(1), F(2), pc, st);
        dev_out("pairs", reinterpret_cast<uint32_t*>(p), static_cast<size_t>(pc) * 2);
    } else if (cmd == "split") {  // cap k cur w h
        uint32_t cap = I(0);
        auto s = dev_in<Site>("sites");
        auto a = adam_in("adam", cap);
        auto idx = dev_in<uint32_t>("idx");
        const float* st7[7];
        for (int k = 0; k < 7; ++k) st7[k] = dev_in<float>("st" + std::to_string(k));
        auto tg = dev_in<float3>("target");
        launchSplitSites(s, a, idx, I(1), st7[0], st7[1], st7[2], st7[3], st7[4], st7[5], st7[6], I(2), tg,
                         N(3), N(4), st);
        dev_out("sites_out", reinterpret_cast<float*>(s), static_cast<size_t>(cap) * 10);
        adam_out("adam_out", a, cap);
    } else if (cmd == "stats") {  // n inv w h cw ch
        uint32_t n = I(0);
        auto c0 = dev_in<uint32_t>("cand0"), c1 = dev_in<uint32_t>("cand1");
        auto tg = dev_in<float3>("target");
        auto mk = dev_in<float>("mask");
        auto s = dev_in<Site>("sites");
        float* o[8];
        for (auto& p : o) p = dev_zero<float>(n);
        launchComputeSiteStatsSimple(c0, c1, tg, mk, s, F(1), n, o[0], o[1], o[2], o[3], o[4], o[5],
                                     o[6], o[7], N(2), N(3), N(4), N(5), st);
        for (int k = 0; k < 8; ++k) dev_out("st" + std::to_string(k), o[k], n);
    } else if (cmd == "prune") {  // k
        size_t cnt;
        auto s = dev_in<Site>("sites", &cnt);
        auto idx = dev_in<uint32_t>("idx");
        launchPruneSitesByIndex(s, idx, I(0), st);
        dev_out("sites_out", reinterpret_cast<float*>(s), cnt * 10);
    } else {
        fprintf(stderr, "unknown command %s\n", cmd.c_str());
        return 1;
    }
    CK(cudaDeviceSynchronize());
    return 0;
}
