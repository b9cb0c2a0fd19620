// main.cpp -- sad_cuda: the command-line host of the reference's CUDA backend
// (backends/cuda/src/sad_cuda.cu) rebuilt on libsad_gb300's C ABI.
//
//   sad_cuda <image.png|jpg> [training options] fit; writes <out-dir>/<stem>.png and
//                                                <out-dir>/<stem>_sites.txt
//   sad_cuda --render <sites.txt|json> [opts]   render; writes <sites>_render.png
//
// Same flags, defaults ($CONFIG_PATH or ./training_config.json, required) and exit codes as the
// reference (sad_cuda.cu:459-517 defaults, 754-895 flags, unknown flag -> exit 1); the log
// lines keep the reference's layout.
// Images are PNG or baseline JPEG (the reference reads any stb format); an image larger
// than MAX_DIM is box-filtered down.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "json.h"
#include "png.h"
#include "sad_gb300.h"

namespace fs = std::filesystem;
using sadcli::Image8;
using sadcli::Json;

namespace {

[[noreturn]] void die(const std::string& msg) {
    std::fprintf(stderr, "%s\n", msg.c_str());
    std::exit(1);
}

void check(sad_status_t st, const char* what) {
    if (st != SAD_OK) die(std::string(what) + ": " + sad_last_error());
}

void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) die(std::string(what) + ": " + cudaGetErrorString(e));
}

std::string read_file(const std::string& path) {
    std::ifstream f(path);
    if (!f) return {};
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

// ---------------------------------------------------------------------------
// defaults: ./training_config.json (sad_cuda.cu:459-517)
// ---------------------------------------------------------------------------
struct Defaults {
    sad_train_config_t train;
    int max_dim = 4096;
};

Defaults load_defaults() {
    Defaults d;
    sad_train_config_default(&d.train);
    // $CONFIG_PATH (exported by run.sh) first, then ./training_config.json as the
    // reference's binary reads it
    const char* env = std::getenv("CONFIG_PATH");
    std::string text = env && *env ? read_file(env) : std::string();
    if (text.empty()) text = read_file("training_config.json");
    if (text.empty()) die("Missing training_config.json (required).");
    Json j;
    try {
        j = sadcli::JsonParser(text).parse();
    } catch (const std::exception& e) {
        die(std::string("training_config.json: ") + e.what());
    }
    sad_train_config_t& c = d.train;
    auto num = [&](const char* k) -> double {
        try {
            return j.at(k).number();
        } catch (const std::exception& e) {
            die(std::string("training_config.json: ") + k + ": " + e.what());
        }
    };
    auto seti = [&](const char* k, int& v) { if (j.has(k)) v = static_cast<int>(num(k)); };
    auto setu = [&](const char* k, uint32_t& v) { if (j.has(k)) v = static_cast<uint32_t>(num(k)); };
    auto setf = [&](const char* k, float& v) { if (j.has(k)) v = static_cast<float>(num(k)); };
    seti("DEFAULT_SITES", c.n_sites);
    seti("DEFAULT_MAX_SITES", c.max_sites);
    seti("DEFAULT_ITERS", c.iterations);
    setf("DEFAULT_TARGET_BPP", c.target_bpp);
    setf("PRUNE_PERCENTILE", c.prune_percentile);
    seti("PRUNE_DURING_DENSIFY", c.prune_during_densify);
    seti("PRUNE_START", c.prune_start);
    seti("PRUNE_FREQ", c.prune_freq);
    seti("PRUNE_END", c.prune_end);
    seti("DENSIFY_START", c.densify_start);
    seti("DENSIFY_FREQ", c.densify_freq);
    seti("DENSIFY_END", c.densify_end);
    setf("DENSIFY_PERCENTILE", c.densify_percentile);
    setf("DENSIFY_SCORE_ALPHA", c.densify_score_alpha);
    seti("CAND_UPDATE_FREQ", c.cand_update_freq);
    seti("CAND_UPDATE_PASSES", c.cand_update_passes);
    seti("CAND_DOWNSCALE", c.cand_downscale);
    setf("CAND_RADIUS_SCALE", c.cand_radius_scale);
    setu("CAND_RADIUS_PROBES", c.cand_radius_probes);
    setu("CAND_INJECT_COUNT", c.cand_inject_count);
    setu("CAND_HILBERT_WINDOW", c.cand_hilbert_window);
    setu("CAND_HILBERT_PROBES", c.cand_hilbert_probes);
    setf("LR_POS_BASE", c.lr_pos);
    setf("LR_TAU_BASE", c.lr_tau);
    setf("LR_RADIUS_BASE", c.lr_radius);
    setf("LR_COLOR_BASE", c.lr_color);
    setf("LR_DIR_BASE", c.lr_dir);
    setf("LR_ANISO_BASE", c.lr_aniso);
    setf("BETA1", c.beta1);
    setf("BETA2", c.beta2);
    setf("EPS", c.eps);
    seti("MAX_DIM", d.max_dim);
    if (!j.has("INIT_LOG_TAU") || !j.has("INIT_RADIUS"))
        die("INIT_LOG_TAU and INIT_RADIUS must be set in training_config.json");
    setf("INIT_LOG_TAU", c.init_log_tau);
    setf("INIT_RADIUS", c.init_radius);
    return d;
}

// ---------------------------------------------------------------------------
// images (sad_cuda.cu:137-229)
// ---------------------------------------------------------------------------
Image8 load_image_or_die(const std::string& path, const char* what) {
    try {
        return sadcli::read_image(path);
    } catch (const std::exception& e) {
        die(std::string("Failed to load ") + what + ": " + path + " (" + e.what() + ")");
    }
}

// Box-filter resample of an 8-bit image to (w, h) (area average per output pixel).
Image8 resample(const Image8& in, int w, int h) {
    Image8 out;
    out.width = w;
    out.height = h;
    out.gray = in.gray;
    out.rgb.resize(static_cast<size_t>(w) * h * 3);
    const double sx = double(in.width) / w, sy = double(in.height) / h;
    for (int y = 0; y < h; ++y) {
        int y0 = int(std::floor(y * sy)), y1 = std::max(y0 + 1, int(std::ceil((y + 1) * sy)));
        for (int x = 0; x < w; ++x) {
            int x0 = int(std::floor(x * sx)), x1 = std::max(x0 + 1, int(std::ceil((x + 1) * sx)));
            double acc[3] = {0, 0, 0};
            int cnt = 0;
            for (int yy = y0; yy < std::min(y1, in.height); ++yy)
                for (int xx = x0; xx < std::min(x1, in.width); ++xx, ++cnt)
                    for (int c = 0; c < 3; ++c) acc[c] += in.rgb[(size_t(yy) * in.width + xx) * 3 + c];
            for (int c = 0; c < 3; ++c)
                out.rgb[(size_t(y) * w + x) * 3 + c] = uint8_t(std::lround(acc[c] / std::max(1, cnt)));
        }
    }
    return out;
}

std::vector<float> to_float_rgb(const Image8& img) {
    std::vector<float> v(img.rgb.size());
    for (size_t i = 0; i < v.size(); ++i) v[i] = img.rgb[i] / 255.0f;
    return v;
}

// Mask: one channel in [0, 1] (grey files directly; colour files through an integer
// luma, (77 r + 150 g + 29 b) >> 8), resampled to the target size.
std::vector<float> load_mask(const std::string& path, int w, int h) {
    Image8 m = load_image_or_die(path, "mask");
    if (m.width != w || m.height != h) m = resample(m, w, h);
    std::vector<float> out(static_cast<size_t>(w) * h);
    for (size_t i = 0; i < out.size(); ++i) {
        const uint8_t* p = &m.rgb[i * 3];
        int v = m.gray ? p[0] : (p[0] * 77 + p[1] * 150 + p[2] * 29) >> 8;
        out[i] = v / 255.0f;
    }
    return out;
}

bool save_render(const std::string& path, const std::vector<float>& rgb, int w, int h) {
    std::vector<uint8_t> out(rgb.size());
    for (size_t i = 0; i < rgb.size(); ++i)
        out[i] = static_cast<uint8_t>(std::lround(std::clamp(rgb[i], 0.0f, 1.0f) * 255.0f));
    return sadcli::write_png(path, out.data(), w, h);
}

// ---------------------------------------------------------------------------
// sites files (sad_cuda.cu:277-420): TXT is pos, rgb, log_tau, radius[, dir, log_aniso];
// the device layout is pos, log_tau, radius, rgb, dir, log_aniso
// ---------------------------------------------------------------------------
struct LoadedSites {
    std::vector<float> sites;  // [n][10] device layout
    int width = 0, height = 0;
    bool has_size = false;
    size_t count() const { return sites.size() / 10; }
};

void push_site(LoadedSites& s, float px, float py, float r, float g, float b, float log_tau,
               float radius, float dx, float dy, float log_aniso) {
    s.sites.insert(s.sites.end(), {px, py, log_tau, radius, r, g, b, dx, dy, log_aniso});
}

LoadedSites load_sites_txt(const std::string& path) {
    std::ifstream f(path);
    if (!f) die("Failed to open sites TXT: " + path);
    LoadedSites out;
    std::string line;
    while (std::getline(f, line)) {
        size_t a = line.find_first_not_of(" \t\r\n");
        if (a == std::string::npos) continue;
        std::string t = line.substr(a);
        if (t[0] == '#') {
            std::string lower = t;
            std::transform(lower.begin(), lower.end(), lower.begin(), ::tolower);
            if (lower.find("image size") != std::string::npos) {
                std::string nums;
                for (char c : t) nums.push_back((std::isdigit(static_cast<unsigned char>(c)) || c == '-') ? c : ' ');
                std::istringstream iss(nums);
                int w = 0, h = 0;
                if (iss >> w >> h) {
                    out.width = w;
                    out.height = h;
                }
            }
            continue;
        }
        std::istringstream iss(t);
        std::vector<float> v;
        float x;
        while (iss >> x) v.push_back(x);
        if (v.size() == 7)
            push_site(out, v[0], v[1], v[2], v[3], v[4], v[5], v[6], 1.0f, 0.0f, 0.0f);
        else if (v.size() == 10)
            push_site(out, v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[9]);
    }
    if (out.sites.empty()) die("No sites found in TXT: " + path);
    out.has_size = out.width > 0 && out.height > 0;
    return out;
}

LoadedSites load_sites_json(const std::string& path) {
    std::string text = read_file(path);
    if (text.empty()) die("Failed to open sites JSON: " + path);
    LoadedSites out;
    try {
        Json j = sadcli::JsonParser(text).parse();
        out.width = static_cast<int>(j.at("image_width").number());
        out.height = static_cast<int>(j.at("image_height").number());
        out.has_size = true;
        for (const Json& s : j.at("sites").arr) {
            const Json& pos = s.at("pos");
            const Json& col = s.at("color");
            float radius = s.has("radius") ? float(s.at("radius").number())
                           : s.has("radius_sq") ? float(s.at("radius_sq").number()) : 0.0f;
            float dx = 1.0f, dy = 0.0f;
            if (s.has("aniso_dir")) {
                const auto& d = s.at("aniso_dir").arr;
                if (d.size() > 0) dx = float(d[0].number());
                if (d.size() > 1) dy = float(d[1].number());
            }
            push_site(out, float(pos.arr.at(0).number()), float(pos.arr.at(1).number()),
                      float(col.arr.at(0).number()), float(col.arr.at(1).number()),
                      float(col.arr.at(2).number()), float(s.at("log_tau").number()), radius, dx, dy,
                      s.has("log_aniso") ? float(s.at("log_aniso").number()) : 0.0f);
        }
    } catch (const std::exception& e) {
        die("Failed to read sites JSON " + path + ": " + e.what());
    }
    if (out.sites.empty()) die("No sites found in JSON: " + path);
    return out;
}

LoadedSites load_sites(const std::string& path) {
    std::string ext = fs::path(path).extension().string();
    std::transform(ext.begin(), ext.end(), ext.begin(), ::tolower);
    return ext == ".json" ? load_sites_json(path) : load_sites_txt(path);
}

bool write_sites_txt(const std::string& path, const std::vector<float>& sites, int w, int h) {
    std::FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    std::fprintf(f, "# SAD Sites (position_x, position_y, color_r, color_g, color_b, log_tau, radius, "
                    "aniso_dir_x, aniso_dir_y, log_aniso)\n");
    std::fprintf(f, "# Image size: %d %d\n", w, h);
    std::fprintf(f, "# Total sites: %zu\n", sites.size() / 10);
    for (size_t i = 0; i + 9 < sites.size(); i += 10) {
        const float* s = &sites[i];
        std::fprintf(f, "%.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g\n", s[0], s[1], s[4], s[5],
                     s[6], s[2], s[3], s[7], s[8], s[9]);
    }
    return std::fclose(f) == 0;
}

// ---------------------------------------------------------------------------
// arguments (sad_cuda.cu:754-895)
// ---------------------------------------------------------------------------
enum class InitMode { Gradient, PerPixel, FromSites };

struct Options {
    bool render = false;
    std::string image, sites_path, out_dir = "results", mask, init_sites, out_path, render_target;
    sad_train_config_t cfg;
    sad_render_config_t rcfg;
    InitMode init = InitMode::Gradient;
    bool ssim_metric = false;
    bool packed_psnr = false;     // Metal CLI --packed-psnr
    bool render_packed = false;   // Metal CLI --render-packed
    int width = 0, height = 0, max_dim = 4096;
};

void usage(const Defaults& d) {
    const sad_train_config_t& c = d.train;
    std::printf("Usage:\n  sad_cuda <image_path> [options]\n  sad_cuda --render <sites.txt> [options]\n\n");
    std::printf("Common options:\n  --help, -h            Show this help\n  --out-dir <path>      Output directory (default: results)\n\n");
    std::printf("Training options:\n");
    std::printf("  --sites N             Number of sites (default: %d)\n", c.n_sites);
    std::printf("  --iters N             Iterations (default: %d)\n", c.iterations);
    std::printf("  --target-bpp F         Target bits-per-pixel\n");
    std::printf("  --mask <path>          Optional mask image (white=keep, black=ignore)\n");
    std::printf("  --init-per-pixel       Per-pixel initialization\n");
    std::printf("  --init-gradient        Gradient-weighted init (default)\n");
    std::printf("  --init-from-sites <p>  Initialize from sites file\n");
    std::printf("  --init-gradient-alpha F Gradient init threshold scale\n");
    std::printf("  --densify              Enable densification\n");
    std::printf("  --prune-during-densify Allow pruning during densification\n");
    std::printf("  --prune-start N        Prune start (default: %d)\n", c.prune_start);
    std::printf("  --prune-end N          Prune end (default: %d)\n", c.prune_end);
    std::printf("  --prune-freq N         Prune frequency (default: %d)\n", c.prune_freq);
    std::printf("  --prune-percentile F   Prune percentile (default: %g)\n", c.prune_percentile);
    std::printf("  --densify-start N      Densify start (default: %d)\n", c.densify_start);
    std::printf("  --densify-end N        Densify end (default: %d)\n", c.densify_end);
    std::printf("  --densify-freq N       Densify frequency (default: %d)\n", c.densify_freq);
    std::printf("  --densify-percentile F Densify percentile (default: %g)\n", c.densify_percentile);
    std::printf("  --densify-score-alpha F Densify score alpha (default: %g)\n", c.densify_score_alpha);
    std::printf("  --cand-freq N          Candidate update freq (default: %d)\n", c.cand_update_freq);
    std::printf("  --cand-passes N        Candidate update passes (default: %d)\n", c.cand_update_passes);
    std::printf("  --cand-downscale N     Downscale candidate textures by N (default: %d)\n", c.cand_downscale);
    std::printf("  --cand-radius-scale F  Radius probe scale (default: %g)\n", c.cand_radius_scale);
    std::printf("  --cand-radius-probes N Radius probes (default: %u)\n", c.cand_radius_probes);
    std::printf("  --cand-hilbert-window N Hilbert window for VPT candidates (default: %u)\n", c.cand_hilbert_window);
    std::printf("  --cand-hilbert-probes N Hilbert probes for VPT candidates (default: %u)\n", c.cand_hilbert_probes);
    std::printf("  --cand-inject N       Candidate random injects (default: %u)\n", c.cand_inject_count);
    std::printf("  --max-sites N          Max sites (default: %d)\n", c.max_sites);
    std::printf("  --lr F                 Learning-rate scale (default: 1)\n");
    std::printf("  --ssim                 Log SSIM\n");
    std::printf("  --packed-psnr          Re-render with the 16-byte packed sites and report PSNR\n");
    std::printf("  --ssim-weight F        SSIM weight (default: 0)\n");
    std::printf("  --log-freq N           Log frequency (default: 1000)\n\n");
    std::printf("Render options:\n");
    std::printf("  --out <path>           Output PNG path\n");
    std::printf("  --width N              Required for TXT sites if no header\n");
    std::printf("  --height N             Required for TXT sites if no header\n");
    std::printf("  --render-cand-passes N Candidate passes (default: 16)\n");
    std::printf("  --render-no-jfa         Disable JFA pre-pass\n");
    std::printf("  --render-jfa-rounds N  JFA rounds (default: 1)\n");
    std::printf("  --render-cand-downscale N Downscale candidate textures by N (default: %d)\n", c.cand_downscale);
    std::printf("  --render-hilbert-window N Hilbert window for VPT candidates (default: %u)\n", c.cand_hilbert_window);
    std::printf("  --render-hilbert-probes N Hilbert probes for VPT candidates (default: %u)\n", c.cand_hilbert_probes);
    std::printf("  --render-cand-inject N Candidate random injects (default: %u)\n", c.cand_inject_count);
    std::printf("  --render-target <path> Optional target image for PSNR\n");
    std::printf("  --render-packed        Render through the 16-byte packed site format\n");
}

Options parse_args(int argc, char** argv, const Defaults& d) {
    Options o;
    o.cfg = d.train;
    o.cfg.densify = 1;
    o.cfg.log_freq = 1000;
    o.max_dim = d.max_dim;
    sad_render_config_default(&o.rcfg);
    o.rcfg.cand_downscale = d.train.cand_downscale;
    o.rcfg.cand_radius_scale = d.train.cand_radius_scale;
    o.rcfg.cand_radius_probes = d.train.cand_radius_probes;
    o.rcfg.cand_inject_count = d.train.cand_inject_count;
    o.rcfg.cand_hilbert_window = d.train.cand_hilbert_window;
    o.rcfg.cand_hilbert_probes = d.train.cand_hilbert_probes;
    std::vector<std::string> a(argv + 1, argv + argc);
    auto need = [&](size_t& i, const std::string& f) -> const std::string& {
        if (i + 1 >= a.size()) die("Missing value for " + f);
        return a[++i];
    };
    auto num_i = [&](size_t& i, const std::string& f) {
        const std::string& v = need(i, f);
        try {
            return std::stoi(v);
        } catch (...) {
            die("Invalid integer for " + f + ": " + v);
        }
    };
    auto num_f = [&](size_t& i, const std::string& f) {
        const std::string& v = need(i, f);
        try {
            return std::stof(v);
        } catch (...) {
            die("Invalid number for " + f + ": " + v);
        }
    };
    sad_train_config_t& c = o.cfg;
    for (size_t i = 0; i < a.size(); ++i) {
        const std::string& f = a[i];
        if (f == "--help" || f == "-h") {
            usage(d);
            std::exit(0);
        } else if (f == "--render") {
            o.render = true;
            o.sites_path = need(i, f);
        } else if (f.rfind("--", 0) != 0) {
            if (!o.image.empty()) die("Unexpected argument: " + f);
            o.image = f;
        } else if (f == "--sites") c.n_sites = num_i(i, f);
        else if (f == "--iters") c.iterations = num_i(i, f);
        else if (f == "--target-bpp") c.target_bpp = num_f(i, f);
        else if (f == "--mask") o.mask = need(i, f);
        else if (f == "--init-per-pixel") o.init = InitMode::PerPixel;
        else if (f == "--init-gradient") o.init = InitMode::Gradient;
        else if (f == "--init-from-sites") {
            o.init = InitMode::FromSites;
            o.init_sites = need(i, f);
        } else if (f == "--init-gradient-alpha") c.init_gradient_alpha = num_f(i, f);
        else if (f == "--densify") c.densify = 1;
        else if (f == "--densify-start") c.densify_start = num_i(i, f);
        else if (f == "--densify-end") c.densify_end = num_i(i, f);
        else if (f == "--densify-freq") c.densify_freq = num_i(i, f);
        else if (f == "--densify-percentile") c.densify_percentile = num_f(i, f);
        else if (f == "--densify-score-alpha") c.densify_score_alpha = num_f(i, f);
        else if (f == "--prune-during-densify") c.prune_during_densify = 1;
        else if (f == "--prune-start") c.prune_start = num_i(i, f);
        else if (f == "--prune-end") c.prune_end = num_i(i, f);
        else if (f == "--prune-freq") c.prune_freq = num_i(i, f);
        else if (f == "--prune-percentile") c.prune_percentile = num_f(i, f);
        else if (f == "--cand-freq") c.cand_update_freq = num_i(i, f);
        else if (f == "--cand-passes") c.cand_update_passes = num_i(i, f);
        else if (f == "--cand-downscale") c.cand_downscale = num_i(i, f);
        else if (f == "--cand-radius-scale") c.cand_radius_scale = num_f(i, f);
        else if (f == "--cand-radius-probes") c.cand_radius_probes = static_cast<uint32_t>(num_i(i, f));
        else if (f == "--cand-inject-count" || f == "--cand-inject") c.cand_inject_count = static_cast<uint32_t>(num_i(i, f));
        else if (f == "--cand-hilbert-window") c.cand_hilbert_window = static_cast<uint32_t>(num_i(i, f));
        else if (f == "--cand-hilbert-probes") c.cand_hilbert_probes = static_cast<uint32_t>(num_i(i, f));
        else if (f == "--max-sites") c.max_sites = num_i(i, f);
        else if (f == "--lr") c.lr_scale = num_f(i, f);
        else if (f == "--ssim") o.ssim_metric = true;
        else if (f == "--packed-psnr") o.packed_psnr = true;
        else if (f == "--render-packed") o.render_packed = true;
        else if (f == "--ssim-weight") c.ssim_weight = num_f(i, f);
        else if (f == "--log-freq") c.log_freq = num_i(i, f);
        else if (f == "--out-dir") o.out_dir = need(i, f);
        else if (f == "--out") o.out_path = need(i, f);
        else if (f == "--width") o.width = num_i(i, f);
        else if (f == "--height") o.height = num_i(i, f);
        else if (f == "--render-cand-passes") o.rcfg.candidate_passes = num_i(i, f);
        else if (f == "--render-no-jfa") o.rcfg.use_jfa = 0;
        else if (f == "--render-jfa-rounds") o.rcfg.jfa_rounds = num_i(i, f);
        else if (f == "--render-cand-downscale") o.rcfg.cand_downscale = num_i(i, f);
        else if (f == "--render-hilbert-window") o.rcfg.cand_hilbert_window = static_cast<uint32_t>(num_i(i, f));
        else if (f == "--render-hilbert-probes") o.rcfg.cand_hilbert_probes = static_cast<uint32_t>(num_i(i, f));
        else if (f == "--render-cand-inject") o.rcfg.cand_inject_count = static_cast<uint32_t>(num_i(i, f));
        else if (f == "--render-target") o.render_target = need(i, f);
        else {
            std::fprintf(stderr, "Unknown option: %s\n", f.c_str());
            usage(d);
            std::exit(1);
        }
    }
    if (o.render_packed && !o.render) die("Error: --render-packed is only valid in render mode");
    if (!o.render && o.image.empty()) {
        usage(d);
        std::exit(1);
    }
    return o;
}

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
template <class T>
struct DeviceBuf {
    T* p = nullptr;
    explicit DeviceBuf(size_t n) { check_cuda(cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(T)), "cudaMalloc"); }
    ~DeviceBuf() { cudaFree(p); }
};

float psnr_of(float mse_sum, double npix) {
    float mse = mse_sum / static_cast<float>(std::max(1.0, npix) * 3.0);
    return mse > 0.0f ? 20.0f * std::log10(1.0f / std::sqrt(mse)) : 100.0f;
}

// ---------------------------------------------------------------------------
// training (sad_cuda.cu:1860-2533)
// ---------------------------------------------------------------------------
int train(Options& o) {
    const auto t_start = std::chrono::steady_clock::now();
    Image8 img = load_image_or_die(o.image, "image");
    if (o.max_dim > 0 && std::max(img.width, img.height) > o.max_dim) {
        double s = double(o.max_dim) / std::max(img.width, img.height);
        img = resample(img, std::max(1, int(std::lround(img.width * s))), std::max(1, int(std::lround(img.height * s))));
    }
    const int w = img.width, h = img.height;
    std::vector<float> target = to_float_rgb(img);
    std::vector<float> mask;
    double mask_sum = double(w) * h;
    if (!o.mask.empty()) {
        mask = load_mask(o.mask, w, h);
        mask_sum = 0;
        for (float v : mask) mask_sum += v > 0.0f;
    }
    sad_train_config_t& c = o.cfg;
    std::vector<float> init_sites;
    if (o.init == InitMode::PerPixel) {
        c.n_sites = w * h;
        c.init_per_pixel = 1;
        init_sites.reserve(static_cast<size_t>(w) * h * 10);
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                const float* col = &target[(size_t(y) * w + x) * 3];
                init_sites.insert(init_sites.end(), {float(x), float(y), c.init_log_tau, c.init_radius,
                                                     col[0], col[1], col[2], 1.0f, 0.0f, 0.0f});
            }
    } else if (o.init == InitMode::FromSites) {
        LoadedSites ls = load_sites(o.init_sites);
        if (ls.has_size && (ls.width != w || ls.height != h)) {
            float sx = float(w) / float(ls.width), sy = float(h) / float(ls.height);
            for (size_t i = 0; i < ls.count(); ++i) {
                ls.sites[i * 10] *= sx;
                ls.sites[i * 10 + 1] *= sy;
            }
        }
        init_sites = std::move(ls.sites);
        c.n_sites = static_cast<int>(init_sites.size() / 10);
    }
    const int log_freq = std::max(1, c.log_freq);
    c.log_freq = 0;  // this host prints the log lines
    sad_trainer_t* t = nullptr;
    check(sad_trainer_create(&c, w, h, &t), "sad_trainer_create");
    sad_trainer_info_t info;
    check(sad_trainer_info(t, &info), "sad_trainer_info");

    int active0 = c.n_sites;
    if (!init_sites.empty()) {
        active0 = 0;
        for (size_t i = 0; i < init_sites.size(); i += 10) active0 += init_sites[i] >= 0.0f;
    }
    std::printf("Training | backend=cuda | image=%dx%d | sites=%d/%d | iters=%d | log-freq=%d | mask=%s | out=%s",
                w, h, active0, c.n_sites, c.iterations, log_freq, o.mask.empty() ? "no" : "yes",
                o.out_dir.c_str());
    if (c.target_bpp > 0.0f) std::printf(" | target-bpp=%.3f", c.target_bpp);
    std::printf("\n");
    const char* init_name = o.init == InitMode::FromSites ? "sites" : o.init == InitMode::PerPixel ? "per-pixel" : "gradient";
    std::printf("Schedule | init=%s | densify=", init_name);
    if (c.densify) std::printf("on cap=%d", info.capacity); else std::printf("off");
    std::printf(" | prune=");
    if (info.prune_percentile > 0.0f)
        std::printf("on %.3f @%d-%d/%d", info.prune_percentile, c.prune_start,
                    c.prune_end > 0 ? c.prune_end : c.iterations - 1, std::max(1, c.prune_freq));
    else
        std::printf("off");
    std::printf(" | cand=freq %d, passes %d, downscale %dx", c.cand_update_freq, c.cand_update_passes, c.cand_downscale);
    if (c.cand_hilbert_probes > 0 && c.cand_hilbert_window > 0)
        std::printf(" hilbert=%ux%u", c.cand_hilbert_probes, c.cand_hilbert_window);
    std::printf("\n");

    check(sad_trainer_set_target_host(t, target.data(), mask.empty() ? nullptr : mask.data()), "set target");
    check(sad_trainer_init(t, init_sites.empty() ? nullptr : init_sites.data(),
                           static_cast<int>(init_sites.size() / 10)), "sad_trainer_init");
    check_cuda(cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(sad_trainer_stream(t))), "init");

    const size_t npix = static_cast<size_t>(w) * h;
    DeviceBuf<float> d_render(npix * 3), d_target(npix * 3), d_mask(npix), d_acc(2);
    if (o.ssim_metric) {
        std::vector<float> ones(npix, 1.0f);
        check_cuda(cudaMemcpy(d_target.p, target.data(), npix * 12, cudaMemcpyHostToDevice), "upload");
        check_cuda(cudaMemcpy(d_mask.p, mask.empty() ? ones.data() : mask.data(), npix * 4, cudaMemcpyHostToDevice), "upload");
    }
    std::printf("Logs | Iter | PSNR | Active | speed | elapsed\n");
    std::fflush(stdout);
    const auto t0 = std::chrono::steady_clock::now();
    float final_psnr = 0.0f, best_psnr = 0.0f, final_ssim = 0.0f, best_ssim = 0.0f;
    std::vector<float> host_sites;
    for (int it = 0; it < c.iterations; ++it) {
        bool log = it % log_freq == 0 || it == c.iterations - 1;
        if (!log) continue;
        check(sad_trainer_run(t, it + 1), "sad_trainer_run");
        float psnr = 0.0f;
        check(sad_trainer_render(t, d_render.p, &psnr), "sad_trainer_render");
        float ssim = 0.0f;
        if (o.ssim_metric) {
            check_cuda(cudaMemset(d_acc.p, 0, 8), "memset");
            check(sad_compute_ssim(d_render.p, d_target.p, d_mask.p, d_acc.p, w, h,
                                   sad_trainer_stream(t)), "sad_compute_ssim");
            float sum = 0.0f;
            check_cuda(cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(sad_trainer_stream(t))), "sync");
            check_cuda(cudaMemcpy(&sum, d_acc.p, 4, cudaMemcpyDeviceToHost), "download");
            ssim = sum / static_cast<float>(std::max(1.0, mask_sum));
        }
        check(sad_trainer_info(t, &info), "sad_trainer_info");
        host_sites.resize(static_cast<size_t>(info.site_buffer) * 10);
        int written = 0;
        check(sad_trainer_get_sites(t, host_sites.data(), info.site_buffer, 1, &written), "get sites");
        double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::printf("Iter %4d | PSNR: %.2f dB", it, psnr);
        if (o.ssim_metric) std::printf(" | SSIM: %.4f", ssim);
        std::printf(" | Active: %d/%d | %.1f it/s | %.1fs\n", written, info.site_buffer,
                    el > 0 ? (it + 1) / el : 0.0, el);
        std::fflush(stdout);
        final_psnr = psnr;
        best_psnr = std::max(best_psnr, psnr);
        final_ssim = ssim;
        best_ssim = std::max(best_ssim, ssim);
    }
    const double train_time = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

    std::vector<float> render(npix * 3);
    float psnr = 0.0f;
    check(sad_trainer_render(t, d_render.p, &psnr), "final render");
    check_cuda(cudaMemcpy(render.data(), d_render.p, npix * 12, cudaMemcpyDeviceToHost), "download");
    std::error_code ec;
    fs::create_directories(o.out_dir, ec);
    std::string stem = fs::path(o.image).stem().string();
    std::string png_path = (fs::path(o.out_dir) / (stem + ".png")).string();
    std::string sites_path = (fs::path(o.out_dir) / (stem + "_sites.txt")).string();
    if (save_render(png_path, render, w, h))
        std::printf("Saved: %s\n", png_path.c_str());
    else
        std::fprintf(stderr, "Failed to save: %s\n", png_path.c_str());
    check(sad_trainer_info(t, &info), "sad_trainer_info");
    host_sites.resize(static_cast<size_t>(info.site_buffer) * 10);
    int written = 0;
    check(sad_trainer_get_sites(t, host_sites.data(), info.site_buffer, 1, &written), "get sites");
    host_sites.resize(static_cast<size_t>(written) * 10);
    if (write_sites_txt(sites_path, host_sites, w, h))
        std::printf("Saved: %s\n", sites_path.c_str());
    else
        std::fprintf(stderr, "Failed to write sites: %s\n", sites_path.c_str());
    if (o.packed_psnr) {
        float packed_psnr = 0.0f;
        check(sad_trainer_render_packed(t, d_render.p, &packed_psnr, nullptr), "sad_trainer_render_packed");
        check_cuda(cudaMemcpy(render.data(), d_render.p, npix * 12, cudaMemcpyDeviceToHost), "download");
        std::string packed_path = (fs::path(o.out_dir) / (stem + "_packed.png")).string();
        if (save_render(packed_path, render, w, h))
            std::printf("Saved: %s\n", packed_path.c_str());
        std::printf("Packed inference PSNR: %.2f dB\n", packed_psnr);
    }
    std::printf("Final PSNR: %.1f dB (best %.1f)\n", final_psnr, best_psnr);
    if (o.ssim_metric) std::printf("Final SSIM: %.4f (best %.4f)\n", final_ssim, best_ssim);
    std::printf("Training time: %.2f s\n", train_time);
    std::printf("Total time: %.2f s\n",
                std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count());
    sad_trainer_destroy(t);
    return 0;
}

// ---------------------------------------------------------------------------
// render-only (sad_cuda.cu:1678-1858)
// ---------------------------------------------------------------------------
int render(Options& o) {
    LoadedSites ls = load_sites(o.sites_path);
    int w = ls.has_size ? ls.width : o.width;
    int h = ls.has_size ? ls.height : o.height;
    if (w <= 0 || h <= 0) die("TXT sites require --width and --height or a header line with image size.");
    const uint32_t n = static_cast<uint32_t>(ls.count());
    std::printf("Loaded %u sites\nRender size: %dx%d\n", n, w, h);
    const size_t npix = static_cast<size_t>(w) * h;
    DeviceBuf<float> d_sites(ls.sites.size()), d_out(npix * 3);
    check_cuda(cudaMemcpy(d_sites.p, ls.sites.data(), ls.sites.size() * 4, cudaMemcpyHostToDevice), "upload");
    size_t scratch_bytes = sad_render_scratch_bytes(n, w, h, o.rcfg.cand_downscale);
    DeviceBuf<unsigned char> d_scratch(scratch_bytes);
    DeviceBuf<uint32_t> d_packed(o.render_packed ? size_t(n) * 4 : 1);
    DeviceBuf<sad_packed_quant_t> d_quant(1);
    if (o.render_packed) {
        // 16-byte sites: pack, then render what they decode to (the packed render path)
        if (w > 32768 || h > 32768) die("--render-packed: image side above 32768");
        check(sad_pack_inference_sites(d_sites.p, n, w, h, d_packed.p, d_quant.p, nullptr),
              "sad_pack_inference_sites");
        check(sad_unpack_inference_sites(d_packed.p, d_quant.p, n, w, h, d_sites.p, nullptr),
              "sad_unpack_inference_sites");
        std::printf("Packed inference sites: %u x 16 bytes\n", n);
    }
    float cand_ms = 0.0f, render_ms = 0.0f;
    check(sad_render_from_sites_timed(&o.rcfg, d_sites.p, n, w, h, d_out.p, d_scratch.p, scratch_bytes, nullptr,
                                      &cand_ms, &render_ms),
          "sad_render_from_sites");
    if (!o.render_target.empty()) {
        Image8 timg = load_image_or_die(o.render_target, "render target");
        if (timg.width != w || timg.height != h) {
            std::fprintf(stderr, "Render target size mismatch; skipping PSNR.\n");
        } else {
            std::vector<float> tf = to_float_rgb(timg);
            DeviceBuf<float> d_t(npix * 3), d_acc(1);
            check_cuda(cudaMemcpy(d_t.p, tf.data(), npix * 12, cudaMemcpyHostToDevice), "upload");
            check_cuda(cudaMemset(d_acc.p, 0, 4), "memset");
            check(sad_compute_mse(d_out.p, d_t.p, nullptr, d_acc.p, w, h, nullptr), "sad_compute_mse");
            float sum = 0.0f;
            check_cuda(cudaMemcpy(&sum, d_acc.p, 4, cudaMemcpyDeviceToHost), "download");
            std::printf("Render PSNR: %.2f dB\n", psnr_of(sum, double(npix)));
        }
    }
    std::printf("Candidate build: %.3f ms | Render: %.3f ms\n", cand_ms, render_ms);
    std::vector<float> out(npix * 3);
    check_cuda(cudaMemcpy(out.data(), d_out.p, npix * 12, cudaMemcpyDeviceToHost), "download");
    std::string out_path = o.out_path.empty()
                               ? (fs::path(o.sites_path).replace_extension("").string() + "_render.png")
                               : o.out_path;
    if (save_render(out_path, out, w, h))
        std::printf("Saved: %s\n", out_path.c_str());
    else
        std::fprintf(stderr, "Failed to save: %s\n", out_path.c_str());
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    Defaults d = load_defaults();
    Options o = parse_args(argc, argv, d);
    return o.render ? render(o) : train(o);
}
