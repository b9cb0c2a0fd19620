// jpeg.cpp -- baseline JPEG reading for the command-line host (ITU-T T.81 / JFIF).
//
// Sequential Huffman-coded DCT (SOF0 / SOF1), 8-bit samples, one (grey) or three (YCbCr)
// components with sampling factors 1-2, restart intervals.  Decoding per T.81 Annex F:
// canonical Huffman codes from DHT, DC prediction per component, run-length AC
// coefficients in zig-zag order, dequantisation, a separable float 8x8 inverse DCT, level
// shift and clamping; half-resolution chroma brought up by a triangle filter (the IJG
// decoder's default upsampling); JFIF YCbCr -> RGB.
// Progressive and arithmetic-coded files are rejected with a message.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <fstream>
#include <iterator>
#include <stdexcept>
#include <string>
#include <vector>

#include "png.h"

namespace sadcli {
namespace {

constexpr int kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                             12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                             35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                             58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

struct Huffman {
    // canonical code tables: for each length l, codes [min[l], max[l]] map to symbols
    // starting at index offset[l] of `symbols`
    int min_code[17] = {};
    int max_code[17] = {};
    int offset[17] = {};
    std::vector<uint8_t> symbols;
    bool defined = false;
};

struct Component {
    int id = 0, h = 1, v = 1, tq = 0;
    int td = 0, ta = 0;
    int dc_pred = 0;
    int bw = 0, bh = 0;            // plane size in blocks (padded to whole MCUs)
    std::vector<uint8_t> plane;    // bw*8 x bh*8 samples
};

class BitReader {
public:
    BitReader(const std::vector<uint8_t>& d, size_t pos) : d_(d), pos_(pos) {}
    int bit() {
        if (nbits_ == 0) fill();
        --nbits_;
        return (acc_ >> nbits_) & 1;
    }
    int bits(int n) {
        int v = 0;
        for (int i = 0; i < n; ++i) v = (v << 1) | bit();
        return v;
    }
    // Restart marker: drop the partial byte, expect RSTn.
    void restart() {
        nbits_ = 0;
        if (pos_ + 1 < d_.size() && d_[pos_] == 0xFF && d_[pos_ + 1] >= 0xD0 && d_[pos_ + 1] <= 0xD7)
            pos_ += 2;
        else
            throw std::runtime_error("JPEG restart marker missing");
    }
    size_t pos() const { return pos_; }

private:
    void fill() {
        if (pos_ >= d_.size()) throw std::runtime_error("truncated JPEG scan");
        uint8_t b = d_[pos_++];
        if (b == 0xFF) {
            if (pos_ >= d_.size()) throw std::runtime_error("truncated JPEG scan");
            uint8_t n = d_[pos_];
            if (n == 0x00) {
                ++pos_;  // stuffed zero
            } else {
                // a marker inside the entropy-coded data: feed ones (T.81 F.2.2.5 leaves
                // the rest of the segment to the caller) without consuming the marker
                --pos_;
                b = 0xFF;
                acc_ = b;
                nbits_ = 8;
                return;
            }
        }
        acc_ = b;
        nbits_ = 8;
    }
    const std::vector<uint8_t>& d_;
    size_t pos_;
    uint32_t acc_ = 0;
    int nbits_ = 0;
};

int decode_symbol(BitReader& br, const Huffman& hf) {
    if (!hf.defined) throw std::runtime_error("JPEG scan uses an undefined Huffman table");
    int code = 0;
    for (int l = 1; l <= 16; ++l) {
        code = (code << 1) | br.bit();
        if (hf.max_code[l] >= 0 && code <= hf.max_code[l] && code >= hf.min_code[l])
            return hf.symbols[hf.offset[l] + code - hf.min_code[l]];
    }
    throw std::runtime_error("invalid JPEG Huffman code");
}

// Value of an n-bit magnitude category (T.81 F.2.2.1, EXTEND).
int extend(int v, int n) { return n == 0 ? 0 : (v < (1 << (n - 1)) ? v - (1 << n) + 1 : v); }

uint16_t be16(const std::vector<uint8_t>& d, size_t p) {
    if (p + 1 >= d.size()) throw std::runtime_error("truncated JPEG segment");
    return static_cast<uint16_t>((d[p] << 8) | d[p + 1]);
}

struct IdctBasis {
    float c[8][8];  // c[x][u] = C(u)/2 * cos((2x+1) u pi / 16)
    IdctBasis() {
        for (int x = 0; x < 8; ++x)
            for (int u = 0; u < 8; ++u)
                c[x][u] = static_cast<float>((u == 0 ? std::sqrt(0.125) : 0.5) * std::cos((2 * x + 1) * u * 3.14159265358979323846 / 16.0));
    }
};

// Separable inverse DCT of one block (T.81 A.3.3), coefficients in natural order.
void idct8x8(const float (&in)[64], uint8_t* out, int stride) {
    static const IdctBasis basis;
    const auto& c = basis.c;
    float tmp[64];
    for (int y = 0; y < 8; ++y)      // rows: tmp[v][x] = sum_u C(u) F(v,u) cos
        for (int x = 0; x < 8; ++x) {
            float s = 0.0f;
            for (int u = 0; u < 8; ++u) s += c[x][u] * in[y * 8 + u];
            tmp[y * 8 + x] = s;
        }
    for (int x = 0; x < 8; ++x)
        for (int y = 0; y < 8; ++y) {
            float s = 0.0f;
            for (int v = 0; v < 8; ++v) s += c[y][v] * tmp[v * 8 + x];
            int p = static_cast<int>(std::lround(s + 128.0f));
            out[y * stride + x] = static_cast<uint8_t>(std::clamp(p, 0, 255));
        }
}

}  // namespace

bool is_jpeg_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    unsigned char h[3] = {0, 0, 0};
    f.read(reinterpret_cast<char*>(h), 3);
    return f.gcount() == 3 && h[0] == 0xFF && h[1] == 0xD8 && h[2] == 0xFF;
}

Image8 read_jpeg(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::vector<uint8_t> d((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    if (d.size() < 4 || d[0] != 0xFF || d[1] != 0xD8) throw std::runtime_error(path + " is not a JPEG file");
    std::array<std::array<uint16_t, 64>, 4> qt{};
    std::array<bool, 4> qt_def{};
    Huffman dc[4], ac[4];
    std::vector<Component> comps;
    int width = 0, height = 0, hmax = 1, vmax = 1, restart = 0;
    bool frame = false, done = false;
    size_t p = 2;
    while (p + 4 <= d.size() && !done) {
        if (d[p] != 0xFF) throw std::runtime_error("JPEG marker expected");
        uint8_t m = d[p + 1];
        p += 2;
        if (m == 0xFF) {  // fill byte
            --p;
            continue;
        }
        if (m == 0xD9) break;  // EOI
        uint16_t len = be16(d, p);
        if (len < 2 || p + len > d.size()) throw std::runtime_error("truncated JPEG segment");
        size_t q = p + 2, end = p + len;
        // every read of the segment stays inside it
        auto need = [&](size_t at, size_t n) {
            if (at + n > end) throw std::runtime_error("truncated JPEG segment");
        };
        switch (m) {
            case 0xDB:  // DQT
                while (q < end) {
                    int pq = d[q] >> 4, tq = d[q] & 15;
                    ++q;
                    if (tq > 3) throw std::runtime_error("invalid JPEG quantisation table id");
                    need(q, pq ? 128 : 64);
                    for (int i = 0; i < 64; ++i) {
                        if (pq) {
                            qt[tq][kZigzag[i]] = be16(d, q);
                            q += 2;
                        } else {
                            qt[tq][kZigzag[i]] = d[q++];
                        }
                    }
                    qt_def[tq] = true;
                }
                break;
            case 0xC4:  // DHT
                while (q < end) {
                    int tc = d[q] >> 4, th = d[q] & 15;
                    ++q;
                    if (tc > 1 || th > 3 || q + 16 > end) throw std::runtime_error("invalid JPEG Huffman table");
                    Huffman& hf = tc == 0 ? dc[th] : ac[th];
                    int counts[17] = {};
                    int total = 0;
                    for (int l = 1; l <= 16; ++l) total += counts[l] = d[q + l - 1];
                    q += 16;
                    if (q + total > end) throw std::runtime_error("truncated JPEG Huffman table");
                    hf.symbols.assign(d.begin() + q, d.begin() + q + total);
                    q += total;
                    int code = 0, k = 0;
                    for (int l = 1; l <= 16; ++l) {
                        hf.offset[l] = k;
                        hf.min_code[l] = code;
                        hf.max_code[l] = counts[l] ? code + counts[l] - 1 : -1;
                        code = (code + counts[l]) << 1;
                        k += counts[l];
                    }
                    hf.defined = true;
                }
                break;
            case 0xC0:
            case 0xC1: {  // SOF0 / SOF1
                need(q, 6);
                if (d[q] != 8) throw std::runtime_error("JPEG sample precision other than 8 bits is not supported");
                height = be16(d, q + 1);
                width = be16(d, q + 3);
                int nc = d[q + 5];
                if (width <= 0 || height <= 0) throw std::runtime_error("JPEG without image size");
                if (uint64_t(width) * height > (uint64_t(1) << 31)) throw std::runtime_error("JPEG dimensions too large");
                if (nc != 1 && nc != 3) throw std::runtime_error("JPEG with other than 1 or 3 components");
                if (frame) throw std::runtime_error("JPEG with more than one frame header");
                q += 6;
                need(q, 3 * size_t(nc));
                for (int i = 0; i < nc; ++i, q += 3) {
                    Component c;
                    c.id = d[q];
                    c.h = d[q + 1] >> 4;
                    c.v = d[q + 1] & 15;
                    c.tq = d[q + 2];
                    if (c.h < 1 || c.h > 2 || c.v < 1 || c.v > 2 || c.tq > 3)
                        throw std::runtime_error("unsupported JPEG sampling factors");
                    hmax = std::max(hmax, c.h);
                    vmax = std::max(vmax, c.v);
                    comps.push_back(c);
                }
                frame = true;
                break;
            }
            case 0xC2:
            case 0xC3:
            case 0xC5:
            case 0xC6:
            case 0xC7:
            case 0xC9:
            case 0xCA:
            case 0xCB:
            case 0xCD:
            case 0xCE:
            case 0xCF:
                throw std::runtime_error("progressive, lossless or arithmetic-coded JPEG is not supported");
            case 0xDD:  // DRI
                need(q, 2);
                restart = be16(d, q);
                break;
            case 0xDA: {  // SOS: one interleaved scan holding every component
                if (!frame) throw std::runtime_error("JPEG scan before frame header");
                need(q, 1);
                int ns = d[q++];
                need(q, 2 * size_t(ns) + 3);
                if (ns != static_cast<int>(comps.size())) throw std::runtime_error("non-interleaved JPEG scans are not supported");
                if (ns == 1) {  // a single-component scan codes one block per MCU (T.81 A.2.2)
                    comps[0].h = comps[0].v = 1;
                    hmax = vmax = 1;
                }
                for (int i = 0; i < ns; ++i, q += 2) {
                    auto it = std::find_if(comps.begin(), comps.end(), [&](const Component& c) { return c.id == d[q]; });
                    if (it == comps.end()) throw std::runtime_error("JPEG scan names an unknown component");
                    it->td = d[q + 1] >> 4;
                    it->ta = d[q + 1] & 15;
                    if (it->td > 3 || it->ta > 3) throw std::runtime_error("invalid JPEG Huffman table id");
                }
                const int mcux = (width + 8 * hmax - 1) / (8 * hmax), mcuy = (height + 8 * vmax - 1) / (8 * vmax);
                uint64_t blocks = 0;
                for (const auto& c : comps) blocks += uint64_t(mcux) * c.h * mcuy * c.v;
                // every coded block takes at least two bits (a DC code and an end-of-block
                // code): a header claiming more blocks than the file can hold is rejected
                // before its planes are allocated
                if (blocks > 4 * uint64_t(d.size() - end)) throw std::runtime_error("truncated JPEG scan");
                for (auto& c : comps) {
                    if (!qt_def[c.tq]) throw std::runtime_error("JPEG component uses an undefined quantisation table");
                    c.bw = mcux * c.h;
                    c.bh = mcuy * c.v;
                    c.plane.assign(size_t(c.bw) * 8 * c.bh * 8, 0);
                    c.dc_pred = 0;
                }
                BitReader br(d, end);
                int todo = restart;
                for (int my = 0; my < mcuy; ++my)
                    for (int mx = 0; mx < mcux; ++mx) {
                        if (restart && todo == 0) {
                            br.restart();
                            for (auto& c : comps) c.dc_pred = 0;
                            todo = restart;
                        }
                        for (auto& c : comps)
                            for (int by = 0; by < c.v; ++by)
                                for (int bx = 0; bx < c.h; ++bx) {
                                    float blk[64] = {};
                                    int t = decode_symbol(br, dc[c.td]);
                                    if (t > 11) throw std::runtime_error("invalid JPEG DC category");
                                    // a valid stream keeps the prediction within +-2^11;
                                    // the clamp only bounds what a corrupt one can build up
                                    c.dc_pred = std::clamp(c.dc_pred + extend(br.bits(t), t), -(1 << 20), 1 << 20);
                                    blk[0] = static_cast<float>(c.dc_pred) * static_cast<float>(qt[c.tq][0]);
                                    for (int k = 1; k < 64;) {
                                        int rs = decode_symbol(br, ac[c.ta]);
                                        int r = rs >> 4, s = rs & 15;
                                        if (s == 0) {
                                            if (r != 15) break;  // end of block
                                            k += 16;
                                            continue;
                                        }
                                        k += r;
                                        if (k > 63) throw std::runtime_error("JPEG coefficient index beyond the block");
                                        int zz = kZigzag[k];
                                        blk[zz] = static_cast<float>(extend(br.bits(s), s)) * static_cast<float>(qt[c.tq][zz]);
                                        ++k;
                                    }
                                    int ox = (mx * c.h + bx) * 8, oy = (my * c.v + by) * 8;
                                    idct8x8(blk, &c.plane[size_t(oy) * c.bw * 8 + ox], c.bw * 8);
                                }
                        if (restart) --todo;
                    }
                // skip to the next marker after the entropy-coded data
                size_t r = br.pos();
                while (r + 1 < d.size() && !(d[r] == 0xFF && d[r + 1] != 0x00 && !(d[r + 1] >= 0xD0 && d[r + 1] <= 0xD7)))
                    ++r;
                p = r;
                done = true;
                continue;
            }
            default:
                break;  // APPn, COM and others
        }
        p = end;
    }
    if (!done) throw std::runtime_error("JPEG without image data");
    Image8 img;
    img.width = width;
    img.height = height;
    img.gray = comps.size() == 1;
    img.rgb.resize(size_t(width) * height * 3);
    // Chroma at half resolution is brought up by a triangle filter per axis (3/4 of the
    // nearer sample, 1/4 of the next one away, edges replicated at the component's own
    // size): the "fancy" upsampling of the IJG decoder, which JPEG readers apply by default.
    auto sample = [&](const Component& c, int x, int y) -> float {
        const int fx = hmax / c.h, fy = vmax / c.v;
        const int cw = (width * c.h + hmax - 1) / hmax, ch = (height * c.v + vmax - 1) / vmax;
        const int stride = c.bw * 8;
        const int i = x / fx, j = y / fy;
        const int ni = fx == 2 ? std::clamp(x % 2 ? i + 1 : i - 1, 0, cw - 1) : i;
        const int nj = fy == 2 ? std::clamp(y % 2 ? j + 1 : j - 1, 0, ch - 1) : j;
        auto col = [&](int ii) -> float {
            float a = c.plane[size_t(j) * stride + ii];
            return fy == 2 ? 0.75f * a + 0.25f * c.plane[size_t(nj) * stride + ii] : a;
        };
        return fx == 2 ? 0.75f * col(i) + 0.25f * col(ni) : col(i);
    };
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x) {
            uint8_t* o = &img.rgb[(size_t(y) * width + x) * 3];
            if (img.gray) {
                o[0] = o[1] = o[2] = comps[0].plane[size_t(y) * comps[0].bw * 8 + x];
                continue;
            }
            float Y = sample(comps[0], x, y), cb = sample(comps[1], x, y) - 128.0f,
                  cr = sample(comps[2], x, y) - 128.0f;
            float rgb[3] = {Y + 1.402f * cr, Y - 0.344136f * cb - 0.714136f * cr, Y + 1.772f * cb};
            for (int k = 0; k < 3; ++k)
                o[k] = static_cast<uint8_t>(std::clamp(static_cast<int>(std::lround(rgb[k])), 0, 255));
        }
    return img;
}

Image8 read_image(const std::string& path) { return is_jpeg_file(path) ? read_jpeg(path) : read_png(path); }

}  // namespace sadcli
